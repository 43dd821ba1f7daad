"""Build the in-tree CUDA library (libeuler2d.so) for sm_103a.

The translation units compile in parallel with nvcc (one -gencode, no
cmake): the sweep kernels and the adjoint sweep kernels once per (precision,
Riemann solver), the auxiliary kernels, the allocation-free audit and the
host runtime.  The FP32 units use fast approximate
reciprocal/square root (--use_fast_math); the FP64 units use IEEE division
and square root.  Objects go to large_sys_eq_opt_gb300/_build/, the library
to large_sys_eq_opt_gb300/libeuler2d.so.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libeuler2d.so")
CLI = os.path.join(PKG, "bin", "euler2d_gb300")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + CSRC, "-I" + INCLUDE]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libeuler2d.so")


def units():
    out = []
    for prec in (32, 64):
        for solver in range(4):
            flags = [f"-DEU_PREC={prec}", f"-DEU_SOLVER={solver}"]
            if prec == 32:
                flags.append("--use_fast_math")
            out.append((os.path.join(CSRC, "kern_sweeps.cu"), f"kern_{prec}_{solver}.o", flags))
    for prec in (32, 64):
        for solver in range(4):
            flags = [f"-DEU_PREC={prec}", f"-DEU_SOLVER={solver}"]
            if prec == 32:
                flags.append("--use_fast_math")
            out.append((os.path.join(CSRC, "adjoint_kernels.cu"), f"adj_{prec}_{solver}.o", flags))
    out.append((os.path.join(CSRC, "aux_kernels.cu"), "aux_kernels.o", []))
    out.append((os.path.join(CSRC, "noalloc.cu"), "noalloc.o", []))
    out.append((os.path.join(CSRC, "grad_kernels.cu"), "grad_kernels.o", []))
    for unit in ("runtime", "api", "api_adjoint", "api_batch", "api_domain"):
        out.append((os.path.join(CSRC, unit + ".cpp"), unit + ".o", ["-x", "cu"]))
    return out


def _sources_digest() -> str:
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE, os.path.join(PKG, "cli")):
        for fn in sorted(os.listdir(d)):
            p = os.path.join(d, fn)
            if os.path.isfile(p):
                h.update(fn.encode())
                with open(p, "rb") as f:
                    h.update(f.read())
    h.update(" ".join(ARCH + COMMON).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile (if sources changed) and return the library path."""
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "stamp")
    digest = _sources_digest()
    if (not force and os.path.exists(LIB) and os.path.exists(CLI) and os.path.exists(stamp)
            and open(stamp).read() == digest):
        return LIB
    cc = nvcc()
    jobs = []
    for src, obj, flags in units():
        cmd = [cc] + ARCH + COMMON + flags + (["-Xptxas", "-v"] if ptxas_info else []) + \
            ["-c", src, "-o", os.path.join(BUILD, obj)]
        jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(run, jobs))
    for cmd, r in results:
        if verbose or ptxas_info:
            sys.stderr.write(r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    objs = [os.path.join(BUILD, obj) for _, obj, _ in units()]
    tmp = LIB + ".tmp"
    link = [cc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + " ".join(link) + "\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    # the C++ command-line driver (links the library through an $ORIGIN rpath)
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    cxx = shutil.which("g++") or "g++"
    cli = [cxx, "-O2", "-std=c++17", "-I" + INCLUDE, os.path.join(PKG, "cli", "euler2d_gb300.cpp"),
           "-o", CLI + ".tmp", "-L" + PKG, "-leuler2d", "-Wl,-rpath,$ORIGIN/..", "-lpthread"]
    r = subprocess.run(cli, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("driver build failed:\n" + " ".join(cli) + "\n" + r.stdout + r.stderr)
    os.replace(CLI + ".tmp", CLI)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
