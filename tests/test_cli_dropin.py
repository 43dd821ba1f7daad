"""The two drop-in surfaces above the C ABI:

* the C++ command-line driver (large_sys_eq_opt_gb300/bin/euler2d_gb300),
  which takes the reference driver's arguments (scripts/cpu/main_cpu.cpp:67-113)
  and writes its CSV snapshots (scripts/cpu/main_cpu.cpp:136-164);
* the C++ shim (large_sys_eq_opt_gb300/shim/solver_cpu_gb300.cpp) that
  replaces src/cpu/solver_cpu.cpp under the reference's unmodified driver.
"""
import os
import subprocess

import numpy as np
import pytest

from oracle.oracle import REFERENCE_TREE, Grid

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "large_sys_eq_opt_gb300")


@pytest.fixture(scope="module")
def cli():
    from large_sys_eq_opt_gb300 import build as B
    B.build()
    return B.CLI


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_cli_rejects_bad_arguments(cli):
    r = subprocess.run([cli, "--solver", "roe"], capture_output=True, text=True)
    assert r.returncode == 1
    assert "Unknown Riemann solver: roe" in r.stderr
    r = subprocess.run([cli, "0"], capture_output=True, text=True)
    assert r.returncode == 1 and "resolution_scale must be positive" in r.stderr
    r = subprocess.run([cli, "--case", "nope"], capture_output=True, text=True)
    assert r.returncode == 1 and "Unknown case name" in r.stderr
    r = subprocess.run([cli, "--bogus"], capture_output=True, text=True)
    assert r.returncode == 1 and "Unknown argument: --bogus" in r.stderr


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU failure path")
def test_cli_fails_loudly_without_gpu(cli):
    r = subprocess.run([cli, "--timing-only"], capture_output=True, text=True)
    assert r.returncode == 1
    assert "no CUDA device" in r.stderr


@pytest.mark.skipif(not os.path.isdir(REFERENCE_TREE), reason="reference sources not present")
def test_shim_links_with_unmodified_reference_driver(cli):
    """main_cpu.cpp + test_cases.cpp + init.cpp from the reference, linked
    against the shim in place of solver_cpu.cpp: every solver symbol resolves
    with the reference's own signatures."""
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    exe = os.path.join(ROOT, "oracle", "_ref", "main_cpu_gb300")
    assert os.access(exe, os.X_OK)
    if not has_gpu():
        r = subprocess.run([exe, "--timing-only"], capture_output=True, text=True)
        assert r.returncode != 0
        assert "no CUDA device" in r.stderr


def read_snapshot(path):
    a = np.loadtxt(path, delimiter=",", skiprows=1)
    with open(path) as f:
        assert f.readline().strip() == "i,j,x,y,rho,rhou,rhov,E"
    return a


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ("hll", "hllc"))
def test_cli_snapshots_match_oracle(cli, port, tmp_path, solver):
    """The reference's own shock-bubble case at scale 1 (500x197, CFL 0.4) to
    t_end with 5 snapshots: snapshot times, steps and every CSV value agree
    with the oracle run to the 6 significant digits the CSV carries."""
    r = subprocess.run([cli, "1", "--case", "shock_bubble", "--solver", solver, "--output", "--outdir",
                        str(tmp_path), "--prefix", "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    import large_sys_eq_opt_gb300.euler2d as E
    cfg = E.case_config("shock_bubble", 1)
    g = Grid(cfg.nx, cfg.ny, cfg.x_min, cfg.x_max, cfg.y_min, cfg.y_max)
    U = port.init_reference_case(g, 0)
    ref = port.run(U, g, cfg.cfl, cfg.t_end, solver, nsnap=5, want_snapshots=True)
    assert f"Total steps = {ref['steps']}" in r.stdout
    for k in range(1, 6):
        path = tmp_path / f"gpu_shock_bubble_{solver}_n1_snapshot_{k}.csv"
        a = read_snapshot(path)
        assert a.shape == (cfg.nx * cfg.ny, 8)
        i = a[:, 0].astype(int)
        j = a[:, 1].astype(int)
        assert i.min() == 2 and i.max() == cfg.nx + 1 and j.min() == 2 and j.max() == cfg.ny + 1
        Sref = ref["snapshots"][k - 1][j, i]
        for q in range(4):
            np.testing.assert_allclose(a[:, 4 + q], Sref[:, q], rtol=1e-5, atol=1e-9)


@pytest.mark.gpu
def test_shim_runs_the_reference_loop_on_the_gpu(cli, tmp_path, port):
    """The shim under the reference's calling pattern, on the GPU: the loop of
    scripts/cpu/main_cpu.cpp:217-262 (tests/dropin/run_shim.cpp, compiled
    here against a stand-in of the reference's headers, since the reference
    tree is not on the GPU host) runs the 256^2 blast to t_end with HLLC,
    then with the exact solver in the same process (one device handle per
    geometry, its solver switched per call).  Step counts equal the oracle's
    and L1(rho) <= 1e-10 at t_end; an uninitialised workspace throws."""
    exe = tmp_path / "run_shim"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "tests", "dropin"),
                        "-I" + os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "dropin", "run_shim.cpp"),
                        os.path.join(PKG, "shim", "solver_cpu_gb300.cpp"), "-L" + PKG, "-leuler2d",
                        "-Wl,-rpath," + PKG, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    g = Grid(256, 256, 0.0, 2.0, 0.0, 2.0)
    U0 = port.init_blast(g)
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        f.write(np.array([g.nx, g.ny], dtype=np.int32).tobytes())
        f.write(np.array([g.x_min, g.x_max, g.y_min, g.y_max, 0.8, 0.25]).tobytes())
        f.write(U0.tobytes())
    solvers = ("hllc", "exact")
    r = subprocess.run([str(exe), str(fin), str(fout), *solvers], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = open(fout, "rb").read()
    rec = 16 + U0.nbytes
    for k, solver in enumerate(solvers):
        steps = int(np.frombuffer(raw[k * rec:k * rec + 8], dtype=np.int64)[0])
        t = float(np.frombuffer(raw[k * rec + 8:k * rec + 16], dtype=np.float64)[0])
        got = np.frombuffer(raw[k * rec + 16:(k + 1) * rec], dtype=np.float64).reshape(U0.shape)
        V = U0.copy()
        ref = port.run(V, g, 0.8, 0.25, solver)
        assert steps == ref["steps"], (solver, steps, ref["steps"])
        assert abs(t - ref["t"]) <= 1e-14
        l1 = float(np.mean(np.abs(got[2:-2, 2:-2, 0] - V[2:-2, 2:-2, 0])))
        assert l1 <= 1e-10, (solver, l1)
