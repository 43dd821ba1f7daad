#!/usr/bin/env python3
"""Throughput of the MUSCL-Hancock split step on one GB300 (or N replicas).

Metric: cell-updates/s, FP32 vs FP64 at the stated L1 error
vs FP64.  Workload: the cylindrical blast (domain [0,2]^2, r=0.4 at (1,1),
rho/p 1/1 inside, 0.125/0.1 outside, transmissive, CFL 0.8) on an 8192^2
grid, HLLC, minmod; synthetic initial state evaluated on the device.

  value  : FP32 HLLC cell-updates/s, state resident in HBM, K steps replayed
           from one CUDA graph (dt from the fused device reduction), timed
           with CUDA events on the library's stream.
  e2e    : the same metric through the drop-in C-ABI call on HOST grids
           (eu_step_host: H2D of the Grid2D AoS state, dt, step, D2H of the
           new state every step, pinned buffers).
  roofline: dominant sweep kernel, algorithmic bytes (read 4 + write 4
           fields per cell per sweep) / average launch time, against the
           measured HBM copy bandwidth.
  cpu_baseline: the CPU oracle (C restatement of the reference solver, FP64,
           OpenMP over all host cores) on a bounded sample of the workload.
  solvers: step times of HLL, HLLC, exact and FORCE on the same grid, FP32
           and FP64, and the exact solver's FP32-vs-FP64 error after 220 steps.
  flops  : secondary figure, the reference algorithm's arithmetic operations
           per cell-update (op-counting oracle, committed fixture) times
           the FP32 throughput.

Multi-GPU: the path is run as independent replicas (one grid per rank, no
collective on the data path); value is the sum over ranks, timing the max.
`--impl reference` times the reference algorithm's CPU implementation (the
oracle port; the reference sources are not available on the GPU host) on the
host cores and prints the same JSON line with "impl": "reference".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# The ensemble gradient leg runs 64 grids on their own streams; 32 hardware
# work queues instead of CUDA's default 8 let more of them run at once.  CUDA
# reads this when the context is created, so it is set before any device use.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "cell-updates/s FP32 vs FP64 at stated L1 err vs FP64; adjoint/forward time ratio"
UNIT = "cell-updates/s"
REF_MAX_STEPS = 60   # reference arm: at most this many timed (and warm-up) full steps


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--n", "--grid", dest="n", type=int, default=8192, help="grid is n x n")
    ap.add_argument("--solver", default="hllc", choices=("hll", "hllc", "exact", "force"))
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--skip-adjoint", action="store_true")
    ap.add_argument("--skip-ensemble", action="store_true")
    ap.add_argument("--skip-solvers", action="store_true", help="skip the HLL / exact / FORCE step times")
    ap.add_argument("--no-autotune", action="store_true", help="keep the planner's launch shape (profiling)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max-reduction over ranks (torch.distributed when WORLD_SIZE > 1)."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch
            import torch.distributed as td
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            td.init_process_group(backend=backend)
            self.td, self.torch = td, torch
            self.backend = backend

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.ws == 1:
            return x
        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = self.torch.tensor([x], dtype=self.torch.float64, device=dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


def bind_to_gpu_cpus(local: int):
    """Pin this process to the CPUs nvidia-smi reports as local to the GPU,
    so that pinned host buffers allocated afterwards come from that node's
    memory (the e2e copies cross the CPU-GPU link, not a socket link).
    Returns the CPU list used, or None."""
    try:
        out = subprocess.run(["nvidia-smi", "topo", "-m"], capture_output=True, text=True, timeout=20).stdout
    except Exception:
        return None
    lines = [l for l in out.splitlines() if l.strip()]
    if not lines:
        return None
    head = lines[0].split("\t")
    col = next((k for k, h in enumerate(head) if "CPU Affinity" in h), None)
    row = next((l.split("\t") for l in lines if l.startswith(f"GPU{local}\t") or l.startswith(f"GPU{local} ")), None)
    if col is None or row is None or col >= len(row):
        return None
    cpus = set()
    for part in row[col].replace(" ", "").split(","):
        if "-" in part:
            a, b = part.split("-")
            if a.isdigit() and b.isdigit():
                cpus.update(range(int(a), int(b) + 1))
        elif part.isdigit():
            cpus.add(int(part))
    cpus &= set(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else cpus
    if not cpus:
        return None
    try:
        os.sched_setaffinity(0, cpus)
    except OSError:
        return None
    return row[col].strip()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def reference_flops(solver: str):
    """Arithmetic operations (add, mul, div, sqrt, pow) per cell-update of the
    reference algorithm for `solver`, counted by the op-counting build of the
    restatement on the 256^2 blast (tests/golden/opcounts.json, generated by
    tests/golden/make_opcounts.py); None when the file is absent."""
    p = os.path.join(ROOT, "tests", "golden", "opcounts.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    return float(d["workloads"]["blast_256"][solver]["arith_per_cell_update"])


def profiled_traffic(key: str):
    """Per-launch DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum)
    recorded from ncu in profiles/*.md as `traffic[<key>] = <bytes>`."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for fn in sorted(os.listdir(d)):
        if not fn.endswith((".md", ".txt")):
            continue
        for line in open(os.path.join(d, fn)):
            line = line.strip().strip("`")
            if line.startswith(f"traffic[{key}]"):
                try:
                    return float(line.split("=")[1].split()[0])
                except (IndexError, ValueError):
                    pass
    return None


def cpu_port_rate(n: int, solver: str, seconds: float, max_steps: int | None = None, warmup: int = 1):
    """Oracle port (C restatement of the reference CPU solver, OpenMP on every
    host core, OMP_PROC_BIND=close OMP_PLACES=cores) on the n x n blast: the
    reference's time loop (scripts/cpu/main_cpu.cpp:221-241) with its grids
    and workspace allocated once -- per step the ghost fill, compute_dt and
    advance_second_order -- `warmup` untimed steps, then until `seconds` of
    work or max_steps."""
    import numpy as np
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_PLACES", "cores")
    from oracle import oracle as O
    O.build(reference=False)
    P = O.Oracle("port")
    threads = os.cpu_count() or 1
    P.set_threads(threads)
    g = O.Grid(n, n, 0.0, 2.0, 0.0, 2.0)
    U = P.init_blast(g)
    Utmp, Unew = g.zeros(), g.zeros()
    fx, fy = np.zeros(4 * (n + 1) * n), np.zeros(4 * n * (n + 1))

    def step(U, Unew):
        P.apply_boundary(U, g)
        dt = P.compute_dt(U, g, 0.8)
        P.advance_second_order(U, g, dt, solver, Utmp, Unew, fx, fy)

    for _ in range(max(1, warmup)):                      # warm-up (touches every buffer)
        step(U, Unew)
        U, Unew = Unew, U
    steps, t0 = 0, time.perf_counter()
    while True:
        step(U, Unew)
        U, Unew = Unew, U
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds or (max_steps and steps >= max_steps):
            break
    rate = n * n * steps / el
    return rate, threads, steps, el


def run_reference(args, dist: Dist):
    if dist.rank != 0:
        return
    # the same K timed steps after W warm-up steps as the GPU arm, bounded so
    # that the run stays within a few minutes (~0.9 s per full 8192^2 FP64
    # step on 16 Grace cores)
    steps_cap = max(1, min(args.steps, REF_MAX_STEPS))
    warm = max(1, min(args.warmup, REF_MAX_STEPS))
    rate, threads, steps, el = cpu_port_rate(args.n, args.solver, seconds=1e9, max_steps=steps_cap, warmup=warm)
    sample = (f"{steps} full {args.n}x{args.n} FP64 {args.solver.upper()} steps (BC + compute_dt + "
              f"advance_second_order, grids and face caches allocated once) after {warm} warm-up steps, "
              f"{el:.1f} s on {threads} threads (OMP_PROC_BIND=close OMP_PLACES=cores)")
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * el / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"blast_{args.n}x{args.n}_{args.solver}", "nx": args.n, "ny": args.n,
                   "solver": args.solver, "precision": "fp64 (the reference has no FP32 path)"},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def adjoint_leg(E, np):
    """Adjoint workload: the 512^2 blast of [0,2]^2, HLLC + minmod, 400 steps
    with the FP64 CFL dt sequence frozen, checkpoints every 32 steps,
    J = sum rho^2 over 0.6 <= r <= 0.8.  Times (CUDA events) the checkpointed
    forward, the backward (recomputation + adjoint sweeps) and the plain
    graph-replayed forward of the same 400 steps."""
    from large_sys_eq_opt_gb300.cases import blast_adjoint_512
    n, nsteps, k = 512, 400, 32
    prob = blast_adjoint_512()
    s64 = E.Solver.for_problem(prob, "fp64", "hllc")
    s64.set_dt_log(nsteps)
    s64.step_n(nsteps)
    dts = s64.dt_log(nsteps)
    s64.close()
    x = (np.arange(n) + 0.5) * (2.0 / n)
    X, Y = np.meshgrid(x, x)
    r = np.sqrt((X - 1.0) ** 2 + (Y - 1.0) ** 2)
    mask = (r >= 0.6) & (r <= 0.8)
    res = {"workload": f"blast_{n}x{n}_hllc_{nsteps}steps_ckpt{k}", "objective": "sum rho^2 over 0.6<=r<=0.8",
           "dt": "FP64 CFL 0.8 sequence frozen"}
    grads = {}
    for prec in ("fp32", "fp64"):
        s = E.Solver.for_problem(prob, prec, "hllc")
        shape = s.autotune(20)
        U0 = s.download()
        fwd, bwd = [], []
        for rep in range(3 if prec == "fp32" else 1):
            s.upload(U0)
            s.adjoint_forward(dts, k)
            gN = np.zeros_like(U0)
            UN = s.download()
            gN[2:-2, 2:-2, 0] = np.where(mask, 2.0 * UN[2:-2, 2:-2, 0], 0.0)
            grads[prec] = s.adjoint_backward(gN)
            f_ms, b_ms = s.adjoint_timing()
            fwd.append(f_ms)
            bwd.append(b_ms)
        s.upload(U0)
        s.step_n(8)   # warm the graph
        s.upload(U0)
        plain = s.time_steps(nsteps)[0]
        s.close()
        f_ms, b_ms = float(np.median(fwd)), float(np.median(bwd))
        res[prec] = {"seg_xy": list(shape), "forward_ckpt_ms": f_ms, "backward_ms": b_ms, "forward_graph_ms": plain,
                     "backward_over_forward": b_ms / plain, "gradient_over_forward": (f_ms + b_ms) / plain}
    a = np.concatenate([grads["fp64"][..., 0].ravel(), grads["fp64"][..., 3].ravel()])
    b = np.concatenate([grads["fp32"][..., 0].ravel(), grads["fp32"][..., 3].ravel()])
    res["fp32_vs_fp64_gradient_rel_l2"] = float(np.linalg.norm(a - b) / np.linalg.norm(a))
    return res


FIELDS = ("rho", "rhou", "rhov", "E", "p")


def field_errors(np, got, ref):
    """Per-field L1 (mean absolute) and Linf differences over the interior."""
    def fields(A):
        r, mu, mv, en = (A[2:-2, 2:-2, k] for k in range(4))
        return (r, mu, mv, en, 0.3999999999999999 * (en - 0.5 * (mu * mu + mv * mv) / r))
    out = {}
    for name, a, b in zip(FIELDS, fields(got), fields(ref)):
        d = np.abs(a - b)
        out[name] = {"l1": float(d.mean()), "linf": float(d.max())}
    return out


def fp32_error_leg(E, np):
    """FP32 form against FP64 per field and per configuration, both on the
    FP64 run's dt sequence: the 256^2 blast to t_end (HLLC), the 1000x396
    reflective shock-bubble to t_end with each of the four Riemann solvers,
    the 512^2 adjoint case (400 steps, HLLC)."""
    from large_sys_eq_opt_gb300.cases import blast_256, blast_adjoint_512, shock_bubble_1000x396
    res = {}
    cases = [("blast256_t_end_hllc", blast_256(), None, "hllc")]
    cases += [(f"shock_bubble_1000x396_t_end_{sv}", shock_bubble_1000x396(), None, sv)
              for sv in ("hll", "hllc", "exact", "force")]
    cases += [("blast512_400steps_hllc", blast_adjoint_512(), 400, "hllc")]
    for name, prob, nsteps, solver in cases:
        s64 = E.Solver.for_problem(prob, "fp64", solver)
        s64.set_dt_log(1 << 16)
        if nsteps is None:
            info = s64.run(prob.cfg.t_end)
            nsteps = info["steps"]
        else:
            s64.step_n(nsteps)
        dts = s64.dt_log(nsteps)
        ref = s64.download()
        s64.close()
        s32 = E.Solver.for_problem(prob, "fp32", solver)
        s32.step_n(nsteps, dts)
        got = s32.download()
        s32.close()
        res[name] = {"steps": int(nsteps), **field_errors(np, got, ref)}
    return res


def developed_leg(E, np, prob, dist, t_dev=0.2):
    """Step times on a developed flow: the 8192^2 FP32 blast is first run
    with HLLC to t = t_dev (the ring has expanded to r ~ 0.8 and the interior
    carries the rarefaction and contact, so few faces see identical states),
    then HLLC and the exact solver are timed from that state (graph-replayed
    steps, CUDA events).  Complements the early-window figures, where nearly
    every face of the grid sees identical left and right states."""
    cells = prob.cfg.nx * prob.cfg.ny
    res = {"t_developed": t_dev}
    s = E.Solver.for_problem(prob, "fp32", "hllc")
    t0 = time.perf_counter()
    info = s.run(t_dev)
    res["steps_to_develop"] = int(info["steps"])
    res["develop_wall_s"] = time.perf_counter() - t0
    U = s.download()
    for solver, w, k in (("hllc", 3, 50), ("exact", 3, 20)):
        s.upload(U)
        s.set_option("solver", {"hll": 0, "hllc": 1, "exact": 2, "force": 3}[solver])
        s.time_steps(w)
        s.upload(U)
        tot, tx, ty = s.time_steps(k)
        res[solver] = {"ms_per_step": tot / k, "value": cells * k * dist.ws / (dist.max(tot) / 1e3),
                       "per_kernel_ms": {"sweep_x": tx / k, "sweep_y": ty / k}, "steps": k}
    s.close()
    return res


def e2e_leg(E, prob, precision, solver, dist, ke=10, warm=3):
    """The metric through the drop-in call on host grids: eu_step_host
    (Grid2D AoS in, BC + compute_dt + advance_second_order, Grid2D AoS out),
    pinned host buffers, `warm` warm-up steps then `ke` timed steps (the
    first calls of a process page in the pinned buffers and staging)."""
    n = prob.cfg.nx
    cells = prob.cfg.nx * prob.cfg.ny
    se = E.Solver.for_problem(prob, precision, solver)
    A = E.PinnedGrid(prob.cfg.nx, prob.cfg.ny)
    B = E.PinnedGrid(prob.cfg.nx, prob.cfg.ny)
    se.download(A.array)
    t, t_end = 0.0, 1e30
    for k in range(warm):                                  # warm-up
        src, dst = (A, B) if k % 2 == 0 else (B, A)
        t += se.step_host(src.array, dst.array, 0.8, t, t_end)
    if warm % 2 == 0:
        A, B = B, A                                        # B holds the latest state
    dist.barrier()
    t0 = time.perf_counter()
    step_s = []
    for k in range(ke):
        src, dst = (B, A) if k % 2 == 0 else (A, B)
        ts = time.perf_counter()
        t += se.step_host(src.array, dst.array, 0.8, t, t_end)
        step_s.append(time.perf_counter() - ts)
    el = dist.max(time.perf_counter() - t0)
    se.close()
    del A, B
    aos = (n + 4) * (prob.cfg.ny + 4) * 32
    return {"value": cells * ke * dist.ws / el, "unit": UNIT, "h2d_bytes_per_step": aos,
            "d2h_bytes_per_step": aos, "steps": ke, "precision": precision,
            "call": "eu_step_host (Grid2D AoS in, BC + compute_dt + advance_second_order, AoS out)",
            "best_step_ms": 1e3 * min(step_s), "median_step_ms": 1e3 * statistics.median(step_s),
            "step_ms": [round(1e3 * x, 2) for x in step_s]}


def ensemble_leg(E, np, steps=20):
    """Uneven ensemble workload (48 blasts on {128..1024}^2, 16 shock-bubbles
    500x198..2000x792, FP32 HLLC, per-instance CFL dt): one persistent launch
    per step after the ensemble autotuner, against the same instances stepped
    one after another on their own handles (each with its own tuned shape
    and graph)."""
    from large_sys_eq_opt_gb300.cases import ensemble_problems
    probs = ensemble_problems()
    with E.Batch(probs, "fp32", "hllc") as b:
        b.start()
        shape = b.autotune(3)
        b.time_steps(3)
        ms = b.time_steps(steps)
        cells = b.cells
    # batched gradients of every instance w.r.t. its two scalar parameters,
    # device-resident (eu_batch_param_gradients); the first call also
    # allocates the adjoint workspace, the second is the timed one.  ckpt_k 0
    # keeps every step's state in HBM when it fits (no recomputation); the
    # same call with checkpoints every 32 steps is timed beside it.
    from large_sys_eq_opt_gb300 import adjoint as A
    nadj = 100
    with E.Batch(probs, "fp32", "hllc") as b:
        b.autotune(2)
        t0 = time.perf_counter()
        A.ensemble_parameter_gradients(E, probs, nadj, "fp32", "hllc", 32, batch=b)
        A.ensemble_parameter_gradients(E, probs, nadj, "fp32", "hllc", 32, batch=b)
        t_k32 = time.perf_counter()
        A.ensemble_parameter_gradients(E, probs, nadj, "fp32", "hllc", 32, batch=b)
        t_k32 = time.perf_counter() - t_k32
        t0 = time.perf_counter()
        A.ensemble_parameter_gradients(E, probs, nadj, "fp32", "hllc", 0, batch=b)
        t_first = time.perf_counter() - t0
        t0 = time.perf_counter()
        parts = {}
        Js, grads, dts, _ = A.ensemble_parameter_gradients(E, probs, nadj, "fp32", "hllc", 0, batch=b,
                                                           timing=parts)
        t_all = time.perf_counter() - t0
        ckpt_k = max(inst.get_option("ckpt_k") for inst in b.instances)
        fwd_ms = max(inst.adjoint_timing()[0] for inst in b.instances)
        bwd_ms = max(inst.adjoint_timing()[1] for inst in b.instances)
        for inst, p in zip(b.instances, probs):
            inst.init_params(p)
        b.start()
        b.step(2)
        for inst, p in zip(b.instances, probs):
            inst.init_params(p)
        b.start()
        plain_ms = b.time_steps(nadj)
    adj = {"steps": nadj, "params": "blast R (ramped interface) and p_in; bubble rho and Mach",
           "path": "device-resident: eu_batch_param_gradients (initial states, checkpointed CFL forwards "
                   "logging their dts, objective and dJ/dU_N, backward sweeps with those dts, tangent "
                   "contractions on the device; 3 numbers per instance to the host)",
           "ckpt_k": ckpt_k, "ckpt_rule": "0 = every step's state resident when it fits in half the free HBM",
           "plain_ensemble_forward_ms": plain_ms, "gradients_wall_s_total": t_all,
           "gradients_wall_s_first_call": t_first, "gradients_over_plain_forward": t_all * 1e3 / plain_ms,
           "gradients_wall_s_ckpt_k32": t_k32, "gradients_over_plain_forward_ckpt_k32": t_k32 * 1e3 / plain_ms,
           "wall_s_param_gradients_call": parts.get("gradients_s"),
           "checkpointed_forward_ms_max_instance": fwd_ms, "backward_device_ms_max_instance": bwd_ms,
           "example_gradients": grads[:2] + grads[48:50]}
    seq_ms = 0.0
    for p in probs:
        with E.Solver.for_problem(p, "fp32", "hllc") as s:
            s.autotune(3)
            s.time_steps(3)
            seq_ms += s.time_steps(steps)[0]
    return {"workload": f"ensemble_{len(probs)}_fp32_hllc", "instances": len(probs), "cells": cells,
            "steps": steps, "seg_xy": list(shape), "ms_per_step": ms / steps,
            "value": cells * steps / (ms / 1e3), "unit": UNIT,
            "sequential_ms_per_step": seq_ms / steps, "speedup_vs_sequential": seq_ms / ms,
            "batched_adjoint": adj}


def pressure(A):
    r, mu, mv, en = (A[2:-2, 2:-2, k] for k in range(4))
    return 0.3999999999999999 * (en - 0.5 * (mu * mu + mv * mv) / r)


def fp64_and_error(E, np, prob, solver, W, K, dist):
    """FP64 throughput over K graph-replayed steps after W, and the FP32 form
    against FP64 after W + K steps on the FP64 dt sequence."""
    cells = prob.cfg.nx * prob.cfg.ny
    s64 = E.Solver.for_problem(prob, "fp64", solver)
    s64.set_dt_log(W + K)
    s64.time_steps(W)
    tot64, tx64, ty64 = s64.time_steps(K)
    v64 = cells * K * dist.ws / (dist.max(tot64) / 1e3)
    dts = s64.dt_log(W + K)
    ref = s64.download()
    s64.close()
    e32 = E.Solver.for_problem(prob, "fp32", solver)
    e32.step_n(W + K, dts)
    got = e32.download()
    e32.close()
    drho = np.abs(got[2:-2, 2:-2, 0] - ref[2:-2, 2:-2, 0])
    dp = np.abs(pressure(got) - pressure(ref))
    fp64 = {"value": v64, "ms_per_step": tot64 / K, "per_kernel_ms": {"sweep_x": tx64 / K, "sweep_y": ty64 / K}}
    err = {"steps": W + K, "dt": "FP64 dt sequence replayed",
           "l1_rho": float(drho.mean()), "linf_rho": float(drho.max()),
           "l1_p": float(dp.mean()), "linf_p": float(dp.max()), "per_field": field_errors(np, got, ref)}
    return fp64, err


def solvers_leg(E, np, prob, dist):
    """Step time of every Riemann solver on the benchmark grid, FP32 and FP64
    (graph-replayed steps, CUDA events), and for the exact solver the FP32
    form against FP64 after 20 + 200 steps on the FP64 dt sequence."""
    cells = prob.cfg.nx * prob.cfg.ny
    res = {}
    for solver in ("hll", "hllc", "exact", "force"):
        r = {}
        for prec, w, k in (("fp32", 3, 10), ("fp64", 1, 3)):
            s = E.Solver.for_problem(prob, prec, solver)
            s.time_steps(w)
            tot, tx, ty = s.time_steps(k)
            s.close()
            r[prec] = {"ms_per_step": tot / k, "value": cells * k * dist.ws / (dist.max(tot) / 1e3)}
        res[solver] = r
    _, err = fp64_and_error(E, np, prob, "exact", 20, 200, dist)
    res["exact"]["fp32_vs_fp64"] = err
    return res


def run_ours(args, dist: Dist):
    import numpy as np

    import large_sys_eq_opt_gb300.euler2d as E
    from large_sys_eq_opt_gb300.cases import blast_large

    E.set_device(dist.local)
    n, K, W = args.n, args.steps, args.warmup
    prob = blast_large(n)
    cells = n * n
    peak, peak_kind = measured_peaks()
    out = {}

    # ---- FP32 device-resident throughput (the headline) -------------------
    s32 = E.Solver.for_problem(prob, "fp32", args.solver)
    shape32 = ((s32.get_option("seg_x"), s32.get_option("seg_y")) if args.no_autotune else s32.autotune(10))
    s32.time_steps(W)
    dist.barrier()
    with ClockSampler(dist.local) as clk:
        tot, tx, ty = s32.time_steps(K)
    dist.barrier()
    tmax = dist.max(tot)
    value = cells * K * dist.ws / (tmax / 1e3)
    esz = 4
    bytes_per_launch = cells * 8 * esz
    dom, tdom = ("sweep_x", tx) if tx >= ty else ("sweep_y", ty)
    achieved = bytes_per_launch / (tdom / K / 1e3) / 1e9
    traffic = profiled_traffic(f"fp32_{args.solver}_{dom}_{n}")
    out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                       "frac": achieved / peak, "traffic": traffic, "kernel": dom,
                       "peak_source": f"{peak_kind} hbm_gbs",
                       "per_kernel_ms": {"sweep_x": tx / K, "sweep_y": ty / K},
                       "algorithmic_bytes_per_launch": bytes_per_launch,
                       # the whole step: 64 B (FP32) per cell-update over the step time
                       "step": {"achieved": 2 * bytes_per_launch / (tmax / K / 1e3) / 1e9,
                                "frac": 2 * bytes_per_launch / (tmax / K / 1e3) / 1e9 / peak,
                                "algorithmic_bytes_per_step": 2 * bytes_per_launch}}
    out["clocks"] = clk.summary()
    fl = reference_flops(args.solver)
    if fl is not None:
        # secondary figure: the reference algorithm's arithmetic rate at this
        # throughput (it repeats work the sweeps do once, so this is an
        # equivalent rate, not the FP32 pipe's)
        out["flops"] = {"reference_arith_per_cell_update": fl,
                        "reference_equivalent_tflops": value * fl / 1e12,
                        "source": "tests/golden/opcounts.json (op-counting oracle, blast 256^2)"}
    s32.close()

    # ---- e2e through the drop-in call on host grids -----------------------
    # (right after the headline leg, before the legs that allocate and free
    # several GB of host arrays, which made single steps stall)
    if not args.skip_e2e:
        import gc
        gc.collect()
        cpus = bind_to_gpu_cpus(dist.local)
        out["e2e"] = e2e_leg(E, prob, "fp32", args.solver, dist)
        out["e2e"]["host_cpus"] = cpus
        gc.collect()
        # the like-for-like drop-in figure: FP64 arithmetic, as the reference
        out["e2e_fp64"] = e2e_leg(E, prob, "fp64", args.solver, dist)

    # ---- FP64 throughput + FP32-vs-FP64 error at the final step -----------
    if not args.skip_fp64:
        out["fp64"], out["fp32_vs_fp64"] = fp64_and_error(E, np, prob, args.solver, W, K, dist)
        out["fp32_vs_fp64"]["speedup"] = value / out["fp64"]["value"]

    # ---- the other Riemann solvers on the same grid ------------------------
    if not args.skip_solvers:
        out["solvers"] = solvers_leg(E, np, prob, dist)

    # ---- developed-flow step times (FP32 HLLC and exact) -------------------
    if not args.skip_solvers:
        out["developed"] = developed_leg(E, np, prob, dist)

    # ---- discrete adjoint: time ratio against the forward -----------------
    if not args.skip_adjoint:
        out["adjoint"] = adjoint_leg(E, np)

    # ---- FP32 error per field and configuration ----------------------------
    if not args.skip_fp64:
        out["fp32_error_by_config"] = fp32_error_leg(E, np)

    # ---- uneven ensemble in one persistent launch per step ---------------
    if not args.skip_ensemble:
        out["ensemble"] = ensemble_leg(E, np)

    # ---- CPU baseline (oracle port on the host cores) ---------------------
    if dist.rank == 0 and dist.ws == 1 and not args.skip_cpu:
        rate, threads, steps, el = cpu_port_rate(n, args.solver, args.cpu_seconds)
        out["cpu_baseline"] = {
            "value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} full {n}x{n} FP64 {args.solver.upper()} steps of the oracle port (BC + compute_dt + "
                      f"advance_second_order, grids and face caches allocated once; OpenMP, {threads} threads, "
                      f"OMP_PROC_BIND=close OMP_PLACES=cores) after 1 warm-up step, {el:.1f} s"}

    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.ws, "steps": K, "warmup": W,
            "ms_per_step": tmax / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"blast_{n}x{n}_{args.solver}_fp32", "nx": n, "ny": n, "solver": args.solver,
                       "limiter": "minmod", "cfl": 0.8, "precision": "fp32 (FP64 pressure recovery under "
                       "cancellation; exact solver: FP32 Newton for p* finished by an FP64 Newton step)",
                       "graph": f"{K} steps in one CUDA graph",
                       "l2": f"inputs larger than L2 ({16 * n * n / 1e9:.2f} GB of interior cells per FP32 "
                             "state buffer vs 126 MB L2)",
                       "parallelism": f"replicas x{dist.ws}",
                       "seg_xy": list(shape32) + ["planner" if args.no_autotune else "autotuned"]},
            "gpu_launches": 2 * K,
            "adjoint_forward_ratio": (out["adjoint"]["fp32"]["backward_over_forward"]
                                      if "adjoint" in out else None),
        }
        line.update(out)
        # the headline figures once more at the end of the line (the part a
        # truncated log keeps): FP32 and FP64, device-resident and e2e, and
        # the CPU baseline they compare with
        summ = {"fp32_value": value, "fp32_e2e": out.get("e2e", {}).get("value"),
                "fp64_value": out.get("fp64", {}).get("value"), "fp64_e2e": out.get("e2e_fp64", {}).get("value"),
                "cpu_baseline_fp64": out.get("cpu_baseline", {}).get("value"),
                "roofline_frac": out["roofline"]["frac"], "roofline_kernel": out["roofline"]["kernel"],
                "roofline_frac_step": out["roofline"]["step"]["frac"]}
        cb = summ["cpu_baseline_fp64"]
        for k in ("fp32_value", "fp32_e2e", "fp64_value", "fp64_e2e"):
            if cb and summ[k]:
                summ[k + "_over_cpu"] = summ[k] / cb
        if summ["fp64_value"]:
            summ["fp32_over_fp64"] = value / summ["fp64_value"]
        if "adjoint" in out:
            summ["adjoint_backward_over_forward"] = {p: out["adjoint"][p]["backward_over_forward"]
                                                     for p in ("fp32", "fp64")}
        if "fp32_error_by_config" in out:
            summ["fp32_l1_rho_by_config"] = {k: v["rho"]["l1"] for k, v in out["fp32_error_by_config"].items()}
        line["summary"] = summ
        print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
