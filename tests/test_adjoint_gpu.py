"""Discrete adjoint on the GPU (eu_adjoint_forward / eu_adjoint_backward).

Objective (the adjoint benchmark's): J = sum of rho^2 over the cells whose
centre lies at radius 0.6 <= r <= 0.8 from (1, 1), at the final step; the
gradient is taken with respect to the initial rho and p fields (E =
p/(gamma-1) at u = v = 0).  Initial state: the blast of [0,2]^2 (rho 1, p 1
inside radius 0.4, rho 0.125, p 0.1 outside), optionally times a smooth
perturbation.

Checks:
  * exactness: the FP64 GPU adjoint's directional derivatives against a
    forward-mode (dual-number) derivative of the same discrete step computed
    on the CPU (tests/adjoint/adj_check.cpp, file mode) -- same branch
    decisions, no truncation error;
  * central finite differences of the FP64 forward (eps 1e-6, the frozen dt
    sequence) along seeded Gaussian directions.  Minmod is only piecewise
    linear: every limiter argument that crosses zero (or |a| = |b|) within
    the eps-perturbation adds an O(eps) error to the difference quotient,
    and on the exactly piecewise-constant blast every ambient cell sits on
    such a kink (minmod(eps a, eps b) = eps minmod(a, b) is not linear in the
    direction).  The difference quotients are therefore compared on the
    smoothly perturbed blast with a tolerance that reflects the kinks, and
    their error is shown to shrink with eps;
  * the FP32 adjoint of the FP32 forward against the FP64 adjoint;
  * checkpoint recomputation is bit-reproducible; the checkpointed forward
    equals eu_step_n; the torch.autograd wrapper returns the adjoint.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAMMA = 1.4
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available for the forward-mode reference")
    exe = tmp_path_factory.mktemp("adj") / "adj_check"
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "large_sys_eq_opt_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "adjoint", "adj_check.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


@pytest.fixture(scope="module")
def E():
    import large_sys_eq_opt_gb300.euler2d as E
    E.load()
    return E


def geometry(n, m=None):
    m = n if m is None else m
    from large_sys_eq_opt_gb300.cases import CaseConfig
    return CaseConfig(n, m, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.25)


def centres(cfg):
    dx = (cfg.x_max - cfg.x_min) / cfg.nx
    dy = (cfg.y_max - cfg.y_min) / cfg.ny
    x = cfg.x_min + (np.arange(cfg.nx) + 0.5) * dx
    y = cfg.y_min + (np.arange(cfg.ny) + 0.5) * dy
    return np.meshgrid(x, y)


def blast_fields(cfg, smooth=1e-3):
    """Blast rho, p times (w, 2 - w) with w = 1 + smooth * (smooth waves)."""
    X, Y = centres(cfg)
    inside = (X - 1.0) ** 2 + (Y - 1.0) ** 2 <= 0.4 ** 2
    rho = np.where(inside, 1.0, 0.125)
    p = np.where(inside, 1.0, 0.1)
    w = 1.0 + smooth * (np.sin(2 * np.pi * (1.3 * X + 0.2)) * np.cos(2 * np.pi * (0.9 * Y + 0.1))
                        + 0.5 * np.sin(2 * np.pi * (2.1 * X + 1.7 * Y)))
    return rho * w, p * (2.0 - w)


def grid_of(cfg, rho, p):
    U = np.zeros((cfg.ny + 4, cfg.nx + 4, 4))
    U[2:-2, 2:-2, 0] = rho
    U[2:-2, 2:-2, 3] = p / (GAMMA - 1.0)
    return U


def ring(cfg):
    X, Y = centres(cfg)
    r = np.sqrt((X - 1.0) ** 2 + (Y - 1.0) ** 2)
    return (r >= 0.6) & (r <= 0.8)


def objective(U, mask):
    return float(np.sum(U[2:-2, 2:-2, 0][mask] ** 2))


def dJ_dU(U, mask):
    g = np.zeros_like(U)
    g[2:-2, 2:-2, 0] = np.where(mask, 2.0 * U[2:-2, 2:-2, 0], 0.0)
    return g


def cfl_dts(E, cfg, U0, solver, nsteps):
    with E.Solver(cfg, "fp64", solver) as s:
        s.upload(U0)
        s.set_dt_log(nsteps)
        s.step_n(nsteps)
        return s.dt_log(nsteps)


def forward_J(s, U0, dts, mask):
    s.upload(U0)
    s.step_n(len(dts), dts)
    return objective(s.download(), mask)


def directions(cfg, count, seed=12345):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        d = rng.standard_normal((2, cfg.ny, cfg.nx))
        out.append(d / np.linalg.norm(d))
    return out


def fd_check(E, cfg, solver, nsteps, k, ndir, bc=None, eps=1e-6, smooth=1e-3):
    rho, p = blast_fields(cfg, smooth)
    U0 = grid_of(cfg, rho, p)
    dts = cfl_dts(E, cfg, U0, solver, nsteps)
    mask = ring(cfg)
    with E.Solver(cfg, "fp64", solver, bc=bc or (0, 0, 0, 0)) as s:
        s.upload(U0)
        s.adjoint_forward(dts, k)
        UN = s.download()
        g = s.adjoint_backward(dJ_dU(UN, mask))
        errs = []
        for d in directions(cfg, ndir):
            ad = float(np.sum(g[2:-2, 2:-2, 0] * d[0]) + np.sum(g[2:-2, 2:-2, 3] * d[1]) / (GAMMA - 1.0))
            Jp = forward_J(s, grid_of(cfg, rho + eps * d[0], p + eps * d[1]), dts, mask)
            Jm = forward_J(s, grid_of(cfg, rho - eps * d[0], p - eps * d[1]), dts, mask)
            fd = (Jp - Jm) / (2 * eps)
            errs.append(abs(ad - fd) / max(abs(fd), 1e-300))
    return errs, g


def forward_mode(harness, tmp, cfg, solver_id, dts, rho, p, mask, dirs, bc):
    """Directional derivatives of J by the CPU forward-mode reference."""
    fin, fout = tmp / "problem.bin", tmp / "result.bin"
    hdr = np.array([cfg.nx, cfg.ny, solver_id, len(dts), *bc, len(dirs)], dtype=np.int32)
    with open(fin, "wb") as f:
        f.write(hdr.tobytes())
        f.write(np.array([2.0 / cfg.nx, 2.0 / cfg.ny]).tobytes())
        for a in (np.asarray(dts), rho, p, mask.astype(np.float64)):
            f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())
        for d in dirs:
            f.write(np.ascontiguousarray(d, dtype=np.float64).tobytes())
    r = subprocess.run([harness, str(fin), str(fout)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = np.fromfile(fout, dtype=np.float64)
    return out[:len(dirs)], out[len(dirs):]


def adjoint_dirs(g, dirs):
    return np.array([np.sum(g[2:-2, 2:-2, 0] * d[0]) + np.sum(g[2:-2, 2:-2, 3] * d[1]) / (GAMMA - 1.0)
                     for d in dirs])


SOLVER_ID = {"hll": 0, "hllc": 1, "exact": 2, "force": 3}


@pytest.mark.parametrize("solver,smooth,bc", [("hll", 1e-3, (0, 0, 0, 0)), ("hllc", 1e-3, (0, 0, 0, 0)),
                                              ("exact", 1e-3, (0, 0, 0, 0)), ("force", 1e-3, (0, 0, 0, 0)),
                                              ("hllc", 1e-3, (1, 0, 1, 1)), ("exact", 2e-2, (1, 1, 0, 1))])
def test_adjoint_matches_forward_mode(E, harness, tmp_path, solver, smooth, bc):
    """48x40 grid, 30 CFL steps, checkpoints every 7 (partial last segment):
    GPU FP64 adjoint = forward-mode derivative to 1e-8 relative.

    The exactly piecewise-constant blast is checked on the CPU only
    (adj_check.cpp): there every ambient limiter argument is an exact tie,
    and whether a tie survives a step depends on the last bit of the
    forward's rounding (the GPU's fused multiply-adds leave 1-ulp ripples
    that the CPU restatement does not), so the two trajectories take
    different -- equally valid -- branches."""
    cfg = geometry(48, 40)
    rho, p = blast_fields(cfg, smooth)
    U0 = grid_of(cfg, rho, p)
    dts = cfl_dts(E, cfg, U0, solver, 30)
    mask = ring(cfg)
    dirs = directions(cfg, 4)
    with E.Solver(cfg, "fp64", solver, bc=bc) as s:
        s.upload(U0)
        s.adjoint_forward(dts, 7)
        g = s.adjoint_backward(dJ_dU(s.download(), mask))
    ad = adjoint_dirs(g, dirs)
    fm, cpu_ad = forward_mode(harness, tmp_path, cfg, SOLVER_ID[solver], dts, rho, p, mask,
                              [d.reshape(-1) for d in dirs], bc)
    np.testing.assert_allclose(cpu_ad, fm, rtol=1e-12)
    np.testing.assert_allclose(ad, fm, rtol=1e-8)


@pytest.mark.parametrize("solver", ("hll", "hllc", "exact", "force"))
def test_adjoint_fd_small(E, solver):
    """Central differences on the 48x40 case: agreement to the kink-limited
    level, and the error shrinks as eps does."""
    cfg = geometry(48, 40)
    e6, _ = fd_check(E, cfg, solver, 30, 7, 4, eps=1e-6, smooth=2e-2)
    e7, _ = fd_check(E, cfg, solver, 30, 7, 4, eps=1e-7, smooth=2e-2)
    print(solver, "fd rel err eps=1e-6", ["%.1e" % e for e in e6], "eps=1e-7", ["%.1e" % e for e in e7])
    assert np.median(e6) <= 1e-3
    assert np.median(e7) <= np.median(e6)


def test_adjoint_backward_repeatable(E):
    """A second backward (every segment recomputed from its checkpoint)
    reproduces the first (last segment still in the ring) bit for bit."""
    cfg = geometry(64)
    rho, p = blast_fields(cfg)
    U0 = grid_of(cfg, rho, p)
    dts = cfl_dts(E, cfg, U0, "hllc", 40)
    mask = ring(cfg)
    with E.Solver(cfg, "fp32", "hllc") as s:
        s.upload(U0)
        s.adjoint_forward(dts, 8)
        gN = dJ_dU(s.download(), mask)
        g1 = s.adjoint_backward(gN)
        g2 = s.adjoint_backward(gN)
    assert np.array_equal(g1, g2)
    assert np.all(g1[:2] == 0) and np.all(g1[:, :2] == 0)


def test_adjoint_forward_matches_step_n(E):
    """The checkpointed forward lands on the same state as eu_step_n."""
    cfg = geometry(96, 80)
    rho, p = blast_fields(cfg)
    U0 = grid_of(cfg, rho, p)
    dts = cfl_dts(E, cfg, U0, "exact", 21)
    for prec in ("fp64", "fp32"):
        with E.Solver(cfg, prec, "exact") as s:
            s.upload(U0)
            s.adjoint_forward(dts, 4)
            a = s.download()
            t, n, _ = s.time()
            s.upload(U0)
            s.step_n(len(dts), dts)
            b = s.download()
        assert np.array_equal(a, b), prec
        assert n >= 21 and abs(t - float(np.sum(dts))) <= 1e-12


@pytest.mark.parametrize("prec,solver", [("fp32", "hllc"), ("fp64", "hllc"), ("fp32", "exact")])
def test_cfl_adjoint_forward_equals_frozen(E, prec, solver):
    """eu_adjoint_forward without a dt list takes eu_step_n's CFL steps
    (the same sizes and state, 19 steps over checkpoints of 4) and its
    backward equals, bit for bit, the backward of a forward given those
    sizes."""
    cfg = geometry(96, 80)
    rho, p = blast_fields(cfg)
    U0 = grid_of(cfg, rho, p)
    mask = ring(cfg)
    with E.Solver(cfg, prec, solver) as s:
        s.upload(U0)
        s.set_dt_log(19)
        s.step_n(19)
        plain, plain_dts = s.download(), s.dt_log(19)
        s.upload(U0)
        s.adjoint_forward(None, 4, nsteps=19)
        a = s.download()
        dts = s.adjoint_dts()
        g1 = s.adjoint_backward(dJ_dU(a, mask))
        s.upload(U0)
        s.adjoint_forward(dts, 4)
        b = s.download()
        g2 = s.adjoint_backward(dJ_dU(b, mask))
    assert np.array_equal(dts, plain_dts)
    assert np.array_equal(a, plain) and np.array_equal(b, plain)
    assert np.array_equal(g1, g2)
    assert np.any(g1 != 0)


def test_adjoint_config_512(E):
    """The adjoint benchmark geometry: 512^2, HLLC + minmod, 400 frozen-dt
    steps, checkpoints every 32, 16 seeded Gaussian directions, central
    differences with eps = 1e-6 of the FP64 forward; the FP32 adjoint of the
    FP32 forward against the FP64 adjoint."""
    cfg = geometry(512)
    errs, g64 = fd_check(E, cfg, "hllc", 400, 32, 16, smooth=2e-2)
    print("fd rel errors", ["%.2e" % e for e in errs], "median %.2e" % np.median(errs))
    # unfrozen differences cross limiter kinks (measured: median 7.6e-5, max
    # 3.4e-4); the branch-frozen check below holds the adjoint to 1e-6
    assert np.median(errs) <= 2e-4 and max(errs) <= 1e-3
    rho, p = blast_fields(cfg, 2e-2)
    U0 = grid_of(cfg, rho, p)
    dts = cfl_dts(E, cfg, U0, "hllc", 400)
    with E.Solver(cfg, "fp32", "hllc") as s:
        s.upload(U0)
        s.adjoint_forward(dts, 32)
        g32 = s.adjoint_backward(dJ_dU(s.download(), ring(cfg)))
        ms = s.adjoint_timing()
    a = np.concatenate([g64[..., 0].ravel(), g64[..., 3].ravel()])
    b = np.concatenate([g32[..., 0].ravel(), g32[..., 3].ravel()])
    rel = np.linalg.norm(a - b) / np.linalg.norm(a)
    print("fp32 vs fp64 adjoint relative L2 %.3e; fp32 forward %.2f ms, backward %.2f ms" % (rel, ms[0], ms[1]))
    assert rel <= 3e-3   # measured 1.3e-3


def test_adjoint_config_512_branch_frozen_fd(E):
    """The adjoint benchmark size against branch-frozen central differences:
    512^2 perturbed blast, HLLC + minmod, 400 steps on the oracle's frozen
    dt sequence, checkpoints every 32, 16 portable seeded Gaussian
    directions.  The reference values come from the CPU oracle run with
    every lane's branch decisions taken from the unperturbed run
    (tests/golden/frozen_fd_512.json, made by tests/golden/make_frozen_fd.py),
    so no limiter or fallback kink is crossed inside the difference and the
    quotient's truncation error is O(eps^2).  What limits a difference
    quotient of 400 FP64 steps is then rounding noise in the +-eps runs,
    which grows as 1/eps: at eps = 1e-3 the quotient is good to ~1e-8 and
    the FP64 GPU adjoint must match every direction to 1e-6; at eps = 1e-6
    (reported) the noise alone is ~1e-5.  The fixture also counts, per
    direction, the decisions on which free +eps and -eps runs would differ:
    those flips are what limits the unfrozen check above."""
    import json
    import sys
    gold = os.path.join(ROOT, "tests", "golden")
    if gold not in sys.path:
        sys.path.insert(0, gold)
    import make_frozen_fd as M
    with open(os.path.join(gold, "frozen_fd_512.json")) as f:
        d = json.load(f)
    n = d["n"]
    rho, p = M.blast_fields(n, d["smooth"])
    U0 = M.initial_grid(n, rho, p)
    dts = np.array(d["dts"])
    mask = M.ring(n)
    big, small = d["by_eps"]["0.001"], d["by_eps"]["1e-06"]
    dirs = M.directions(n, len(big["fd"]), d["seed"])
    with E.Solver(geometry(n), "fp64", d["solver"]) as s:
        s.upload(U0)
        s.adjoint_forward(dts, 32)
        UN = s.download()
        g = s.adjoint_backward(dJ_dU(UN, mask))
    J = objective(UN, mask)
    assert abs(J - d["J0"]) <= 1e-10 * abs(d["J0"]), (J, d["J0"])
    ad = adjoint_dirs(g, dirs)
    rel = np.abs(ad - np.array(big["fd"])) / np.abs(np.array(big["fd"]))
    rel6 = np.abs(ad - np.array(small["fd"])) / np.abs(np.array(small["fd"]))
    print("branch-frozen fd, eps 1e-3: rel errors", ["%.1e" % e for e in rel], "max %.2e" % rel.max())
    print("branch-frozen fd, eps 1e-6: rel errors", ["%.1e" % e for e in rel6], "median %.2e" % np.median(rel6))
    print("branch flips between free +eps and -eps runs per direction (eps 1e-6)", small["flips"])
    assert rel.max() <= 1e-6


def test_autograd_wrapper(E):
    import torch
    from large_sys_eq_opt_gb300.autograd import FrozenSteps
    cfg = geometry(48)
    rho, p = blast_fields(cfg)
    U0 = grid_of(cfg, rho, p)
    dts = cfl_dts(E, cfg, U0, "hll", 12)
    mask = torch.from_numpy(ring(cfg))
    with E.Solver(cfg, "fp64", "hll") as s:
        x = torch.from_numpy(U0.copy()).requires_grad_(True)
        UN = FrozenSteps.apply(x, s, dts, 5)
        J = (UN[2:-2, 2:-2, 0][mask] ** 2).sum()
        J.backward()
        s.upload(U0)
        s.adjoint_forward(dts, 5)
        ref = s.adjoint_backward(dJ_dU(s.download(), mask.numpy()))
    np.testing.assert_allclose(x.grad.numpy(), ref, rtol=0, atol=0)
