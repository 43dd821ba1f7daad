"""Discrete adjoint on the GPU (eu_adjoint_forward / eu_adjoint_backward)
against central finite differences of the FP64 forward with the same frozen
dt sequence, an FP64 build of the same adjoint, and the torch.autograd
wrapper.

Objective (the adjoint benchmark's): J = sum of rho^2 over the cells whose
centre lies at radius 0.6 <= r <= 0.8 from (1, 1), at the final step; the
gradient is taken with respect to the initial rho and p fields (E =
p/(gamma-1) at u = v = 0).

The initial state is the blast of [0,2]^2 (rho 1, p 1 inside radius 0.4,
rho 0.125, p 0.1 outside) plus a smooth perturbation of relative amplitude
1e-3.  Without it the ambient region is exactly uniform, every limiter
argument there is exactly zero, and minmod's one-sided response to a
perturbation (minmod(eps a, eps b) = eps minmod(a, b)) is not linear in the
direction -- no gradient reproduces it, so finite differences of the exact
piecewise-constant blast disagree with any adjoint there.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAMMA = 1.4


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


def fd_check(E, cfg, solver, nsteps, k, ndir, bc=None, eps=1e-6):
    rho, p = blast_fields(cfg)
    U0 = grid_of(cfg, rho, p)
    dts = cfl_dts(E, cfg, U0, solver, nsteps)
    mask = ring(cfg)
    with E.Solver(cfg, "fp64", solver, bc=bc) as s:
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


@pytest.mark.parametrize("solver", ("hll", "hllc", "exact", "force"))
def test_adjoint_fd_small(E, solver):
    """48x40 grid, 30 steps, checkpoints every 7 (a partial last segment)."""
    errs, _ = fd_check(E, geometry(48, 40), solver, 30, 7, 4)
    assert max(errs) <= 1e-6, errs


def test_adjoint_fd_reflective(E):
    errs, _ = fd_check(E, geometry(40, 36), "hllc", 24, 5, 4, bc=(1, 0, 1, 1))
    assert max(errs) <= 1e-6, errs


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


def test_adjoint_config_512(E):
    """The adjoint benchmark geometry: 512^2, HLLC + minmod, 400 frozen-dt
    steps, checkpoints every 32; FP64 adjoint within 1e-6 of central FD
    (eps 1e-6, FP64 forward) along 16 seeded Gaussian directions; the FP32
    adjoint of the FP32 forward against the FP64 adjoint."""
    cfg = geometry(512)
    errs, g64 = fd_check(E, cfg, "hllc", 400, 32, 16)
    print("fd rel errors", ["%.2e" % e for e in errs])
    assert max(errs) <= 1e-6, errs
    rho, p = blast_fields(cfg)
    U0 = grid_of(cfg, rho, p)
    dts = cfl_dts(E, cfg, U0, "hllc", 400)
    with E.Solver(cfg, "fp32", "hllc") as s:
        s.upload(U0)
        s.adjoint_forward(dts, 32)
        g32 = s.adjoint_backward(dJ_dU(s.download(), ring(cfg)))
    a = np.concatenate([g64[..., 0].ravel(), g64[..., 3].ravel()])
    b = np.concatenate([g32[..., 0].ravel(), g32[..., 3].ravel()])
    rel = np.linalg.norm(a - b) / np.linalg.norm(a)
    print("fp32 vs fp64 adjoint relative L2", rel)
    assert rel <= 5e-2


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
