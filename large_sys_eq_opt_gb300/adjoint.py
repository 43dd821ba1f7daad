"""Gradients of an instance objective with respect to its scalar case
parameters, through the discrete adjoint (batched over an ensemble).

For every instance the objective is of the adjoint benchmark's kind:
  blast          J = sum rho^2 over cells with 0.6 <= r <= 0.8 from the
                 blast centre, after the instance's frozen steps;
  shock-bubble   J = sum rho^2 over cells with 1.2 r_b <= d <= 1.6 r_b from
                 the bubble centre.
dJ/dtheta = <dJ/dU_0, dU_0/dtheta>, with dJ/dU_0 from eu_batch_adjoint_* and
dU_0/dtheta from the closed-form initial states below:
  blast p_in     the inside state's energy p_in/(gamma-1);
  blast R        measure-based: the inside indicator is the one-cell linear
                 ramp frac = clip(1/2 - (r - R)/h, 0, 1), h = min(dx, dy)
                 (the cell-average of a straight interface crossing the
                 cell), so dU_0/dR = (U_in - U_out)/h on the ramp cells --
                 the differentiated instances start from this ramped state;
  bubble rho_b   the bubble cells' density (E is unchanged: u = 0 there);
  Mach           the Rankine-Hugoniot post-shock state left of the shock
                 (src/test_cases.cpp:35-46), differentiated in closed form.
"""
from __future__ import annotations

import math

import numpy as np

from .cases import BlastParams, Problem, ShockBubbleParams

GAMMA = 1.4
G1 = GAMMA - 1.0


def centres(cfg):
    dx = (cfg.x_max - cfg.x_min) / cfg.nx
    dy = (cfg.y_max - cfg.y_min) / cfg.ny
    x = cfg.x_min + (np.arange(cfg.nx) + 0.5) * dx
    y = cfg.y_min + (np.arange(cfg.ny) + 0.5) * dy
    X, Y = np.meshgrid(x, y)
    return X, Y, dx, dy


def _grid(cfg, rho, mx, my, E):
    U = np.zeros((cfg.ny + 4, cfg.nx + 4, 4))
    U[2:-2, 2:-2, 0] = rho
    U[2:-2, 2:-2, 1] = mx
    U[2:-2, 2:-2, 2] = my
    U[2:-2, 2:-2, 3] = E
    return U


def blast_state(prob: Problem):
    """Ramped blast state and its tangents {"r": dU/dR, "p_in": dU/dp_in}."""
    cfg, b = prob.cfg, prob.params
    X, Y, dx, dy = centres(cfg)
    h = min(dx, dy)
    r = np.sqrt((X - b.cx) ** 2 + (Y - b.cy) ** 2)
    s = 0.5 - (r - b.r) / h
    frac = np.clip(s, 0.0, 1.0)
    ramp = (s > 0.0) & (s < 1.0)
    rho = b.rho_out + frac * (b.rho_in - b.rho_out)
    p = b.p_out + frac * (b.p_in - b.p_out)
    U = _grid(cfg, rho, 0.0, 0.0, p / G1)
    dfrac = np.where(ramp, 1.0 / h, 0.0)
    dR = _grid(cfg, dfrac * (b.rho_in - b.rho_out), 0.0, 0.0, dfrac * (b.p_in - b.p_out) / G1)
    dP = _grid(cfg, 0.0, 0.0, 0.0, frac / G1)
    return U, {"r": dR, "p_in": dP}


def post_shock(p: ShockBubbleParams):
    """(rho2, u2, p2) and their derivatives with respect to the Mach number."""
    a0 = math.sqrt(GAMMA * p.p0 / p.rho0)
    M = p.mach
    M2 = M * M
    den = (GAMMA - 1.0) * M2 + 2.0
    rho2 = p.rho0 * (GAMMA + 1.0) * M2 / den
    p2 = p.p0 * (1.0 + 2.0 * GAMMA / (GAMMA + 1.0) * (M2 - 1.0))
    u2 = 2.0 * a0 / (GAMMA + 1.0) * (M - 1.0 / M)
    drho2 = p.rho0 * (GAMMA + 1.0) * 4.0 * M / (den * den)
    dp2 = p.p0 * 2.0 * GAMMA / (GAMMA + 1.0) * 2.0 * M
    du2 = 2.0 * a0 / (GAMMA + 1.0) * (1.0 + 1.0 / M2)
    return (rho2, u2, p2), (drho2, du2, dp2)


def bubble_state(prob: Problem):
    """Shock-bubble state (cell centres, as the device initialiser) and its
    tangents {"rho_bubble": ..., "mach": ...}."""
    cfg, s = prob.cfg, prob.params
    X, Y, _, _ = centres(cfg)
    (rho2, u2, p2), (drho2, du2, dp2) = post_shock(s)
    left = X < s.shock_x
    bub = (X - s.bub_cx) ** 2 + (Y - s.bub_cy) ** 2 <= s.bub_r * s.bub_r
    rho = np.where(left, rho2, s.rho0)
    u = np.where(left, u2, 0.0)
    p = np.where(left, p2, s.p0)
    rho = np.where(bub, s.rho_bubble, rho)
    U = _grid(cfg, rho, rho * u, 0.0, p / G1 + 0.5 * rho * u * u)
    L = left & ~bub
    dM = _grid(cfg, np.where(L, drho2, 0.0), np.where(L, drho2 * u2 + rho2 * du2, 0.0), 0.0,
               np.where(L, dp2 / G1 + 0.5 * (drho2 * u2 * u2 + 2.0 * rho2 * u2 * du2), 0.0))
    dB = _grid(cfg, np.where(bub, 1.0, 0.0), np.where(bub, u, 0.0), 0.0, np.where(bub, 0.5 * u * u, 0.0))
    return U, {"rho_bubble": dB, "mach": dM}


def initial_state(prob: Problem):
    if isinstance(prob.params, BlastParams):
        return blast_state(prob)
    return bubble_state(prob)


def objective_mask(prob: Problem) -> np.ndarray:
    X, Y, _, _ = centres(prob.cfg)
    if isinstance(prob.params, BlastParams):
        b = prob.params
        r = np.sqrt((X - b.cx) ** 2 + (Y - b.cy) ** 2)
        return (r >= 0.6) & (r <= 0.8)
    s = prob.params
    d = np.sqrt((X - s.bub_cx) ** 2 + (Y - s.bub_cy) ** 2)
    return (d >= 1.2 * s.bub_r) & (d <= 1.6 * s.bub_r)


def objective(U: np.ndarray, mask: np.ndarray) -> float:
    return float(np.sum(U[2:-2, 2:-2, 0][mask] ** 2))


def objective_grad(U: np.ndarray, mask: np.ndarray) -> np.ndarray:
    g = np.zeros_like(U)
    g[2:-2, 2:-2, 0] = np.where(mask, 2.0 * U[2:-2, 2:-2, 0], 0.0)
    return g


PARAM_NAMES = {"blast": ("r", "p_in"), "shock_bubble": ("rho_bubble", "mach")}


def ensemble_parameter_gradients(E, problems, nsteps: int, precision="fp32", solver="hllc", ckpt_k: int = 0,
                                 batch=None, device=True, timing: dict | None = None):
    """J and dJ/dtheta of every instance after (at most) nsteps CFL steps,
    each instance stopping at its own t_end; the step sizes are then held
    fixed.

    device=True keeps everything on the GPU (eu_batch_param_gradients):
    initial states, the checkpointed forwards -- which take the CFL steps
    themselves and log their sizes, the same steps as an ensemble run --,
    objective, dJ/dU_N, backward sweeps and the tangent contractions, all
    instances concurrently.  device=False is the same computation with the
    dt lists from one ensemble run and the grids passing through host
    arrays and the formulas of this module.  Returns (J list, gradient dict
    list, dts list, batch); `timing`, when given, receives the wall seconds
    of the gradient call ("gradients_s") on the device path."""
    own = batch is None
    b = batch if batch is not None else E.Batch(problems, precision, solver)
    try:
        if device:
            import time
            t1 = time.perf_counter()
            J, dJ = b.param_gradients(problems, None, ckpt_k, nsteps=nsteps)
            if timing is not None:
                timing["gradients_s"] = time.perf_counter() - t1
            dts = [inst.adjoint_dts() for inst in b.instances]
            kinds = ["blast" if isinstance(p.params, BlastParams) else "shock_bubble" for p in problems]
            grads = [dict(zip(PARAM_NAMES[k], map(float, g))) for k, g in zip(kinds, dJ)]
            return [float(x) for x in J], grads, dts, b
        states = [initial_state(p) for p in problems]
        for inst, (U0, _) in zip(b.instances, states):
            inst.upload(U0)
            inst.set_dt_log(nsteps)
        b.start()
        b.step(nsteps)
        dts = []
        for inst in b.instances:
            _, n, _ = inst.time()
            dts.append(inst.dt_log(min(n, nsteps)))
        for inst, (U0, _) in zip(b.instances, states):
            inst.upload(U0)
        b.adjoint_forward(dts, ckpt_k)
        masks = [objective_mask(p) for p in problems]
        finals = [inst.download() for inst in b.instances]
        Js = [objective(U, m) for U, m in zip(finals, masks)]
        gU0 = b.adjoint_backward([objective_grad(U, m) for U, m in zip(finals, masks)])
        grads = [{k: float(np.sum(g * t)) for k, t in tang.items()} for g, (_, tang) in zip(gU0, states)]
        return Js, grads, dts, b
    finally:
        if own:
            b.close()
