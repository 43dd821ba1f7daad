"""Problem setup: the reference's case table and the parameterised cases.

Mirrors the reference's setup surface (head/test_cases.hpp:8-35,
src/test_cases.cpp:104-195): ``CaseConfig``, ``parse_case_id``,
``get_case_config``, ``get_n_case_config``, and extends it with
parameterised blast / shock-bubble descriptions so the benchmark workloads
(256^2 blast, 1000x396 shock-bubble with reflective walls, 8192^2 blast,
512^2 adjoint blast, uneven ensembles) can be expressed.  Initial states are
evaluated on the device by the library (``eu_init_*``); the formulas are those
of src/test_cases.cpp:11-101.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

GAMMA = 1.4  # head/physics.hpp:11

TRANSMISSIVE = 0
REFLECTIVE = 1


@dataclass
class CaseConfig:
    """head/test_cases.hpp:8-18 (ng is fixed at 2 by the solver)."""
    nx: int
    ny: int
    ng: int
    x_min: float
    x_max: float
    y_min: float
    y_max: float
    cfl: float
    t_end: float


@dataclass
class BlastParams:
    """Cylindrical blast: state (rho_in, p_in) where r^2 <= R^2 from (cx, cy),
    (rho_out, p_out) elsewhere, at rest (src/test_cases.cpp:78-101)."""
    cx: float = 1.0
    cy: float = 1.0
    r: float = 0.4
    rho_in: float = 1.0
    p_in: float = 1.0
    rho_out: float = 0.125
    p_out: float = 0.1


@dataclass
class ShockBubbleParams:
    """Planar shock of Mach ``mach`` at x < shock_x into ambient (rho0, p0),
    post-shock state from the Rankine-Hugoniot relations; a bubble of density
    rho_bubble (pressure unchanged) of radius bub_r at (bub_cx, bub_cy)
    (src/test_cases.cpp:24-69)."""
    rho0: float = 1.0
    p0: float = 1.0
    mach: float = 1.22
    shock_x: float = 0.005
    bub_cx: float = 0.035
    bub_cy: float = 0.0445
    bub_r: float = 0.025
    rho_bubble: float = 0.138


@dataclass
class Problem:
    """A case the GPU library can initialise and run: geometry + CFL/t_end,
    boundary condition per side (left, right, bottom, top) and the state."""
    cfg: CaseConfig
    kind: str                     # "blast" | "shock_bubble"
    params: object
    bc: tuple = (TRANSMISSIVE,) * 4
    nsnap: int = 5
    name: str = ""


_CASES = {
    # src/test_cases.cpp:132-162
    "shock_bubble": CaseConfig(500, 197, 2, 0.0, 0.225, 0.0, 0.089, 0.4, 0.0011741),
    "blast_wave": CaseConfig(500, 500, 2, 0.0, 1.0, 0.0, 1.0, 0.4, 0.2),
}

_REFERENCE_PARAMS = {
    # src/test_cases.cpp:25-33 (dimensional air/helium) and :79-89
    "shock_bubble": ShockBubbleParams(rho0=1.29, p0=1.01325e5, mach=1.22, shock_x=0.005,
                                      bub_cx=0.035, bub_cy=0.0445, bub_r=0.025, rho_bubble=0.214),
    "blast_wave": BlastParams(cx=0.5, cy=0.5, r=0.1, rho_in=1.0, p_in=100.0, rho_out=1.0, p_out=1.0),
}


def parse_case_id(name: str) -> str:
    """src/test_cases.cpp:104-117 (raises on an unknown name)."""
    if name not in _CASES:
        raise RuntimeError(f"Unknown case name: {name}. Supported cases are: shock_bubble, blast_wave.")
    return name


def get_case_config(name: str) -> CaseConfig:
    return replace(_CASES[parse_case_id(name)])


def get_n_case_config(name: str, n: int) -> CaseConfig:
    """src/test_cases.cpp:184-195."""
    if n < 1:
        raise RuntimeError("get_n_case_config: n must be >= 1.")
    c = get_case_config(name)
    c.nx *= n
    c.ny *= n
    return c


def reference_problem(name: str, n: int = 1) -> Problem:
    kind = "shock_bubble" if name == "shock_bubble" else "blast"
    return Problem(get_n_case_config(name, n), kind, replace(_REFERENCE_PARAMS[name]),
                   name=f"{name}_n{n}")


# ---------------------------------------------------------------------------
# Benchmark workloads (synthetic inputs with the shapes of the published
# configurations: the reference ships no dataset).
# ---------------------------------------------------------------------------
def blast_256() -> Problem:
    """Cylindrical blast on [0,2]^2, 256^2, transmissive, CFL 0.8, t_end 0.25,
    5 snapshots."""
    return Problem(CaseConfig(256, 256, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.25), "blast", BlastParams(),
                   name="blast_256")


def shock_bubble_1000x396() -> Problem:
    """Single-gas shock-bubble on [0,0.225]x[0,0.089], 1000x396, transmissive
    in x and reflective in y, CFL 0.8, t_end 0.1."""
    return Problem(CaseConfig(1000, 396, 2, 0.0, 0.225, 0.0, 0.089, 0.8, 0.1), "shock_bubble",
                   ShockBubbleParams(), bc=(TRANSMISSIVE, TRANSMISSIVE, REFLECTIVE, REFLECTIVE),
                   name="shock_bubble_1000x396")


def blast_large(n: int = 8192) -> Problem:
    """The 256^2 blast geometry at n x n cells (throughput workload)."""
    return Problem(CaseConfig(n, n, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.25), "blast", BlastParams(),
                   name=f"blast_{n}")


def blast_adjoint_512() -> Problem:
    return Problem(CaseConfig(512, 512, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.25), "blast", BlastParams(),
                   name="blast_512_adjoint")


def post_shock_state(p: ShockBubbleParams):
    """Rankine-Hugoniot post-shock (rho2, u2, p2) (src/test_cases.cpp:35-46)."""
    a0 = math.sqrt(GAMMA * p.p0 / p.rho0)
    M2 = p.mach * p.mach
    rho2 = p.rho0 * ((GAMMA + 1.0) * M2) / ((GAMMA - 1.0) * M2 + 2.0)
    p2 = p.p0 * (1.0 + 2.0 * GAMMA / (GAMMA + 1.0) * (M2 - 1.0))
    u2 = 2.0 * a0 / (GAMMA + 1.0) * (p.mach - 1.0 / p.mach)
    return rho2, u2, p2


def ensemble_problems(seed: int = 2024, n_blast: int = 48, n_bubble: int = 16) -> list:
    """The uneven ensemble workload (fixed seed): n_blast blasts on [0,2]^2
    with inner radius U[0.2, 0.5], inner p log-uniform in [1, 100], inner rho
    1, outer rho 0.125 and p 0.1, on grids drawn from {128^2, 256^2, 512^2,
    1024^2} (transmissive, CFL 0.8, t_end 0.25); and n_bubble shock-bubbles
    on [0,0.225]x[0,0.089] with bubble rho U[0.1, 3.0] and Mach U[1.1, 2.0]
    on nx uniform in [500, 2000], ny = round(0.396 nx) (reflective in y,
    CFL 0.8, t_end 0.1)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_blast):
        n = int(rng.choice([128, 256, 512, 1024]))
        r = float(rng.uniform(0.2, 0.5))
        p_in = float(10.0 ** rng.uniform(0.0, 2.0))
        out.append(Problem(CaseConfig(n, n, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.25), "blast",
                           BlastParams(r=r, p_in=p_in), name=f"blast{k}_{n}"))
    for k in range(n_bubble):
        nx = int(rng.integers(500, 2001))
        ny = int(round(0.396 * nx))
        rho_b = float(rng.uniform(0.1, 3.0))
        mach = float(rng.uniform(1.1, 2.0))
        out.append(Problem(CaseConfig(nx, ny, 2, 0.0, 0.225, 0.0, 0.089, 0.8, 0.1), "shock_bubble",
                           ShockBubbleParams(mach=mach, rho_bubble=rho_b),
                           bc=(TRANSMISSIVE, TRANSMISSIVE, REFLECTIVE, REFLECTIVE), name=f"bubble{k}_{nx}x{ny}"))
    return out

