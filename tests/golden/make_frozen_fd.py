"""Generate tests/golden/frozen_fd_512.json: branch-frozen central differences
of the adjoint benchmark's objective, the reference for the GPU adjoint at
the benchmark size (TEST FIXTURE GENERATOR; runs the CPU oracle only).

Workload (the adjoint benchmark): the blast of [0,2]^2 at 512^2 (rho 1, p 1
inside radius 0.4 of (1, 1), rho 0.125, p 0.1 outside, u = v = 0) times a
smooth 2% perturbation (w, 2 - w), HLLC + minmod, transmissive, 400 steps
with the CFL 0.8 dt sequence of the oracle's own run frozen; objective
J = sum of rho^2 over the cells with 0.6 <= r <= 0.8 at the end; 16
directions in (rho, p) with independent N(0, 1) entries from a portable
generator (SplitMix64 + Box-Muller, seed 12345), normalised.

For each direction and for eps = 1e-3 and 1e-6 the fixture holds the
branch-frozen difference quotient (oracle/shadow_fd.cpp: the +-eps runs
replay the unperturbed run's limiter, fallback and Riemann branch
decisions) and the number of decisions on which free +eps and -eps runs
would differ.  It also holds the frozen dt sequence, which the GPU test
replays.

Why two eps: with the branches frozen the map is smooth, so the quotient's
truncation error is O(eps^2) and small even at eps = 1e-3; what limits it
is rounding noise in the +-eps forward runs, which grows as 1/eps (400
FP64 steps: ~1e-5 relative at eps = 1e-6, ~1e-8 at 1e-3, measured on the
256^2 case against a forward-mode derivative).  eps = 1e-3 is the check at
the 1e-6 bar; eps = 1e-6 is reported beside it.

Usage: python tests/golden/make_frozen_fd.py [n] [nsteps]  (about 10 minutes
on 8 cores at the default 512 / 400).
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

GAMMA_M1 = 0.3999999999999999     # head/physics.hpp:11, GAMMA - 1
SEED = 12345
EPS = (1e-3, 1e-6)
SMOOTH = 2e-2
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser of uint64 counters (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def gaussian(seed: int, stream: int, count: int) -> np.ndarray:
    """count N(0, 1) values, Box-Muller on two SplitMix64 uniforms per value;
    the same on every platform up to the last bit of log / cos."""
    base = np.uint64((seed * 1000003 + stream) & 0xFFFFFFFFFFFFFFFF) << np.uint64(24)
    i = np.arange(count, dtype=np.uint64)
    with np.errstate(over="ignore"):
        a = _splitmix64(base + np.uint64(2) * i)
        b = _splitmix64(base + np.uint64(2) * i + np.uint64(1))
    u1 = ((a >> np.uint64(11)).astype(np.float64) + 1.0) * 2.0 ** -53    # (0, 1]
    u2 = (b >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def directions(n: int, count: int = 16, seed: int = SEED):
    """count normalised (rho, p) directions of shape (2, n, n)."""
    out = []
    for k in range(count):
        d = gaussian(seed, k, 2 * n * n).reshape(2, n, n)
        out.append(d / np.linalg.norm(d))
    return out


def centres(n: int):
    x = (np.arange(n) + 0.5) * (2.0 / n)
    return np.meshgrid(x, x)


def blast_fields(n: int, smooth: float = SMOOTH):
    X, Y = centres(n)
    inside = (X - 1.0) ** 2 + (Y - 1.0) ** 2 <= 0.4 ** 2
    w = 1.0 + smooth * (np.sin(2 * np.pi * (1.3 * X + 0.2)) * np.cos(2 * np.pi * (0.9 * Y + 0.1))
                        + 0.5 * np.sin(2 * np.pi * (2.1 * X + 1.7 * Y)))
    return np.where(inside, 1.0, 0.125) * w, np.where(inside, 1.0, 0.1) * (2.0 - w)


def ring(n: int):
    X, Y = centres(n)
    r = np.sqrt((X - 1.0) ** 2 + (Y - 1.0) ** 2)
    return (r >= 0.6) & (r <= 0.8)


def initial_grid(n: int, rho, p):
    U = np.zeros((n + 4, n + 4, 4))
    U[2:-2, 2:-2, 0] = rho
    U[2:-2, 2:-2, 3] = p / GAMMA_M1
    return U


def build_case(n: int, nsteps: int, solver: str = "hllc"):
    """Grid, initial state, the oracle's CFL dt sequence, mask, directions."""
    from oracle import oracle as O
    P = O.Oracle("port")
    g = O.Grid(n, n, 0.0, 2.0, 0.0, 2.0)
    rho, p = blast_fields(n)
    U0 = initial_grid(n, rho, p)
    V = U0.copy()
    r = P.run(V, g, 0.8, 1e30, solver, max_steps=nsteps)
    return g, U0, r["dts"], ring(n), directions(n)


def main():
    from oracle import oracle as O
    O.build(reference=False)
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 512
    nsteps = int(sys.argv[2]) if len(sys.argv) > 2 else 400
    g, U0, dts, mask, dirs = build_case(n, nsteps)
    out = {"workload": f"blast_{n}x{n}_hllc_{nsteps}steps_smooth{SMOOTH}", "n": n, "nsteps": nsteps,
           "solver": "hllc", "smooth": SMOOTH, "seed": SEED,
           "objective": "sum rho^2 over 0.6 <= r <= 0.8 from (1, 1)",
           "directions": "SplitMix64 + Box-Muller N(0,1) in (rho, p), normalised",
           "dts": [float(x) for x in dts], "by_eps": {}}
    t0 = time.time()
    for eps in EPS:
        res = O.frozen_fd(U0, g, dts, "hllc", dirs, eps, mask)
        out["J0"] = res["J0"]
        out["by_eps"][repr(eps)] = {"eps": eps, "fd": res["fd"].tolist(), "Jp": res["Jp"].tolist(),
                                    "Jm": res["Jm"].tolist(), "flips": [int(x) for x in res["flips"]]}
    el = time.time() - t0
    out["seconds"] = el
    path = os.path.join(HERE, f"frozen_fd_{n}.json")
    with open(path, "w") as f:
        json.dump(out, f)
    print(f"wrote {path} ({el:.0f} s)")


if __name__ == "__main__":
    main()
