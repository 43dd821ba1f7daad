"""Generate the golden fixtures under tests/golden/ from the UNMODIFIED reference
CPU solver (oracle/_ref/libref_euler2d.so, built by `make -C oracle ref` from
the reference sources).  Run from the repository root:

    make -C oracle ref oracle && python tests/golden/make_golden.py

Outputs (all committed):
  riemann_kat.npz   -- interface fluxes of head/riemann.hpp:650-672 for 1000
                       seeded state pairs (incl. fallback-triggering ones),
                       4 solvers x 2 directions.
  step_cases.npz    -- one compute_dt, one advance_second_order and one
                       advance_first_order (src/cpu/solver_cpu.cpp:287-499)
                       on small odd-sized grids, 4 solvers.
  run_cases.npz     -- full time loops (scripts/cpu/main_cpu.cpp:206-262) of
                       the blast geometry at 48x40 for 4 solvers: dt
                       sequence, snapshot steps/times, final grid.
  run_cases.json    -- 256x256 blast HLLC to t_end=0.25: step count, dt
                       sequence, snapshot schedule and a SHA-256 of the final
                       grid bytes; plus the reference's own logged step
                       counts and snapshot times (validation/*.csv,
                       outputs/baseline/cpu_stdout.txt) as known answers.
"""
from __future__ import annotations

import csv
import hashlib
import json
import os
import re
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle.oracle import REFERENCE_TREE, Grid, Oracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
GM1 = 1.4 - 1.0


def prim_to_cons(rho, u, v, p):
    return np.stack([rho, rho * u, rho * v, p / GM1 + 0.5 * rho * (u * u + v * v)], -1)


def riemann_states(rng, n):
    rho = np.exp(rng.normal(0.0, 1.0, n))
    u = rng.normal(0.0, 1.5, n)
    v = rng.normal(0.0, 1.5, n)
    p = np.exp(rng.normal(0.0, 1.5, n))
    return prim_to_cons(rho, u, v, p)


def make_riemann(R: Oracle, rng):
    n = 1000
    UL, UR = riemann_states(rng, n), riemann_states(rng, n)
    # fallback triggers: negative density, zero energy, near-vacuum, strong
    # rarefaction (states rushing apart), strong shock, non-finite entries
    UL[0:20, 0] *= -1.0
    UR[20:40, 3] = 0.0
    UL[40:60, 0] = 1e-13
    UL[60:100] = prim_to_cons(np.ones(40), -8.0 * np.ones(40), np.zeros(40), 0.01 * np.ones(40))
    UR[60:100] = prim_to_cons(np.ones(40), 8.0 * np.ones(40), np.zeros(40), 0.01 * np.ones(40))
    UL[100:140] = prim_to_cons(np.ones(40), 20.0 * np.ones(40), np.zeros(40), 1000.0 * np.ones(40))
    UR[100:140] = prim_to_cons(0.1 * np.ones(40), -20.0 * np.ones(40), np.zeros(40), 0.01 * np.ones(40))
    UR[140:150, 1] = np.inf
    UL[150:160, 2] = np.nan
    UR[160:200] = UL[160:200]                 # identical states
    F = np.zeros((4, 2, n, 4))
    for s in range(4):
        for d in range(2):
            for k in range(n):
                F[s, d, k] = R.riemann_flux(UL[k], UR[k], d, s)
    return dict(UL=UL, UR=UR, F=F)


def grid_states(O: Oracle, rng):
    """Small odd-sized initial grids (ghosts filled by the reference BC)."""
    cases = {}
    g = Grid(17, 13, 0.0, 2.0, 0.0, 1.5)
    U = O.init_blast(g, cx=1.0, cy=0.7, r=0.45, rho_in=1.0, p_in=1.0, rho_out=0.125, p_out=0.1)
    cases["blast"] = (g, U)
    g = Grid(19, 11, 0.0, 0.225, 0.0, 0.089)
    U = O.init_shock_bubble(g, bub_cx=0.09, bub_cy=0.04, bub_r=0.03, shock_x=0.05)
    cases["shock_bubble"] = (g, U)
    g = Grid(15, 16, -1.0, 1.0, 0.0, 3.0)
    rho = np.exp(rng.normal(0, 0.5, g.shape[:2]))
    u = rng.normal(0, 1.0, g.shape[:2])
    v = rng.normal(0, 1.0, g.shape[:2])
    p = np.exp(rng.normal(0, 0.8, g.shape[:2]))
    cases["random"] = (g, np.ascontiguousarray(prim_to_cons(rho, u, v, p)))
    g = Grid(14, 9, 0.0, 1.0, 0.0, 1.0)
    rho = np.where(rng.random(g.shape[:2]) < 0.15, 1e-11, 1.0)
    u = np.where(rng.random(g.shape[:2]) < 0.5, -6.0, 6.0)
    v = rng.normal(0, 3.0, g.shape[:2])
    p = np.where(rng.random(g.shape[:2]) < 0.2, 1e-10, 2.0)
    cases["near_vacuum"] = (g, np.ascontiguousarray(prim_to_cons(rho, u, v, p)))
    g = Grid(1, 12, 0.0, 0.5, 0.0, 1.0)
    rho = 1.0 + 0.5 * np.sin(np.linspace(0, 6, g.shape[0]))[:, None] * np.ones(g.shape[:2])
    cases["one_column"] = (g, np.ascontiguousarray(prim_to_cons(rho, 0.2 * rho, 0.5 + 0 * rho, 1.0 + 0 * rho)))
    for k in cases:
        cases[k][1].setflags(write=True)
    return cases


def make_steps(R: Oracle, P: Oracle, rng):
    out = {}
    for name, (g, U) in grid_states(P, rng).items():
        R.apply_boundary(U, g)
        try:
            dt = R.compute_dt(U, g, 0.8)
        except RuntimeError:
            dt = 1e-3
        out[f"{name}/geom"] = np.array([g.nx, g.ny, g.x_min, g.x_max, g.y_min, g.y_max])
        out[f"{name}/U"] = U.copy()
        out[f"{name}/dt"] = np.array([dt])
        for s, sname in enumerate(("hll", "hllc", "exact", "force")):
            Utmp, Unew = R.advance_second_order(U, g, dt, s)
            out[f"{name}/{sname}/Utmp"] = Utmp
            out[f"{name}/{sname}/Unew"] = Unew
            out[f"{name}/{sname}/U1"] = R.advance_first_order(U, g, dt, s)
    return out


def make_runs(R: Oracle, P: Oracle):
    out = {}
    g = Grid(48, 40, 0.0, 2.0, 0.0, 2.0)
    for sname in ("hll", "hllc", "exact", "force"):
        U = P.init_blast(g)
        r = R.run(U, g, 0.8, 0.25, sname, nsnap=5)
        out[f"blast48/{sname}/final"] = U
        out[f"blast48/{sname}/dts"] = r["dts"]
        out[f"blast48/{sname}/snap_step"] = r["snap_step"]
        out[f"blast48/{sname}/snap_t"] = r["snap_t"]
        out[f"blast48/{sname}/t"] = np.array([r["t"]])
    g = Grid(48, 40, 0.0, 2.0, 0.0, 2.0)
    out["blast48/U0"] = P.init_blast(g)
    return out


def parse_reference_logs():
    """Step counts logged by the reference (validation/cpu_mpi_fullnode_external_timing_11470.csv)
    and the snapshot times of outputs/baseline/cpu_stdout.txt:1-8."""
    steps = {}
    path = os.path.join(REFERENCE_TREE, "validation", "cpu_mpi_fullnode_external_timing_11470.csv")
    with open(path) as f:
        for lineno, row in enumerate(csv.DictReader(f), start=2):
            if row["arch"] == "cpu_omp" and row["n"] == "1":
                key = f"{row['case']}/{row['solver']}/n1"
                steps[key] = dict(steps=int(row["total_steps"]), nx=int(row["nx"]), ny=int(row["ny"]),
                                  source=f"validation/cpu_mpi_fullnode_external_timing_11470.csv:{lineno}")
    snaps = []
    with open(os.path.join(REFERENCE_TREE, "outputs", "baseline", "cpu_stdout.txt")) as f:
        for line in f:
            m = re.search(r"Wrote snapshot (\d+) at t = ([0-9.eE+-]+)", line)
            if m:
                snaps.append(m.group(2))
    return steps, dict(case="shock_bubble", solver="hll", n=1, snapshot_t_6sig=snaps,
                       source="outputs/baseline/cpu_stdout.txt:1-8")


def main():
    R, P = Oracle("reference"), Oracle("port")
    rng = np.random.default_rng(20261203)
    rk = make_riemann(R, rng)
    np.savez_compressed(os.path.join(OUT, "riemann_kat.npz"), **rk)
    st = make_steps(R, P, rng)
    np.savez_compressed(os.path.join(OUT, "step_cases.npz"), **st)
    ru = make_runs(R, P)
    np.savez_compressed(os.path.join(OUT, "run_cases.npz"), **ru)

    info = {}
    g = Grid(256, 256, 0.0, 2.0, 0.0, 2.0)
    U = P.init_blast(g)
    r = R.run(U, g, 0.8, 0.25, "hllc", nsnap=5)
    info["blast256_hllc"] = dict(
        nx=256, ny=256, cfl=0.8, t_end=0.25, steps=int(r["steps"]), t=r["t"].hex(),
        dts=[float(x).hex() for x in r["dts"]],
        snap_step=[int(x) for x in r["snap_step"]], snap_t=[float(x).hex() for x in r["snap_t"]],
        final_sha256=hashlib.sha256(U.tobytes()).hexdigest(),
        final_interior_sums=[float(x).hex() for x in U[2:-2, 2:-2].sum(axis=(0, 1))])
    steps, snaps = parse_reference_logs()
    info["reference_logged_steps"] = steps
    info["reference_logged_snapshots"] = snaps
    with open(os.path.join(OUT, "run_cases.json"), "w") as f:
        json.dump(info, f, indent=1)
    for fn in ("riemann_kat.npz", "step_cases.npz", "run_cases.npz", "run_cases.json"):
        print(fn, os.path.getsize(os.path.join(OUT, fn)))


if __name__ == "__main__":
    main()
