"""The CPU oracle (C restatement) pinned against fixtures produced by the
unmodified reference solver (tests/golden/make_golden.py) and against the
reference's own logged known answers."""
import hashlib
import json
import os
import platform

import numpy as np
import pytest

from oracle.oracle import Grid

SOLVERS = ("hll", "hllc", "exact", "force")
# HLL, HLLC and FORCE use only + - * / sqrt fmin fmax: bit-exact on every
# host.  The exact solver calls libm pow, which may differ in the last bit
# between x86-64 and aarch64 libm builds.
X86 = platform.machine() in ("x86_64", "AMD64")


def same(a, b, solver):
    a = np.asarray(a)
    b = np.asarray(b)
    if solver != "exact" or X86:
        return np.array_equal(a.view(np.int64), b.view(np.int64)) or np.array_equal(a, b, equal_nan=True)
    return np.allclose(a, b, rtol=1e-12, atol=1e-300, equal_nan=True)


def test_riemann_kat(port, golden_dir):
    d = np.load(os.path.join(golden_dir, "riemann_kat.npz"))
    UL, UR, F = d["UL"], d["UR"], d["F"]
    for s, sname in enumerate(SOLVERS):
        for direction in range(2):
            got = np.stack([port.riemann_flux(UL[k], UR[k], direction, s) for k in range(len(UL))])
            assert same(got, F[s, direction], sname), (sname, direction)


def test_step_cases(port, golden_dir):
    d = np.load(os.path.join(golden_dir, "step_cases.npz"))
    names = sorted({k.split("/")[0] for k in d.files})
    assert len(names) == 5
    for name in names:
        geom = d[f"{name}/geom"]
        g = Grid(int(geom[0]), int(geom[1]), *geom[2:])
        U = np.ascontiguousarray(d[f"{name}/U"])
        dt = float(d[f"{name}/dt"][0])
        if name != "near_vacuum":
            assert port.compute_dt(U, g, 0.8) == dt
        for sname in SOLVERS:
            Utmp, Unew = port.advance_second_order(U, g, dt, sname)
            assert same(Utmp, d[f"{name}/{sname}/Utmp"], sname), (name, sname)
            assert same(Unew, d[f"{name}/{sname}/Unew"], sname), (name, sname)
            U1 = port.advance_first_order(U, g, dt, sname)
            assert same(U1, d[f"{name}/{sname}/U1"], sname), (name, sname)


def test_run_cases_blast48(port, golden_dir):
    d = np.load(os.path.join(golden_dir, "run_cases.npz"))
    g = Grid(48, 40, 0.0, 2.0, 0.0, 2.0)
    U0 = port.init_blast(g)
    assert np.array_equal(U0, d["blast48/U0"])
    for sname in SOLVERS:
        U = U0.copy()
        r = port.run(U, g, 0.8, 0.25, sname, nsnap=5)
        assert np.array_equal(r["snap_step"], d[f"blast48/{sname}/snap_step"])
        assert same(r["dts"], d[f"blast48/{sname}/dts"], sname)
        assert same(r["snap_t"], d[f"blast48/{sname}/snap_t"], sname)
        assert same(U, d[f"blast48/{sname}/final"], sname)


def test_blast256_hllc_bitexact(port, golden_dir):
    info = json.load(open(os.path.join(golden_dir, "run_cases.json")))["blast256_hllc"]
    g = Grid(256, 256, 0.0, 2.0, 0.0, 2.0)
    U = port.init_blast(g)
    r = port.run(U, g, info["cfl"], info["t_end"], "hllc", nsnap=5)
    assert r["steps"] == info["steps"]
    assert [float.fromhex(x) for x in info["dts"]] == list(r["dts"])
    assert list(r["snap_step"]) == info["snap_step"]
    assert hashlib.sha256(U.tobytes()).hexdigest() == info["final_sha256"]


@pytest.mark.parametrize("case,solver", [("blast_wave", "hllc"), ("shock_bubble", "hll")])
def test_reference_logged_step_counts(port, golden_dir, case, solver):
    """Known answers logged by the reference itself at n=1
    (validation/cpu_mpi_fullnode_external_timing_11470.csv and
    outputs/baseline/cpu_stdout.txt)."""
    from large_sys_eq_opt_gb300.cases import get_n_case_config
    info = json.load(open(os.path.join(golden_dir, "run_cases.json")))
    kat = info["reference_logged_steps"][f"{case}/{solver}/n1"]
    cfg = get_n_case_config(case, 1)
    assert (cfg.nx, cfg.ny) == (kat["nx"], kat["ny"])
    g = Grid(cfg.nx, cfg.ny, cfg.x_min, cfg.x_max, cfg.y_min, cfg.y_max)
    U = port.init_reference_case(g, 0 if case == "shock_bubble" else 1)
    r = port.run(U, g, cfg.cfl, cfg.t_end, solver, nsnap=5)
    assert r["steps"] == kat["steps"]
    if case == "shock_bubble":
        snaps = info["reference_logged_snapshots"]["snapshot_t_6sig"]
        assert [f"{t:.6g}" for t in r["snap_t"]] == snaps


def test_reflective_wall_keeps_planar_flow(port):
    """Reflective y walls on a y-uniform x shock tube: the flow must stay
    exactly y-uniform with zero y momentum (no reference counterpart)."""
    g = Grid(40, 6, 0.0, 1.0, 0.0, 0.15, bc=("transmissive", "transmissive", "reflective", "reflective"))
    U = g.zeros()
    for i in range(g.nx + 4):
        x = (i - 2 + 0.5) / g.nx
        rho, p = (1.0, 1.0) if x < 0.5 else (0.125, 0.1)
        U[:, i] = [rho, 0.0, 0.0, p / 0.3999999999999999]
    for sname in SOLVERS:
        V = U.copy()
        port.run(V, g, 0.8, 0.1, sname)
        inner = V[2:-2, 2:-2]
        assert np.all(inner[:, :, 2] == 0.0)
        assert np.all(inner == inner[:1]), sname


def test_reflective_mirror_symmetry(port):
    """A blast centred on the lower wall with a reflective bottom equals the
    lower half of the full-domain blast (mirror symmetry)."""
    full = Grid(24, 24, 0.0, 1.0, -0.5, 0.5)
    half = Grid(24, 12, 0.0, 1.0, 0.0, 0.5, bc=("transmissive", "transmissive", "reflective", "transmissive"))
    Uf = port.init_blast(full, cx=0.5, cy=0.0, r=0.2, rho_in=1.0, p_in=2.0, rho_out=0.5, p_out=0.3)
    Uh = port.init_blast(half, cx=0.5, cy=0.0, r=0.2, rho_in=1.0, p_in=2.0, rho_out=0.5, p_out=0.3)
    for sname in ("hll", "hllc", "force"):
        A, B = Uf.copy(), Uh.copy()
        port.run(A, full, 0.8, 0.05, sname)
        port.run(B, half, 0.8, 0.05, sname)
        top_half = A[2 + 12:-2, 2:-2]
        np.testing.assert_allclose(B[2:-2, 2:-2], top_half, rtol=1e-12, atol=1e-12)
