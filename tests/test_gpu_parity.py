"""FP64 CUDA path vs the CPU oracle (restatement of the reference solver) on
the same inputs, through the C ABI.  Tolerances: the spec bar for the
FP64 drop-in is <= 1e-10 L1 (mean absolute difference over interior cells)
in density at t_end; single steps are held to 1e-12 relative."""
import os

import numpy as np
import pytest

from oracle.oracle import Grid, Oracle

pytestmark = pytest.mark.gpu
SOLVERS = ("hll", "hllc", "exact", "force")


@pytest.fixture(scope="module")
def E():
    import large_sys_eq_opt_gb300.euler2d as E
    E.load()
    return E


def interior(U):
    return U[2:-2, 2:-2]


def l1(a, b):
    return float(np.mean(np.abs(a - b)))


def cfg_of(g: Grid, cfl=0.8, t_end=0.25):
    from large_sys_eq_opt_gb300.cases import CaseConfig
    return CaseConfig(g.nx, g.ny, 2, g.x_min, g.x_max, g.y_min, g.y_max, cfl, t_end)


def bc_of(g: Grid):
    return tuple(0 if b in ("transmissive", 0) else 1 for b in g.bc)


def test_device_initial_states_match_oracle(E, port):
    g = Grid(256, 256, 0.0, 2.0, 0.0, 2.0)
    with E.Solver(cfg_of(g), "fp64", "hllc") as s:
        s._check(s._L.eu_init_blast(s._h, 1.0, 1.0, 0.4, 1.0, 1.0, 0.125, 0.1))
        got = s.download()
    assert np.array_equal(interior(got), interior(port.init_blast(g)))
    g = Grid(1000, 396, 0.0, 0.225, 0.0, 0.089)
    with E.Solver(cfg_of(g), "fp64", "hllc") as s:
        s._check(s._L.eu_init_shock_bubble(s._h, 1.0, 1.0, 1.22, 0.005, 0.035, 0.0445, 0.025, 0.138))
        got = s.download()
    assert np.array_equal(interior(got), interior(port.init_shock_bubble(g)))


def test_upload_download_roundtrip(E, port):
    g = Grid(37, 23, 0.0, 1.0, 0.0, 1.0)
    U = port.init_blast(g, cx=0.5, cy=0.5, r=0.2)
    port.apply_boundary(U, g)
    with E.Solver(cfg_of(g), "fp64", "hll") as s:
        s.upload(U)
        assert np.array_equal(s.download(), U)


def test_compute_dt_matches_oracle(E, port):
    g = Grid(256, 256, 0.0, 2.0, 0.0, 2.0)
    U = port.init_blast(g)
    with E.Solver(cfg_of(g), "fp64", "hllc") as s:
        s.upload(U)
        dt = s.compute_dt(0.8)
    ref = port.compute_dt(U, g, 0.8)
    assert abs(dt - ref) <= 1e-15 * ref


@pytest.mark.parametrize("solver", SOLVERS)
def test_single_step_golden_cases(E, golden_dir, solver):
    d = np.load(os.path.join(golden_dir, "step_cases.npz"))
    names = sorted({k.split("/")[0] for k in d.files})
    for name in names:
        geom = d[f"{name}/geom"]
        g = Grid(int(geom[0]), int(geom[1]), *geom[2:])
        U = np.ascontiguousarray(d[f"{name}/U"])
        dt = float(d[f"{name}/dt"][0])
        with E.Solver(cfg_of(g), "fp64", solver) as s:
            Utmp, Unew = s.advance_host(U, dt)
            U1 = s.advance_first_order_host(U, dt)
        for lbl, got, ref in (("Utmp", Utmp, d[f"{name}/{solver}/Utmp"]), ("Unew", Unew, d[f"{name}/{solver}/Unew"]),
                              ("U1", U1, d[f"{name}/{solver}/U1"])):
            scale = np.maximum(np.abs(ref), 1.0)
            err = float(np.max(np.abs(got - ref) / scale))
            assert err <= 1e-12, (name, solver, lbl, err)


@pytest.mark.parametrize("solver", SOLVERS)
def test_blast256_run_to_t_end(E, port, solver):
    """The reference's 256^2 blast case: CFL 0.8, t_end 0.25, 5 snapshots."""
    g = Grid(256, 256, 0.0, 2.0, 0.0, 2.0)
    U = port.init_blast(g)
    ref = port.run(U, g, 0.8, 0.25, solver, nsnap=5, want_snapshots=True)
    snaps = {}
    with E.Solver(cfg_of(g), "fp64", solver) as s:
        s._check(s._L.eu_init_blast(s._h, 1.0, 1.0, 0.4, 1.0, 1.0, 0.125, 0.1))
        info = s.run(0.25, nsnap=5, callback=lambda k, step, t, A: snaps.__setitem__(k, (step, t, A)))
        got = s.download()
    assert info["steps"] == ref["steps"]
    assert abs(info["t"] - ref["t"]) <= 1e-15
    assert sorted(snaps) == [1, 2, 3, 4, 5]
    for k in range(5):
        step, t, A = snaps[k + 1]
        assert step == ref["snap_step"][k]
        assert abs(t - ref["snap_t"][k]) <= 1e-14
        assert l1(interior(A)[..., 0], interior(ref["snapshots"][k])[..., 0]) <= 1e-10
    assert l1(interior(got)[..., 0], interior(U)[..., 0]) <= 1e-10


@pytest.mark.parametrize("solver", SOLVERS)
def test_reflective_shock_bubble_to_t_end(E, port, solver):
    """The 1000x396 single-gas shock-bubble (Mach 1.22 shock, bubble rho 0.138,
    transmissive in x, reflective in y, CFL 0.8) run to t_end = 0.1 with each
    Riemann solver: the FP64 path against the oracle (equal step count and
    snapshot steps, L1(rho) <= 1e-10 at t_end, the other fields reported and
    held to 1e-9), and the FP32 form on the FP64 dt sequence (L1(rho) <= 1e-5
    against the FP64 oracle, the FP32 form's bar)."""
    g = Grid(1000, 396, 0.0, 0.225, 0.0, 0.089, bc=("transmissive", "transmissive", "reflective", "reflective"))
    U = port.init_shock_bubble(g)
    ref = port.run(U, g, 0.8, 0.1, solver, nsnap=5, want_snapshots=False)
    snaps = {}
    with E.Solver(cfg_of(g, 0.8, 0.1), "fp64", solver, bc=bc_of(g)) as s:
        s._check(s._L.eu_init_shock_bubble(s._h, 1.0, 1.0, 1.22, 0.005, 0.035, 0.0445, 0.025, 0.138))
        s.set_dt_log(1 << 14)
        info = s.run(0.1, nsnap=5, callback=lambda k, step, t, A: snaps.__setitem__(k, (step, t)))
        got = s.download()
        dts = s.dt_log(info["steps"])
    assert info["steps"] == ref["steps"]
    assert abs(info["t"] - ref["t"]) <= 1e-15
    for k in range(5):
        assert snaps[k + 1][0] == ref["snap_step"][k]
        assert abs(snaps[k + 1][1] - ref["snap_t"][k]) <= 1e-14
    errs = [l1(interior(got)[..., f], interior(U)[..., f]) for f in range(4)]
    assert errs[0] <= 1e-10, (solver, errs)
    assert max(errs) <= 1e-9, (solver, errs)
    with E.Solver(cfg_of(g, 0.8, 0.1), "fp32", solver, bc=bc_of(g)) as s:
        s._check(s._L.eu_init_shock_bubble(s._h, 1.0, 1.0, 1.22, 0.005, 0.035, 0.0445, 0.025, 0.138))
        s.step_n(len(dts), dts)
        got32 = s.download()
    e32 = l1(interior(got32)[..., 0], interior(U)[..., 0])
    assert e32 <= 1e-5, (solver, e32)
    print(f"shock-bubble {solver}: {ref['steps']} steps, FP64 L1 per field {errs}, FP32 L1(rho) {e32:.3e}")


@pytest.mark.parametrize("shape", [(17, 13), (1, 24), (24, 1), (130, 5), (5, 131), (1, 1), (2, 2), (3, 1)])
def test_odd_sizes_multi_step(E, port, shape):
    nx, ny = shape
    g = Grid(nx, ny, 0.0, 1.0, 0.0, 1.0)
    U = port.init_blast(g, cx=0.3, cy=0.6, r=0.25, rho_in=1.0, p_in=2.0, rho_out=0.3, p_out=0.2)
    V = U.copy()
    ref = port.run(V, g, 0.8, 0.1, "hllc", max_steps=12)
    full = U.copy()
    rfull = port.run(full, g, 0.8, 0.1, "hllc")
    with E.Solver(cfg_of(g, 0.8, 0.1), "fp64", "hllc") as s:
        s.upload(U)                      # formula ghosts: the run applies the BC first
        info = s.run(0.1)
        assert info["steps"] == rfull["steps"]
        got = s.download()
    err = float(np.max(np.abs(interior(got) - interior(full)) / np.maximum(np.abs(interior(full)), 1.0)))
    assert err <= 1e-10, (shape, err)
    W = U.copy()
    port.apply_boundary(W, g)            # the loop body applies the BC before advancing
    with E.Solver(cfg_of(g, 0.8, 0.1), "fp64", "hllc") as s:
        s.upload(W)
        for dt in ref["dts"]:
            s.advance(dt)
        got = s.download()
    err = float(np.max(np.abs(interior(got) - interior(V)) / np.maximum(np.abs(interior(V)), 1.0)))
    assert err <= 1e-11, (shape, err)


def test_fp32_blast256_error_vs_fp64(E, port):
    g = Grid(256, 256, 0.0, 2.0, 0.0, 2.0)
    U = port.init_blast(g)
    port.run(U, g, 0.8, 0.25, "hllc")
    with E.Solver(cfg_of(g), "fp32", "hllc") as s:
        s._check(s._L.eu_init_blast(s._h, 1.0, 1.0, 0.4, 1.0, 1.0, 0.125, 0.1))
        s.run(0.25)
        got = s.download()
    e = l1(interior(got)[..., 0], interior(U)[..., 0])
    print(f"FP32 HLLC blast256 L1(rho) vs FP64 oracle = {e:.3e}")
    assert e <= 1e-5


def test_graph_steps_match_single_steps(E, port):
    g = Grid(200, 150, 0.0, 2.0, 0.0, 1.5)
    from large_sys_eq_opt_gb300.cases import CaseConfig
    with E.Solver(cfg_of(g), "fp64", "hllc") as a, E.Solver(cfg_of(g), "fp64", "hllc") as b:
        for s in (a, b):
            s._check(s._L.eu_init_blast(s._h, 1.0, 0.75, 0.3, 1.0, 1.0, 0.125, 0.1))
        dts = []
        for _ in range(9):
            dt = a.compute_dt(0.8)
            a.advance(dt)
            dts.append(dt)
        b.step_n(9, dts)
        assert np.array_equal(a.download(), b.download())
        b.step_n(5)
        t, n, _ = b.time()
        assert n == 14


def test_nonphysical_state_is_reported(E):
    g = Grid(32, 32)
    with E.Solver(cfg_of(g), "fp64", "hllc") as s:
        s.upload(np.zeros((36, 36, 4)))
        with pytest.raises(E.EulerError) as ei:
            s.compute_dt(0.8)
        assert ei.value.code == 4


@pytest.mark.parametrize("prec", ("fp32", "fp64"))
@pytest.mark.parametrize("nx", (37, 256, 257, 258, 259))
def test_device_ghost_lines_after_a_step(E, prec, nx):
    """After one device step the y-sweep must leave the x-ghost columns of the
    new state equal to the boundary rule applied to its interior (the next
    x-sweep reads them), and the x-sweep must leave Utmp's y-ghost rows equal
    to the rule applied to its interior (the y-sweep reads them)."""
    from large_sys_eq_opt_gb300.cases import CaseConfig
    ny = 45
    for bc in ((0, 0, 0, 0), (1, 1, 1, 1)):
        cfg = CaseConfig(nx, ny, 2, 0.0, 1.0, 0.0, 1.0, 0.8, 0.25)
        with E.Solver(cfg, prec, "hllc", bc=bc) as s:
            s._check(s._L.eu_init_blast(s._h, 0.3, 0.4, 0.2, 1.0, 2.0, 0.2, 0.3))
            s.apply_boundary()
            s.advance(s.compute_dt(0.8))
            S = s.read_planes(1)
            rows = slice(2, ny + 2)
            i0, iN = 6, nx + 5                     # S columns of interior 0 and nx-1
            for g, src in ((5, i0), (4, i0 if bc[0] == 0 else i0 + 1)):
                sign = np.array([1, -1 if bc[0] else 1, 1, 1])[:, None]
                assert np.array_equal(S[:, rows, g], sign * S[:, rows, src]), (prec, nx, bc, g)
            for g, src in ((nx + 6, iN), (nx + 7, iN if bc[1] == 0 else iN - 1)):
                sign = np.array([1, -1 if bc[1] else 1, 1, 1])[:, None]
                assert np.array_equal(S[:, rows, g], sign * S[:, rows, src]), (prec, nx, bc, g)
            Tm = s.read_planes(2)
            cols = slice(8, nx + 8)
            for r, src in ((1, 2), (0, 2 if bc[2] == 0 else 3)):
                sign = np.array([1, 1, -1 if bc[2] else 1, 1])[:, None]
                assert np.array_equal(Tm[:, r, cols], sign * Tm[:, src, cols]), (prec, nx, bc, r)
            for r, src in ((ny + 2, ny + 1), (ny + 3, ny + 1 if bc[3] == 0 else ny)):
                sign = np.array([1, 1, -1 if bc[3] else 1, 1])[:, None]
                assert np.array_equal(Tm[:, r, cols], sign * Tm[:, src, cols]), (prec, nx, bc, r)


@pytest.mark.parametrize("nx,ny", ((257, 131), (130, 67)))
def test_fp32_device_run_tracks_fp64_oracle(E, port, nx, ny):
    """FP32 device-resident run (fused dt, graphs, ghost lines written by the
    sweeps) against the FP64 oracle on odd sizes."""
    g = Grid(nx, ny, 0.0, 2.0, 0.0, 1.0)
    U = port.init_blast(g, cx=1.0, cy=0.5, r=0.3)
    port.run(U, g, 0.8, 0.1, "hllc")
    with E.Solver(cfg_of(g, 0.8, 0.1), "fp32", "hllc") as s:
        s._check(s._L.eu_init_blast(s._h, 1.0, 0.5, 0.3, 1.0, 1.0, 0.125, 0.1))
        info = s.run(0.1)
        got = s.download()
    assert info["status"] == 0
    e = l1(interior(got)[..., 0], interior(U)[..., 0])
    assert e <= 1e-5, e


@pytest.mark.parametrize("prec", ("fp32", "fp64"))
def test_autotune_keeps_state_and_results(E, prec):
    """The autotuner restores state and time, picks legal shapes, and the
    steps it makes faster give the same bits (every cell's arithmetic is
    independent of where the line segments start)."""
    from large_sys_eq_opt_gb300.cases import blast_large
    prob = blast_large(300)
    with E.Solver.for_problem(prob, prec, "hllc") as a, E.Solver.for_problem(prob, prec, "hllc") as b:
        before = b.download()
        t0 = b.time()
        sx, sy = b.autotune(4)
        assert np.array_equal(b.download(), before)
        assert b.time() == t0
        cx = 8 if prec == "fp32" else 4
        assert sx % cx == 0 and sy % 4 == 0
        assert (b.get_option("seg_x"), b.get_option("seg_y")) == (sx, sy)
        a.step_n(12)
        b.step_n(12)
        assert np.array_equal(a.download(), b.download())


def test_run_with_zero_t_end_takes_no_step(E, port):
    g = Grid(40, 30, 0.0, 2.0, 0.0, 2.0)
    U = port.init_blast(g)
    with E.Solver(cfg_of(g), "fp64", "hllc") as s:
        s.upload(U)
        before = s.download()
        info = s.run(0.0)
        assert info["steps"] == 0 and info["t"] == 0.0
        assert np.array_equal(s.download(), before)


@pytest.mark.parametrize("nsnap", (1, 3, 16))
def test_snapshot_schedule_counts(E, port, nsnap):
    """Snapshots at the first step with t >= t_end k / nsnap
    (scripts/cpu/main_cpu.cpp:208-215,244-261) for 1, 3 and the maximum 16.
    The schedule's last time is computed as t_end * k / nsnap, which can
    round above t_end (0.2 * 3 / 3 = 0.20000000000000004): the reference loop
    then never writes that snapshot, and neither does the device loop."""
    g = Grid(64, 48, 0.0, 2.0, 0.0, 2.0)
    U = port.init_blast(g)
    ref = port.run(U.copy(), g, 0.8, 0.2, "hllc", nsnap=nsnap, want_snapshots=True)
    got = {}
    with E.Solver(cfg_of(g, 0.8, 0.2), "fp64", "hllc") as s:
        s.upload(U)
        info = s.run(0.2, nsnap=nsnap, callback=lambda k, step, t, A: got.__setitem__(k, (step, t, A)))
    reached = [k for k in range(1, nsnap + 1) if info["t"] >= 0.2 * k / nsnap]
    assert info["t"] == ref["t"]
    assert sorted(got) == reached
    if nsnap == 3:
        assert reached == [1, 2]
    for k in range(len(reached)):
        step, t, A = got[k + 1]
        assert step == ref["snap_step"][k]
        assert abs(t - ref["snap_t"][k]) <= 1e-14
        assert l1(interior(A)[..., 0], interior(ref["snapshots"][k])[..., 0]) <= 1e-10


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("fp32", 1e-5)])
@pytest.mark.parametrize("solver", SOLVERS)
def test_uniform_flow_stays_uniform(E, port, solver, prec, tol):
    """A uniform moving state with transmissive boundaries is a steady
    solution: every face solves the same Riemann problem (for the exact
    solver the identical-states route), so the flux differences vanish and
    ten steps change no cell beyond the rounding of the update (carried as
    U + lam F_left - lam F_right).  The oracle agrees; dt is the CFL step of
    the uniform state."""
    g = Grid(64, 48, 0.0, 2.0, 0.0, 1.5)
    U = g.zeros()
    r, u, v, p = 1.3, 0.7, -0.4, 2.1
    U[...] = (r, r * u, r * v, p / 0.3999999999999999 + 0.5 * r * (u * u + v * v))
    ref = U.copy()
    out = port.run(ref, g, 0.8, 1.0, solver, max_steps=10)
    with E.Solver(cfg_of(g, 0.8, 1.0), prec, solver) as s:
        s.upload(U)
        s.set_dt_log(10)
        s.step_n(10)
        got = s.download()
        dts = s.dt_log(10)
    assert np.all(np.abs(interior(got) - interior(U)) <= tol * np.maximum(np.abs(interior(U)), 1.0))
    assert np.all(np.abs(interior(ref) - interior(U)) <= 1e-13 * np.maximum(np.abs(interior(U)), 1.0))
    assert np.allclose(dts, out["dts"], rtol=1e-6 if prec == "fp32" else 1e-14, atol=0)
