"""Parity at the full size of the throughput workload (the 8192^2 blast):
two FP64 steps against the oracle (the oracle finishes them in seconds on
the host cores), and properties that hold at any size and need no long
oracle run -- FP32 against FP64 on the same dt sequence, conservation of the
totals while no wave has reached the boundary, mirror symmetry of the
centred blast, and bit-identical results across repeated runs and launch
shapes."""
import numpy as np
import pytest

from large_sys_eq_opt_gb300.cases import blast_large
from oracle.oracle import Grid

pytestmark = pytest.mark.gpu

N = 8192


@pytest.fixture(scope="module")
def E():
    import large_sys_eq_opt_gb300.euler2d as E
    E.load()
    return E


def rho_l1(a, b):
    return float(np.mean(np.abs(a[2:-2, 2:-2, 0] - b[2:-2, 2:-2, 0])))


def test_fp64_two_steps_match_oracle(E, port):
    """src/cpu/solver_cpu.cpp:287-309 + :400-499 at 8192^2: the same dt (to
    1e-15 relative) and every interior value within 1e-12 relative."""
    g = Grid(N, N, 0.0, 2.0, 0.0, 2.0)
    U = port.init_blast(g)
    with E.Solver.for_problem(blast_large(N), "fp64", "hllc") as s:
        s.upload(U)
        s.set_dt_log(2)
        s.step_n(2)
        dts = s.dt_log(2)
        got = s.download()
    ref = port.run(U, g, 0.8, 0.25, "hllc", max_steps=2)     # U advanced in place
    assert ref["steps"] == 2
    assert np.all(np.abs(dts - ref["dts"]) <= 1e-15 * ref["dts"])
    for f in range(4):
        a, b = got[2:-2, 2:-2, f], U[2:-2, 2:-2, f]
        err = float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))
        assert err <= 1e-12, (f, err)
    assert rho_l1(got, U) <= 1e-14


@pytest.fixture(scope="module")
def fp64_run(E):
    """20 FP64 steps from the device-initialised blast: dt sequence, totals
    before and after, final state."""
    with E.Solver.for_problem(blast_large(N), "fp64", "hllc") as s:
        t0 = s.totals()
        s.set_dt_log(20)
        s.step_n(20)
        dts = s.dt_log(20)
        t1 = s.totals()
        U = s.download()
    return dts, t0, t1, U


def test_fp32_matches_fp64_on_same_dts(E, fp64_run):
    """The FP32 form against FP64 at full size: L1(rho) well inside the 1e-5
    target, every field within 1e-4 absolute."""
    dts, _, _, ref = fp64_run
    with E.Solver.for_problem(blast_large(N), "fp32", "hllc") as s:
        s.step_n(20, dts)
        got = s.download()
    assert rho_l1(got, ref) <= 1e-6
    for f in range(4):
        assert float(np.max(np.abs(got[2:-2, 2:-2, f] - ref[2:-2, 2:-2, f]))) <= 1e-4, f


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-11), ("fp32", 1e-6)])
def test_totals_conserved_before_waves_reach_boundary(E, fp64_run, prec, tol):
    """After 20 steps (t ~ 1e-3) the blast is far from the transmissive
    boundary, so mass and energy are conserved and the net momentum of the
    symmetric blast stays zero, up to rounding (FP64 audit, eu_totals)."""
    dts = fp64_run[0]
    with E.Solver.for_problem(blast_large(N), prec, "hllc") as s:
        t0 = s.totals()
        s.step_n(20, dts)
        t1 = s.totals()
    assert abs(t1[0] - t0[0]) <= tol * t0[0]
    assert abs(t1[3] - t0[3]) <= tol * t0[3]
    assert abs(t1[1]) <= tol * t0[0] and abs(t1[2]) <= tol * t0[0]


def test_fp64_mirror_symmetry(E, fp64_run):
    """The blast centred in [0,2]^2 is symmetric under x -> 2 - x (rho*u
    negated) and y -> 2 - y (rho*v negated); the split step keeps both
    symmetries up to rounding."""
    U = fp64_run[3][2:-2, 2:-2, :]
    mx = U[:, ::-1, :].copy()
    mx[..., 1] *= -1.0
    assert float(np.max(np.abs(U - mx))) <= 1e-10
    my = U[::-1, :, :].copy()
    my[..., 2] *= -1.0
    assert float(np.max(np.abs(U - my))) <= 1e-10


def test_fp32_bits_independent_of_run_and_launch_shape(E):
    """Ten FP32 steps twice with the planner's launch shape and once with
    other segment lengths: identical bits."""
    prob = blast_large(N)
    outs = []
    for seg in (None, None, (64, 32)):
        with E.Solver.for_problem(prob, "fp32", "hllc") as s:
            if seg is not None:
                s.set_option("seg_x", seg[0])
                s.set_option("seg_y", seg[1])
            s.step_n(10)
            outs.append(s.download())
    assert np.array_equal(outs[0], outs[1])
    assert np.array_equal(outs[0], outs[2])
