"""The y-sweep's row segments against its input boxes (8 rows in FP32, 4 in
FP64, outputs in groups of 4): every segment length gives the same bits,
whether a task's last box is full, half used or the only box, with a grid
height that is not a multiple of the box, reflective and transmissive y
boundaries, and the oracle's state after the same steps."""
import numpy as np
import pytest

from large_sys_eq_opt_gb300.cases import (REFLECTIVE, TRANSMISSIVE, BlastParams, CaseConfig, Problem,
                                          ShockBubbleParams)

pytestmark = pytest.mark.gpu

SEGS = (4, 8, 12, 36, 40, 116, 128)


@pytest.fixture(scope="module")
def E():
    import large_sys_eq_opt_gb300.euler2d as E
    E.load()
    return E


def problems():
    bub = (TRANSMISSIVE, TRANSMISSIVE, REFLECTIVE, REFLECTIVE)
    return [
        Problem(CaseConfig(150, 203, 2, 0.0, 2.0, 0.0, 2.7, 0.8, 1.0), "blast", BlastParams(r=0.4, p_in=20.0),
                name="blast_150x203"),
        Problem(CaseConfig(210, 83, 2, 0.0, 0.225, 0.0, 0.089, 0.8, 1.0), "shock_bubble",
                ShockBubbleParams(mach=1.6, rho_bubble=2.0), bc=bub, name="bubble_210x83"),
    ]


def run(E, prob, prec, solver, seg_y, steps=12):
    with E.Solver.for_problem(prob, prec, solver) as s:
        if seg_y is not None:
            s.set_option("seg_y", seg_y)
        s.set_dt_log(steps)
        s.step_n(steps)
        return s.download(), s.dt_log(steps)


@pytest.mark.parametrize("prec,solver", [("fp32", "hllc"), ("fp32", "hll"), ("fp32", "force"), ("fp32", "exact"),
                                         ("fp64", "hllc")])
def test_segment_lengths_give_the_same_bits(E, prec, solver):
    for prob in problems():
        ref, dts = run(E, prob, prec, solver, None)
        assert np.all(np.isfinite(ref))
        for seg in SEGS:
            got, d = run(E, prob, prec, solver, seg)
            assert np.array_equal(d, dts), (prob.name, seg)
            assert np.array_equal(got, ref), (prob.name, seg)


def test_fp64_matches_oracle_at_every_segment_length(E, port):
    """FP64 HLLC, 6 steps, against the oracle's restatement of the
    reference's loop (the same tolerance as the other FP64 parity tests)."""
    from oracle.oracle import Grid
    prob = problems()[0]
    c = prob.cfg
    g = Grid(c.nx, c.ny, c.x_min, c.x_max, c.y_min, c.y_max)
    U0 = port.init_blast(g, r=prob.params.r, p_in=prob.params.p_in)
    Uo = U0.copy()
    dts_o = port.run(Uo, g, c.cfl, 1.0e9, solver="hllc", max_steps=6)["dts"]
    for seg in (4, 12, 116):
        with E.Solver.for_problem(prob, "fp64", "hllc") as s:
            s.set_option("seg_y", seg)
            s.upload(U0)
            s.set_dt_log(6)
            s.step_n(6)
            got, dts = s.download(), s.dt_log(6)
        np.testing.assert_allclose(dts, dts_o, rtol=1e-13)
        np.testing.assert_allclose(got[2:-2, 2:-2], Uo[2:-2, 2:-2], rtol=1e-10, atol=1e-12)


def test_solver_switch_reencodes_the_y_boxes(E):
    """A handle switched between solvers whose y-sweeps load boxes of other
    heights (FP32 HLLC 8 rows, exact 4) steps, and runs the adjoint's
    checkpointed forward, exactly as fresh handles of each solver given the
    same state (frozen dts)."""
    prob = problems()[0]
    dts = [2.0e-3, 1.5e-3, 1.2e-3]
    with E.Solver.for_problem(prob, "fp32", "hllc") as s:
        U0 = s.download()
        s.step_n(3, dts)
        s.set_option("solver", 2)          # exact
        s.step_n(3, dts)
        s.set_option("solver", 1)          # HLLC
        s.step_n(3, dts)
        got = s.download()
        s.upload(U0)
        s.adjoint_forward(dts, ckpt_k=2)   # builds the forward ring with HLLC's boxes
        s.set_option("solver", 2)
        s.upload(U0)
        s.adjoint_forward(dts, ckpt_k=2)   # reuses the ring with the exact solver's
        got_adj = s.download()
    U = U0
    for solver in ("hllc", "exact", "hllc"):
        with E.Solver.for_problem(prob, "fp32", solver) as r:
            r.upload(U)
            r.step_n(3, dts)
            U = r.download()
    assert np.array_equal(got, U)
    with E.Solver.for_problem(prob, "fp32", "exact") as r:
        r.upload(U0)
        r.adjoint_forward(dts, ckpt_k=2)
        assert np.array_equal(got_adj, r.download())


def test_solver_switch_discards_the_adjoint_forward(E):
    """A backward pass after a solver switch would linearise another
    solver's steps: it is refused until the next forward pass."""
    prob = problems()[0]
    dts = [2.0e-3, 1.5e-3]
    with E.Solver.for_problem(prob, "fp32", "hllc") as s:
        s.adjoint_forward(dts, ckpt_k=2)
        seed = np.zeros_like(s.download())
        seed[2:-2, 2:-2, 0] = 1.0
        s.set_option("solver", 0)          # HLL
        with pytest.raises(E.EulerError):
            s.adjoint_backward(seed)
        s.adjoint_forward(dts, ckpt_k=2)
        g = s.adjoint_backward(seed)
        assert np.all(np.isfinite(g))
