"""Uneven ensembles (eu_batch_*): many grids with their own sizes,
boundaries, parameters, CFL and t_end advanced by one persistent launch per
step.  Each instance must reproduce, bit for bit, the run of its own handle
(same step count, same dt sequence, same final state)."""
import numpy as np
import pytest

from large_sys_eq_opt_gb300.cases import (REFLECTIVE, TRANSMISSIVE, BlastParams, CaseConfig, Problem,
                                          ShockBubbleParams)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E():
    import large_sys_eq_opt_gb300.euler2d as E
    E.load()
    return E


def small_ensemble():
    bub = (TRANSMISSIVE, TRANSMISSIVE, REFLECTIVE, REFLECTIVE)
    return [
        Problem(CaseConfig(64, 64, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.1), "blast", BlastParams(r=0.3, p_in=5.0)),
        Problem(CaseConfig(96, 80, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.08), "blast", BlastParams(r=0.45, p_in=30.0)),
        Problem(CaseConfig(37, 53, 2, 0.0, 2.0, 0.0, 2.0, 0.5, 0.05), "blast", BlastParams(r=0.25, p_in=2.0)),
        Problem(CaseConfig(200, 79, 2, 0.0, 0.225, 0.0, 0.089, 0.8, 0.02), "shock_bubble",
                ShockBubbleParams(mach=1.6, rho_bubble=2.0), bc=bub),
        Problem(CaseConfig(150, 59, 2, 0.0, 0.225, 0.0, 0.089, 0.8, 0.03), "shock_bubble",
                ShockBubbleParams(mach=1.15, rho_bubble=0.2), bc=bub),
        Problem(CaseConfig(1, 40, 2, 0.0, 1.0, 0.0, 2.0, 0.8, 0.05), "blast", BlastParams(cx=0.5, r=0.5)),
    ]


@pytest.mark.parametrize("prec,solver", [("fp32", "hllc"), ("fp64", "hllc"), ("fp32", "exact"),
                                         ("fp32", "force"), ("fp32", "hll"), ("fp64", "hll")])
def test_ensemble_matches_single_runs(E, prec, solver):
    """Every instance of an uneven ensemble equals its own handle's run to
    t_end bit for bit (steps, time and state)."""
    probs = small_ensemble()
    with E.Batch(probs, prec, solver) as b:
        b.start()
        b.run()
        got = [inst.download() for inst in b.instances]
        times = [inst.time() for inst in b.instances]
    for p, g, (t, n, _) in zip(probs, got, times):
        with E.Solver.for_problem(p, prec, solver) as s:
            info = s.run(p.cfg.t_end)
            ref = s.download()
        assert n == info["steps"], p
        assert t == info["t"], p
        assert np.array_equal(g, ref), p


def test_ensemble_autotune_keeps_results(E):
    probs = small_ensemble()
    with E.Batch(probs, "fp32", "hllc") as a, E.Batch(probs, "fp32", "hllc") as b:
        a.start()
        b.start()
        sx, sy = b.autotune(2)
        assert sx % 8 == 0 and sy % 4 == 0
        a.step(25)
        b.step(25)
        for u, v in zip(a.instances, b.instances):
            assert np.array_equal(u.download(), v.download())


def test_ensemble_workload_builds_and_steps(E):
    """The 64-instance benchmark ensemble (48 blasts, 16 shock-bubbles)
    steps, and a few instances match their own handles after 6 steps."""
    from large_sys_eq_opt_gb300.cases import ensemble_problems
    probs = ensemble_problems()
    with E.Batch(probs, "fp32", "hllc") as b:
        b.start()
        done = b.step(6)
        assert not done
        picks = [0, 7, 47, 48, 63]
        got = {i: b.instances[i].download() for i in picks}
    # six CFL steps end far before any instance's t_end, so the unclipped
    # eu_step_n of the instance's own handle is the reference
    for i in picks:
        with E.Solver.for_problem(probs[i], "fp32", "hllc") as s:
            s.step_n(6)
            assert np.array_equal(got[i], s.download()), probs[i].name


def test_batched_parameter_gradients_match_fd(E):
    """dJ/dtheta of every instance of a small mixed batch (FP64) through the
    batched adjoint, against central differences of J(theta +- eps) run on
    the instance's own handle with the same frozen dts."""
    from large_sys_eq_opt_gb300 import adjoint as A
    bub = (TRANSMISSIVE, TRANSMISSIVE, REFLECTIVE, REFLECTIVE)
    probs = [
        Problem(CaseConfig(48, 48, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.25), "blast", BlastParams(r=0.33, p_in=7.0)),
        Problem(CaseConfig(64, 56, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.25), "blast", BlastParams(r=0.45, p_in=40.0)),
        Problem(CaseConfig(120, 48, 2, 0.0, 0.225, 0.0, 0.089, 0.8, 0.1), "shock_bubble",
                ShockBubbleParams(mach=1.5, rho_bubble=2.2), bc=bub),
        Problem(CaseConfig(150, 59, 2, 0.0, 0.225, 0.0, 0.089, 0.8, 0.1), "shock_bubble",
                ShockBubbleParams(mach=1.2, rho_bubble=0.3), bc=bub),
    ]
    Js, grads, dts, _ = A.ensemble_parameter_gradients(E, probs, 60, precision="fp64", solver="hllc", ckpt_k=16)
    from dataclasses import replace
    for p, J, g, d in zip(probs, Js, grads, dts):
        mask = A.objective_mask(p)
        with E.Solver(p.cfg, "fp64", "hllc", bc=p.bc) as s:
            for name, val in g.items():
                theta = getattr(p.params, name)
                eps = 1e-6 * abs(theta)
                J2 = []
                for sgn in (1.0, -1.0):
                    q = replace(p, params=replace(p.params, **{name: theta + sgn * eps}))
                    s.upload(A.initial_state(q)[0])
                    s.step_n(len(d), d)
                    J2.append(A.objective(s.download(), mask))
                fd = (J2[0] - J2[1]) / (2 * eps)
                print(p.name or p.kind, name, "adjoint %.10e fd %.10e" % (val, fd))
                assert abs(val - fd) <= 1e-5 * abs(fd) + 1e-9 * abs(J), (p, name, val, fd)


def test_device_parameter_gradients_equal_host_path(E):
    """eu_batch_param_gradients (initial states, CFL forwards, objective,
    dJ/dU_N and the tangent contractions on the device) against the same
    computation with the dt lists from an ensemble run and the grids
    passing through host arrays (adjoint.py formulas), FP64: the same dt
    lists bit for bit, J and gradients to rounding."""
    from large_sys_eq_opt_gb300 import adjoint as A
    bub = (TRANSMISSIVE, TRANSMISSIVE, REFLECTIVE, REFLECTIVE)
    probs = [
        Problem(CaseConfig(64, 64, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.25), "blast", BlastParams(r=0.37, p_in=12.0)),
        Problem(CaseConfig(140, 55, 2, 0.0, 0.225, 0.0, 0.089, 0.8, 0.1), "shock_bubble",
                ShockBubbleParams(mach=1.7, rho_bubble=0.4), bc=bub),
    ]
    Jd, gd, dtd, _ = A.ensemble_parameter_gradients(E, probs, 40, precision="fp64", solver="hllc", ckpt_k=8)
    Jh, gh, dth, _ = A.ensemble_parameter_gradients(E, probs, 40, precision="fp64", solver="hllc", ckpt_k=8,
                                                    device=False)
    for a, b in zip(dtd, dth):
        assert np.array_equal(a, b)
    for a, b in zip(Jd, Jh):
        assert abs(a - b) <= 1e-12 * abs(b)
    for a, b in zip(gd, gh):
        for k in b:
            assert abs(a[k] - b[k]) <= 1e-9 * abs(b[k]) + 1e-12, (k, a[k], b[k])


@pytest.mark.parametrize("prec,solver", [("fp32", "hllc"), ("fp64", "hllc"), ("fp32", "exact")])
def test_param_gradients_cfl_forward_equals_dt_run(E, prec, solver):
    """eu_batch_param_gradients without dt lists: each instance's forward
    takes the ensemble run's CFL steps -- the first blast reaches its t_end
    after 14 of the 30 steps (the oracle's count), partway through a
    checkpoint segment of 4 and at the end of one of 7; k = 0 keeps all 30
    states (one segment) -- and J and the gradients equal, bit for bit,
    those of the call given the ensemble run's dt lists.  The forwards run
    as shared ensemble launches; the backward reads every state from the
    ring with k = 0 and recomputes earlier segments with each instance's own
    launches with k = 4 and 7, with the same bits."""
    from large_sys_eq_opt_gb300 import adjoint as A
    bub = (TRANSMISSIVE, TRANSMISSIVE, REFLECTIVE, REFLECTIVE)
    probs = [
        Problem(CaseConfig(64, 64, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.05), "blast", BlastParams(r=0.37, p_in=12.0)),
        Problem(CaseConfig(140, 55, 2, 0.0, 0.225, 0.0, 0.089, 0.8, 0.1), "shock_bubble",
                ShockBubbleParams(mach=1.7, rho_bubble=0.4), bc=bub),
        Problem(CaseConfig(96, 80, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.25), "blast", BlastParams(r=0.3, p_in=5.0)),
    ]
    nsteps = 30
    res = {}
    with E.Batch(probs, prec, solver) as b:
        for k in (4, 7, 0):
            Jc, gc, dtc, _ = A.ensemble_parameter_gradients(E, probs, nsteps, prec, solver, ckpt_k=k, batch=b)
            for inst, p in zip(b.instances, probs):
                inst.init_params(p)
                inst.set_dt_log(nsteps)
            b.start()
            b.step(nsteps)
            dts = [inst.dt_log(min(inst.time()[1], nsteps)) for inst in b.instances]
            J, dJ = b.param_gradients(probs, dts, k)
            if k == 0:
                assert [inst.get_option("ckpt_k") for inst in b.instances] == [len(dts[0]), nsteps, nsteps]
            assert len(dts[0]) < nsteps, len(dts[0])
            assert [len(d) for d in dts[1:]] == [nsteps, nsteps]
            for a, d in zip(dtc, dts):
                assert np.array_equal(a, d), k
            assert np.array_equal(np.array(Jc), J), k
            assert np.array_equal(np.array([list(g.values()) for g in gc]), dJ), k
            assert np.all(np.isfinite(dJ))
            res[k] = (J, dJ)
    for k in (4, 7):
        assert np.array_equal(res[k][0], res[0][0]), k
        assert np.array_equal(res[k][1], res[0][1]), k


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_batch_adjoint_forward_matches_single_steps(E, prec):
    """eu_batch_adjoint_forward (the instances' steps as shared ensemble
    launches, checkpoints every 3 steps) lands every instance on the state,
    time and step count of its own handle's eu_step_n with the same dts."""
    probs = small_ensemble()[:5]
    nsteps = [7, 11, 5, 9, 8]
    dts = []
    for p, n in zip(probs, nsteps):
        with E.Solver.for_problem(p, prec, "hllc") as s:
            s.set_dt_log(n)
            s.step_n(n)
            dts.append(s.dt_log(n))
    with E.Batch(probs, prec, "hllc") as b:
        U0 = [inst.download() for inst in b.instances]
        b.adjoint_forward(dts, 3)
        got = [inst.download() for inst in b.instances]
        times = [inst.time() for inst in b.instances]
    for p, u0, d, g, (t, n, _) in zip(probs, U0, dts, got, times):
        with E.Solver.for_problem(p, prec, "hllc") as s:
            s.upload(u0)
            s.step_n(len(d), d)
            ref = s.download()
        assert np.array_equal(g, ref), p
        assert n == len(d)
        assert abs(t - float(np.sum(d))) <= 1e-12, p
