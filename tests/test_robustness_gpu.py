"""Robustness on the GPU: the reference's own logged known answers, canary
values in every unused column and padding (a stand-in for a race/bounds
sanitizer), restart files, the bounded-wait failure path ("a flag that
nothing sets") and out-of-memory by request."""
import math
import os

import numpy as np
import pytest

from large_sys_eq_opt_gb300.cases import BlastParams, CaseConfig, Problem, blast_large, reference_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E():
    import large_sys_eq_opt_gb300.euler2d as E
    E.load()
    return E


# Step counts of the reference CPU solver at n = 1 for each case and solver
# (validation/cpu_mpi_fullnode_external_timing_11470.csv:2-17,
# outputs/cpu_*_n1_timing.txt:16) and the snapshot times of shock_bubble/HLL
# n = 1 as printed by the reference driver (outputs/baseline/cpu_stdout.txt:1-8).
KNOWN_STEPS = {("blast_wave", "hll"): 2306, ("blast_wave", "hllc"): 2335, ("blast_wave", "exact"): 2334,
               ("blast_wave", "force"): 2308, ("shock_bubble", "hll"): 6359, ("shock_bubble", "hllc"): 6913,
               ("shock_bubble", "exact"): 6912, ("shock_bubble", "force"): 6539}
KNOWN_SNAP_T = ["0.000234916", "0.000469817", "0.000704535", "0.000939401", "0.0011741"]


@pytest.mark.parametrize("case,solver", sorted(KNOWN_STEPS))
def test_reference_step_counts(E, case, solver):
    p = reference_problem(case, 1)
    times = {}
    with E.Solver(p.cfg, "fp64", solver) as s:
        s.init_reference_case(case)
        info = s.run(p.cfg.t_end, nsnap=5, callback=lambda k, step, t, U: times.__setitem__(k, t))
    assert info["steps"] == KNOWN_STEPS[(case, solver)]
    if (case, solver) == ("shock_bubble", "hll"):
        assert ["%g" % times[k] for k in range(1, 6)] == KNOWN_SNAP_T


def unused_mask(rows_total, pitch, nx, ny, coff):
    """True where a plane of a buffer holds no cell: columns left of the
    2-column ghost frame and right of it, up to the pitch."""
    m = np.ones((rows_total, pitch), dtype=bool)
    m[: ny + 4, coff - 2: coff + nx + 2] = False
    return m


@pytest.mark.parametrize("prec", ("fp32", "fp64"))
@pytest.mark.parametrize("nx,ny", ((37, 23), (64, 40), (130, 67)))
def test_canaries_in_unused_memory(E, prec, nx, ny):
    """NaN canaries in every unused column of both state buffers and of the
    x-sweep output: 6 steps give the same bits as without them (nothing
    unused reaches an output) and the canaries are still there (nothing
    writes outside the grid and its ghost frame)."""
    prob = Problem(CaseConfig(nx, ny, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.25), "blast", BlastParams(r=0.5))
    with E.Solver.for_problem(prob, prec, "hllc") as ref:
        ref.step_n(6)
        want = ref.download()
    with E.Solver.for_problem(prob, prec, "hllc") as s:
        offs = {0: 6, 1: 6, 2: 8}
        masks = {}
        for which, coff in offs.items():
            planes = s.read_planes(which)
            rows, pitch = planes.shape[1], planes.shape[2]
            full = np.empty(4 * s._plane_len(which), dtype=planes.dtype)
            full[:] = np.nan
            flat = full.reshape(4, -1)
            m = unused_mask(rows, pitch, nx, ny, coff)
            body = planes.copy()
            body[:, m] = np.nan
            flat[:, : rows * pitch] = body.reshape(4, -1)
            s.write_planes(which, full)
            masks[which] = m
        s.step_n(6)
        got = s.download()
        for which, m in masks.items():
            planes = s.read_planes(which)
            assert np.all(np.isnan(planes[:, m])), which
    assert np.array_equal(got, want)


def test_restart_file_round_trip(E, tmp_path):
    prob = blast_large(96)
    path = tmp_path / "state.bin"
    with E.Solver.for_problem(prob, "fp64", "hllc") as a:
        a.step_n(7)
        a.save_state(path)
        t7 = a.time()
        a.step_n(6)
        want = a.download()
        t13 = a.time()
    with E.Solver(prob.cfg, "fp64", "hllc") as b:
        b.load_state(path)
        assert b.time()[:2] == t7[:2]
        b.step_n(6)
        assert np.array_equal(b.download(), want)
        assert b.time()[:2] == t13[:2]
    with E.Solver(CaseConfig(97, 96, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.25), "fp64", "hllc") as c:
        with pytest.raises(E.EulerError):
            c.load_state(path)


def test_bounded_wait_expires_with_status(E):
    """Ensemble y-sweep tasks told to wait for x-sweep tasks that do not
    exist: the 2 s bounded wait expires, the step reports EU_ERR_TIMEOUT, and
    the device keeps working."""
    probs = [blast_large(64), blast_large(48)]
    with E.Batch(probs, "fp32", "hllc") as b:
        b.start()
        b.set_wait_extra(1)
        with pytest.raises(E.EulerError) as ei:
            b.step(1)
        assert ei.value.code == 5
    with E.Solver.for_problem(blast_large(64), "fp32", "hllc") as s:
        s.step_n(5)
        assert np.isfinite(s.download()).all()


def test_out_of_memory_by_request(E):
    """Two FP64 handles that together need more than the free device memory:
    the second fails with EU_ERR_NOMEM and the first keeps working."""
    import torch
    free = torch.cuda.mem_get_info()[0]
    cells = int(0.6 * free / 100)          # ~96 B per cell for three FP64 buffers
    n = int(math.isqrt(cells))
    if n * n > (1 << 31) - 1:
        pytest.skip("device too large for the per-handle cell limit")
    cfg = CaseConfig(n, n, 2, 0.0, 2.0, 0.0, 2.0, 0.8, 0.25)
    with E.Solver(cfg, "fp64", "hll") as a:
        with pytest.raises(E.EulerError) as ei:
            E.Solver(cfg, "fp64", "hll")
        assert ei.value.code == 3
        a._check(a._L.eu_apply_boundary(a._h))
    with E.Solver.for_problem(blast_large(64), "fp32", "hllc") as s:
        s.step_n(3)
