"""The reference's own CUDA path on this GPU, beside this library's FP64 path.

The reference's GPU solver (src/gpu/solver_gpu.cu) is compiled unmodified
into a device image on the build host (`make -C oracle ref`, which needs the
reference tree) and stepped by oracle/ref_gpu_harness.cu, which replays the
reference's host loop (scripts/gpu/main_gpu.cu:242-266: compute_dt_gpu with
its per-step 8-byte readback, then advance_second_order_gpu).

  * parity: the reference kernels and this library's FP64 path, from the
    same 256^2 blast, agree after 40 HLLC steps (the reference's own CPU/GPU
    agreement is at the 1e-10 level, mse_results/mse_summary_all_cases.csv)
    -- this pins the harness's use of the image;
  * throughput: FP64 HLLC on the 8192^2 blast, the reference's loop against
    this library's graph-replayed FP64 steps (both FP64 arithmetic, same
    state): this library must be faster.  Both numbers are printed.
"""
import numpy as np
import pytest

from oracle import oracle as O
from oracle.oracle import Grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E():
    if not O.reference_gpu_available():
        pytest.skip("the reference's GPU device image was not built (needs the reference tree on the build host)")
    import large_sys_eq_opt_gb300.euler2d as E
    E.load()
    return E


def blast_problem(n):
    from large_sys_eq_opt_gb300.cases import blast_large
    return blast_large(n)


def test_reference_gpu_kernels_agree_with_fp64_path(E, port):
    n, steps = 256, 40
    g = Grid(n, n, 0.0, 2.0, 0.0, 2.0)
    U = port.init_blast(g)
    port.apply_boundary(U, g)
    R = U.copy()
    r = O.reference_gpu_run(R, g, "hllc", 0.8, 0, steps)
    with E.Solver.for_problem(blast_problem(n), "fp64", "hllc") as s:
        s.upload(U)
        s.set_dt_log(steps)
        s.step_n(steps)
        got = s.download()
        dts = s.dt_log(steps)
    np.testing.assert_allclose(r["dts"], dts, rtol=1e-12)
    d = np.abs(R[2:-2, 2:-2, 0] - got[2:-2, 2:-2, 0])
    assert float(d.mean()) <= 1e-10 and float(d.max()) <= 1e-8, (float(d.mean()), float(d.max()))


def test_fp64_path_beats_reference_gpu_kernels(E):
    n = 8192
    prob = blast_problem(n)
    with E.Solver.for_problem(prob, "fp64", "hllc") as s:
        U = s.download()
        s.time_steps(2)
        s.upload(U)
        tot, tx, ty = s.time_steps(10)
    ours = n * n * 10 / (tot / 1e3)
    g = Grid(n, n, 0.0, 2.0, 0.0, 2.0)
    r = O.reference_gpu_run(U, g, "hllc", 0.8, 2, 10)
    ref = n * n * 10 / (r["wall_ms"] / 1e3)
    print(f"FP64 HLLC 8192^2: this library {ours:.3e} cell-updates/s ({tot / 10:.2f} ms/step); "
          f"reference kernels {ref:.3e} ({r['wall_ms'] / 10:.2f} ms/step: dt {r['dt_ms'] / 10:.2f}, "
          f"x {r['x_ms'] / 10:.2f}, y {r['y_ms'] / 10:.2f}); ratio {ours / ref:.2f}")
    assert ours > ref
