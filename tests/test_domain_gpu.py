"""Slab decomposition of one grid (eu_domain_*): the grid split into slabs of
whole rows with a 2-row halo exchanged between the x- and y-sweeps and one
dt for all slabs (the semantics of the reference's domain decomposition,
src/cpu/solver_mpi.cpp:246-291, :340-443, :547-573) reproduces one handle's
run on the whole grid bit for bit: same interior, same time and step count.
Covers uneven slabs, FP32 and FP64, two solvers, reflective outer walls."""
import numpy as np
import pytest

from oracle.oracle import Grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E():
    import large_sys_eq_opt_gb300.euler2d as E
    E.load()
    return E


CASES = [
    # (grid, bc, precision, solver, slabs, steps)
    ("blast256", (0, 0, 0, 0), "fp64", "hllc", 2, 40),
    ("blast256", (0, 0, 0, 0), "fp32", "hllc", 3, 60),
    ("bubble", (0, 0, 1, 1), "fp64", "exact", 3, 40),
    ("bubble", (0, 0, 1, 1), "fp32", "force", 4, 60),
]


@pytest.mark.parametrize("case,bc,prec,solver,slabs,steps", CASES)
def test_slabs_equal_the_whole_grid(E, port, case, bc, prec, solver, slabs, steps):
    from large_sys_eq_opt_gb300.cases import CaseConfig
    if case == "blast256":
        g = Grid(256, 256, 0.0, 2.0, 0.0, 2.0)
        U = port.init_blast(g)
        t_end = 0.25
    else:
        g = Grid(1000, 396, 0.0, 0.225, 0.0, 0.089, bc=("transmissive", "transmissive", "reflective", "reflective"))
        U = port.init_shock_bubble(g)
        t_end = 0.1
    cfg = CaseConfig(g.nx, g.ny, 2, g.x_min, g.x_max, g.y_min, g.y_max, 0.8, t_end)
    with E.Solver(cfg, prec, solver, bc=bc) as s:
        s.upload(U)
        s.step_n(steps // 2)          # each call starts from a dt of the state, as the domain's
        s.step_n(steps - steps // 2)
        ref = s.download()
        t_ref, n_ref, _ = s.time()
    with E.Domain(cfg, prec, solver, bc=bc, nslabs=slabs) as d:
        d.upload(U)
        d.step_n(steps // 2)
        d.step_n(steps - steps // 2)
        got = d.download()
        t, n = d.time()
    assert n == n_ref and t == t_ref
    assert np.array_equal(got[2:-2, 2:-2], ref[2:-2, 2:-2])


def test_slabs_run_to_t_end(E, port):
    """A run clipped at t_end stops every slab at the same step as the whole grid."""
    from large_sys_eq_opt_gb300.cases import CaseConfig
    g = Grid(128, 96, 0.0, 2.0, 0.0, 1.5)
    U = port.init_blast(g, cx=1.0, cy=0.75, r=0.3)
    cfg = CaseConfig(g.nx, g.ny, 2, g.x_min, g.x_max, g.y_min, g.y_max, 0.8, 0.05)
    with E.Solver(cfg, "fp64", "hll") as s:
        s.upload(U)
        info = s.run(0.05)
        ref = s.download()
    with E.Domain(cfg, "fp64", "hll", nslabs=2) as d:
        d.upload(U)
        d.step_n(10 ** 6, 0.05)
        got = d.download()
        t, n = d.time()
    assert n == info["steps"] and t == info["t"]
    assert np.array_equal(got[2:-2, 2:-2], ref[2:-2, 2:-2])
