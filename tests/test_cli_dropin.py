"""The two drop-in surfaces above the C ABI:

* the C++ command-line driver (large_sys_eq_opt_gb300/bin/euler2d_gb300),
  which takes the reference driver's arguments (scripts/cpu/main_cpu.cpp:67-113)
  and writes its CSV snapshots (scripts/cpu/main_cpu.cpp:136-164);
* the C++ shim (large_sys_eq_opt_gb300/shim/solver_cpu_gb300.cpp) that
  replaces src/cpu/solver_cpu.cpp under the reference's unmodified driver.
"""
import os
import subprocess

import numpy as np
import pytest

from oracle.oracle import REFERENCE_TREE, Grid

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "large_sys_eq_opt_gb300")


@pytest.fixture(scope="module")
def cli():
    from large_sys_eq_opt_gb300 import build as B
    B.build()
    return B.CLI


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_cli_rejects_bad_arguments(cli):
    r = subprocess.run([cli, "--solver", "roe"], capture_output=True, text=True)
    assert r.returncode == 1
    assert "Unknown Riemann solver: roe" in r.stderr
    r = subprocess.run([cli, "0"], capture_output=True, text=True)
    assert r.returncode == 1 and "resolution_scale must be positive" in r.stderr
    r = subprocess.run([cli, "--case", "nope"], capture_output=True, text=True)
    assert r.returncode == 1 and "Unknown case name" in r.stderr
    r = subprocess.run([cli, "--bogus"], capture_output=True, text=True)
    assert r.returncode == 1 and "Unknown argument: --bogus" in r.stderr


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU failure path")
def test_cli_fails_loudly_without_gpu(cli):
    r = subprocess.run([cli, "--timing-only"], capture_output=True, text=True)
    assert r.returncode == 1
    assert "no CUDA device" in r.stderr


@pytest.mark.skipif(not os.path.isdir(REFERENCE_TREE), reason="reference sources not present")
def test_shim_links_with_unmodified_reference_driver(cli):
    """main_cpu.cpp + test_cases.cpp + init.cpp from the reference, linked
    against the shim in place of solver_cpu.cpp: every solver symbol resolves
    with the reference's own signatures."""
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    exe = os.path.join(ROOT, "oracle", "_ref", "main_cpu_gb300")
    assert os.access(exe, os.X_OK)
    if not has_gpu():
        r = subprocess.run([exe, "--timing-only"], capture_output=True, text=True)
        assert r.returncode != 0
        assert "no CUDA device" in r.stderr


def read_snapshot(path):
    a = np.loadtxt(path, delimiter=",", skiprows=1)
    with open(path) as f:
        assert f.readline().strip() == "i,j,x,y,rho,rhou,rhov,E"
    return a


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ("hll", "hllc"))
def test_cli_snapshots_match_oracle(cli, port, tmp_path, solver):
    """The reference's own shock-bubble case at scale 1 (500x197, CFL 0.4) to
    t_end with 5 snapshots: snapshot times, steps and every CSV value agree
    with the oracle run to the 6 significant digits the CSV carries."""
    r = subprocess.run([cli, "1", "--case", "shock_bubble", "--solver", solver, "--output", "--outdir",
                        str(tmp_path), "--prefix", "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    import large_sys_eq_opt_gb300.euler2d as E
    cfg = E.case_config("shock_bubble", 1)
    g = Grid(cfg.nx, cfg.ny, cfg.x_min, cfg.x_max, cfg.y_min, cfg.y_max)
    U = port.init_reference_case(g, 0)
    ref = port.run(U, g, cfg.cfl, cfg.t_end, solver, nsnap=5, want_snapshots=True)
    assert f"Total steps = {ref['steps']}" in r.stdout
    for k in range(1, 6):
        path = tmp_path / f"gpu_shock_bubble_{solver}_n1_snapshot_{k}.csv"
        a = read_snapshot(path)
        assert a.shape == (cfg.nx * cfg.ny, 8)
        i = a[:, 0].astype(int)
        j = a[:, 1].astype(int)
        assert i.min() == 2 and i.max() == cfg.nx + 1 and j.min() == 2 and j.max() == cfg.ny + 1
        Sref = ref["snapshots"][k - 1][j, i]
        for q in range(4):
            np.testing.assert_allclose(a[:, 4 + q], Sref[:, q], rtol=1e-5, atol=1e-9)
