"""The branch-frozen central differences (oracle/shadow_fd.cpp), which the
GPU adjoint is checked against at the adjoint benchmark's size, checked on
the CPU:

  * the unperturbed lane of the multi-lane run is the oracle's own run, bit
    for bit (same arithmetic, same dt sequence);
  * the frozen difference quotients equal the forward-mode (dual-number)
    directional derivative of the same discrete step on the same branches
    (tests/adjoint/adj_check.cpp, file mode, which runs the adjoint's own
    forward arithmetic) to 1e-6 relative -- the two are independent codes
    for one derivative;
  * free +eps / -eps runs would cross limiter kinks: the flip counts are
    positive, which is why the unfrozen differences cannot reach 1e-6.
"""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
if GOLD not in sys.path:
    sys.path.insert(0, GOLD)

import make_frozen_fd as M  # noqa: E402
from oracle import oracle as O  # noqa: E402


@pytest.fixture(scope="module")
def case():
    O.build(reference=False)
    return M.build_case(48, 30)


def test_nominal_lane_is_the_oracle_run(case):
    g, U0, dts, mask, dirs = case
    res = O.frozen_fd(U0, g, dts, "hllc", dirs[:2], 1e-6, mask)
    P = O.Oracle("port")
    V = U0.copy()
    r = P.run(V, g, 0.8, 1e30, "hllc", max_steps=len(dts))
    assert np.array_equal(r["dts"], dts)
    assert np.array_equal(res["U"][2:-2, 2:-2], V[2:-2, 2:-2])


def test_frozen_fd_equals_forward_mode_derivative(case, tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available for the forward-mode reference")
    exe = tmp_path / "adj_check"
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "large_sys_eq_opt_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "adjoint", "adj_check.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    g, U0, dts, mask, dirs = case
    dirs = dirs[:4]
    res = O.frozen_fd(U0, g, dts, "hllc", dirs, 1e-6, mask)
    rho, p = M.blast_fields(g.nx)
    fin, fout = tmp_path / "problem.bin", tmp_path / "result.bin"
    hdr = np.array([g.nx, g.ny, 1, len(dts), 0, 0, 0, 0, len(dirs)], dtype=np.int32)
    with open(fin, "wb") as f:
        f.write(hdr.tobytes())
        f.write(np.array([2.0 / g.nx, 2.0 / g.ny]).tobytes())
        for a in (np.asarray(dts), rho, p, mask.astype(np.float64)):
            f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())
        for d in dirs:
            f.write(np.ascontiguousarray(d.reshape(-1), dtype=np.float64).tobytes())
    r = subprocess.run([str(exe), str(fin), str(fout)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    fm = np.fromfile(fout, dtype=np.float64)[:len(dirs)]
    rel = np.abs(res["fd"] - fm) / np.abs(fm)
    assert rel.max() <= 1e-6, (rel, res["fd"], fm)
    assert np.all(res["flips"] > 0)


def test_portable_directions_are_standard_normal():
    z = M.gaussian(M.SEED, 0, 200000)
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01
    d = M.directions(8, 2)
    assert len(d) == 2 and d[0].shape == (2, 8, 8)
    assert abs(np.linalg.norm(d[1]) - 1.0) < 1e-12
    assert not np.array_equal(d[0], d[1])
