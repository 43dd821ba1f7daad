"""CPU check of the hand-written adjoint's building blocks and of the tiled
line adjoint (the code the GPU kernels run) against central finite
differences in FP64 (tests/adjoint/adj_check.cpp)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_adjoint_vjps_match_finite_differences(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = tmp_path / "adj_check"
    src = os.path.join(ROOT, "tests", "adjoint", "adj_check.cpp")
    inc = os.path.join(ROOT, "large_sys_eq_opt_gb300", "csrc")
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-I" + inc, src, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL CHECKS PASSED" in r.stdout
