"""The C-ABI library loads on a CPU-only host and exports every symbol that
include/euler2d.h declares (no compute call is made here)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    from large_sys_eq_opt_gb300 import build as B
    B.build()
    import large_sys_eq_opt_gb300.euler2d as E
    return E.load()


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "euler2d.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(eu_[a-z0-9_]+)\s*\(", src)) - {"eu_snapshot_cb"})


def test_header_declares_the_binding_surface():
    import large_sys_eq_opt_gb300.euler2d as E
    assert set(declared_symbols()) == set(E.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "large_sys_eq_opt_gb300", "libeuler2d.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\s[TW]\s+(eu_\w+)$", out, flags=re.M))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    for s in declared_symbols():
        assert hasattr(lib, s)


def test_abi_version_and_errors_without_gpu(lib):
    import ctypes as C
    import large_sys_eq_opt_gb300.euler2d as E
    assert lib.eu_abi_version() == 1
    c = E.EuCase()
    assert lib.eu_get_case_config(b"blast_wave", 2, C.byref(c)) == 0
    assert (c.nx, c.ny, c.cfl, c.t_end) == (1000, 1000, 0.4, 0.2)
    assert lib.eu_get_case_config(b"nope", 1, C.byref(c)) == 1
    assert b"Unknown case name" in lib.eu_last_error(None)
    assert lib.eu_get_case_config(b"shock_bubble", 0, C.byref(c)) == 1


def test_case_table_matches_python_mirror(lib):
    import large_sys_eq_opt_gb300.euler2d as E
    from large_sys_eq_opt_gb300.cases import get_n_case_config
    for name in ("shock_bubble", "blast_wave"):
        for n in (1, 2, 8):
            assert E.case_config(name, n) == get_n_case_config(name, n)
