"""Argument validation of the C ABI, exercised without a GPU: every bad
request is rejected with EU_ERR_INVALID (1) before the device is touched,
and the library never throws or exits."""
import ctypes as C

import pytest

from large_sys_eq_opt_gb300 import euler2d as E


@pytest.fixture(scope="module")
def L():
    from large_sys_eq_opt_gb300 import build as B
    B.build()
    return E.load()


def make(L, nx, ny, ng=2, prec=0, solver=1, limiter=0, bc=None, dom=(0.0, 1.0, 0.0, 1.0)):
    c = E.EuCase(nx, ny, ng, dom[0], dom[1], dom[2], dom[3], 0.8, 0.1)
    h = C.c_void_p()
    b = (C.c_int * 4)(*bc) if bc is not None else None
    return L.eu_create(C.byref(c), prec, solver, limiter, b, C.byref(h)), h


@pytest.mark.parametrize("args,msg", [
    (dict(nx=0, ny=8), b"nx and ny"),
    (dict(nx=8, ny=-1), b"nx and ny"),
    (dict(nx=8, ny=8, ng=3), b"ghost width"),
    (dict(nx=8, ny=8, dom=(1.0, 1.0, 0.0, 1.0)), b"empty domain"),
    (dict(nx=8, ny=8, prec=7), b"precision"),
    (dict(nx=8, ny=8, solver=9), b"solver"),
    (dict(nx=8, ny=8, limiter=1), b"minmod"),
    (dict(nx=50000, ny=50000), b"too large"),
    (dict(nx=8, ny=8, bc=(0, 0, 2, 0)), b"boundary kind"),
    (dict(nx=1, ny=8, bc=(1, 0, 0, 0)), b"nx >= 2"),
    (dict(nx=8, ny=1, bc=(0, 0, 0, 1)), b"ny >= 2"),
])
def test_create_rejects_bad_arguments(L, args, msg):
    rc, h = make(L, **args)
    assert rc == 1
    assert not h.value
    assert msg in L.eu_last_error(None)


def test_null_handles_are_rejected(L):
    assert L.eu_advance(None, 0.1) == 1
    assert L.eu_step_n(None, 3, None) == 1
    assert L.eu_totals(None, None) == 1
    assert L.eu_adjoint_forward(None, 1, None, 4) == 1
    n = C.c_longlong()
    assert L.eu_adjoint_dts(None, None, 0, C.byref(n)) == 1
    assert L.eu_batch_adjoint_forward(None, None, None, 0) == 1
    assert L.eu_batch_step(None, 1, None) == 1
    assert L.eu_batch_handle(None, 0) is None
    L.eu_destroy(None)          # no-op
    L.eu_batch_destroy(None)    # no-op


def test_batch_create_validates(L):
    b = C.c_void_p()
    assert L.eu_batch_create(0, None, None, 1, 1, C.byref(b)) == 1
    assert L.eu_batch_create(300, None, None, 1, 1, C.byref(b)) == 1
    assert b"256" in L.eu_batch_last_error(None)


def test_case_helpers_validate(L):
    out = E.EuCase()
    assert L.eu_get_case_config(b"nope", 1, C.byref(out)) == 1
    assert b"Unknown case name" in L.eu_last_error(None)
    assert L.eu_get_case_config(b"blast_wave", 0, C.byref(out)) == 1
    assert L.eu_get_case_config(b"shock_bubble", 2, C.byref(out)) == 0
    assert (out.nx, out.ny) == (1000, 394)   # src/test_cases.cpp:136-137,191-192
