"""eu_totals_noalloc (the allocation-free conserved-totals audit) against
eu_totals on a handle holding the same grid.  Collected last, so it runs both
alone and after every other test in the session."""
import ctypes as C

import numpy as np
import pytest

from oracle.oracle import Grid

pytestmark = pytest.mark.gpu

MAX_ROWS = 16384  # the entry point's fixed scratch: 8 doubles per interior row


@pytest.fixture(scope="module")
def E():
    import large_sys_eq_opt_gb300.euler2d as E
    E.load()
    return E


def handle_totals(E, g, U):
    from large_sys_eq_opt_gb300.cases import CaseConfig
    cfg = CaseConfig(g.nx, g.ny, 2, g.x_min, g.x_max, g.y_min, g.y_max, 0.8, 0.25)
    with E.Solver(cfg, "fp64", "hllc") as s:
        s.upload(U)
        return np.array(s.totals())


def mem_free():
    import torch
    return torch.cuda.mem_get_info()[0]


@pytest.mark.parametrize("shape", [(256, 256), (1000, 396), (37, 23), (1, 1), (8192, 300)])
def test_noalloc_totals_match_handle_totals_twice(E, port, shape):
    import torch
    nx, ny = shape
    g = Grid(nx, ny, 0.0, 2.0, 0.0, 2.0)
    U = port.init_blast(g, cx=1.0, cy=0.7, r=0.4)
    U[..., 1] += np.linspace(-0.3, 0.5, U.shape[1])[None, :]   # non-trivial momentum totals
    U[..., 2] -= np.linspace(-0.2, 0.4, U.shape[0])[:, None]
    ref = handle_totals(E, g, U)
    dev = torch.from_numpy(U).cuda()
    out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    L = E.load()
    scale = np.abs(U[2:-2, 2:-2]).sum(axis=(0, 1))
    for call in range(2):
        torch.cuda.synchronize()
        free0 = mem_free()
        rc = L.eu_totals_noalloc(dev.data_ptr(), nx, ny, out.data_ptr(), stream)
        assert rc == 0, L.eu_last_error(None)
        torch.cuda.synchronize()
        if call == 1:
            assert mem_free() == free0  # after the first call's set-up nothing is allocated
        got = out.cpu().numpy()
        # Neumaier sums in a different order: agree to a few ulps of sum|x|
        assert np.all(np.abs(got - ref) <= 1e-14 * scale + 1e-300), (call, got, ref)
        out.fill_(float("nan"))


def test_noalloc_rejects_bad_arguments(E):
    import torch
    L = E.load()
    ny = MAX_ROWS + 1
    dev = torch.zeros((ny + 4) * 5 * 4, dtype=torch.float64, device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    assert L.eu_totals_noalloc(dev.data_ptr(), 1, ny, out.data_ptr(), None) == 1
    assert b"16384" in L.eu_last_error(None)
    assert L.eu_totals_noalloc(dev.data_ptr(), 1, MAX_ROWS, out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    host = np.zeros(4)
    assert L.eu_totals_noalloc(host.ctypes.data_as(C.c_void_p), 1, 4, out.data_ptr(), None) == 1
    assert b"device memory" in L.eu_last_error(None)
    assert L.eu_totals_noalloc(dev.data_ptr() + 8, 1, 4, out.data_ptr(), None) == 1
    assert L.eu_totals_noalloc(None, 1, 4, out.data_ptr(), None) == 1
    assert L.eu_totals_noalloc(dev.data_ptr(), 0, 4, out.data_ptr(), None) == 1
    # d_out given as a host pointer (pinned or pageable) is rejected too
    assert L.eu_totals_noalloc(dev.data_ptr(), 1, 4, host.ctypes.data_as(C.c_void_p), None) == 1
    assert b"device memory" in L.eu_last_error(None)


def test_noalloc_accepts_managed_memory_and_8_byte_aligned_output(E, port):
    """Managed (unified) memory passes the pointer checks, and d_out needs
    only 8-byte alignment: the totals land in the second double of a
    managed buffer, equal to eu_totals on a handle."""
    import torch
    try:
        cu = C.CDLL("libcuda.so.1")
    except OSError:
        pytest.skip("libcuda.so.1 not loadable")
    nx, ny = 64, 40
    g = Grid(nx, ny, 0.0, 2.0, 0.0, 2.0)
    U = port.init_blast(g, cx=1.1, cy=0.9, r=0.5)
    ref = handle_totals(E, g, U)
    torch.cuda.synchronize()        # torch's primary context is current on this thread
    nbytes = U.nbytes + 64
    ptr = C.c_uint64(0)
    assert cu.cuMemAllocManaged(C.byref(ptr), C.c_size_t(nbytes), C.c_uint(1)) == 0   # CU_MEM_ATTACH_GLOBAL
    try:
        base = ptr.value
        out_addr = base + U.nbytes + 8          # 8-byte but not 16-byte aligned
        assert out_addr % 16 == 8
        C.memmove(C.c_void_p(base), U.ctypes.data_as(C.c_void_p), U.nbytes)
        L = E.load()
        assert L.eu_totals_noalloc(base, nx, ny, out_addr, None) == 0, L.eu_last_error(None)
        torch.cuda.synchronize()
        got = np.frombuffer((C.c_double * 4).from_address(out_addr), dtype=np.float64).copy()
        scale = np.abs(U[2:-2, 2:-2]).sum(axis=(0, 1))
        assert np.all(np.abs(got - ref) <= 1e-14 * scale + 1e-300), (got, ref)
    finally:
        torch.cuda.synchronize()
        assert cu.cuMemFree_v2(ptr) == 0
