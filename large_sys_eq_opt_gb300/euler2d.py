"""Python binding of the C ABI (include/euler2d.h) -- a thin ctypes layer.

The product is libeuler2d.so (hand-written sm_103a kernels + C++ runtime);
this module only marshals arguments.  There is no CPU fallback: loading fails
loudly when the library is missing, and creating a solver fails when no
sm_103a GPU is present.

The surface mirrors the reference's solver API:
    Solver.compute_dt(cfl)                 compute_dt        (src/cpu/solver_cpu.cpp:287-309)
    Solver.advance(dt)                     advance_second_order (src/cpu/solver_cpu.cpp:400-499)
    Solver.advance_host(Uold, dt)          the same on host Grid2D arrays
    Solver.run(t_end, nsnap, callback)     the time loop of scripts/cpu/main_cpu.cpp:206-262
Host grids are float64 numpy arrays of shape (ny+4, nx+4, 4) -- the Grid2D
AoS layout of head/cpu/grid_cpu.hpp:10-89.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .cases import BlastParams, CaseConfig, Problem, ShockBubbleParams

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libeuler2d.so")

FP64, FP32 = 0, 1
SOLVERS = {"hll": 0, "hllc": 1, "exact": 2, "force": 3}
ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "non-physical state",
          5: "device wait timed out", 6: "bad state"}

_dp = C.POINTER(C.c_double)


class EuCase(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("ng", C.c_int),
                ("x_min", C.c_double), ("x_max", C.c_double), ("y_min", C.c_double), ("y_max", C.c_double),
                ("cfl", C.c_double), ("t_end", C.c_double)]


class EuCaseParams(C.Structure):
    """eu_case_params: kind 0 blast (cx, cy, R, rho_in, p_in, rho_out, p_out),
    kind 1 shock-bubble (rho0, p0, mach, shock_x, bub_cx, bub_cy, bub_r, rho_bubble)."""
    _fields_ = [("kind", C.c_int), ("v", C.c_double * 8)]


def case_params(prob: Problem) -> EuCaseParams:
    from .cases import BlastParams
    q = prob.params
    if isinstance(q, BlastParams):
        return EuCaseParams(0, (C.c_double * 8)(q.cx, q.cy, q.r, q.rho_in, q.p_in, q.rho_out, q.p_out, 0.0))
    return EuCaseParams(1, (C.c_double * 8)(q.rho0, q.p0, q.mach, q.shock_x, q.bub_cx, q.bub_cy, q.bub_r,
                                            q.rho_bubble))


class EuRunInfo(C.Structure):
    _fields_ = [("t", C.c_double), ("steps", C.c_longlong), ("status", C.c_int), ("nsnap_written", C.c_int)]


SNAP_CB = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_longlong, C.c_double, _dp, C.c_int, C.c_int)

# Every symbol include/euler2d.h declares (checked by the CPU test suite).
EXPORTS = (
    "eu_create", "eu_destroy", "eu_last_error", "eu_abi_version", "eu_get_case_config",
    "eu_init_reference_case", "eu_init_blast", "eu_init_shock_bubble", "eu_upload_aos",
    "eu_download_aos", "eu_compute_dt", "eu_advance", "eu_step_n", "eu_run", "eu_get_time",
    "eu_totals", "eu_compute_dt_host", "eu_advance_host", "eu_step_host", "eu_time_steps",
    "eu_host_alloc", "eu_host_free", "eu_device_info", "eu_apply_boundary", "eu_set_dt_log",
    "eu_get_dt_log", "eu_set_device", "eu_set_option", "eu_get_option", "eu_read_planes",
    "eu_advance_first_order", "eu_advance_first_order_host", "eu_totals_noalloc",
    "eu_adjoint_forward", "eu_adjoint_backward", "eu_adjoint_timing", "eu_autotune",
    "eu_batch_create", "eu_batch_destroy", "eu_batch_last_error", "eu_batch_handle", "eu_batch_start",
    "eu_batch_step", "eu_batch_run", "eu_batch_time_steps", "eu_batch_autotune",
    "eu_batch_adjoint_forward", "eu_batch_adjoint_backward", "eu_batch_set_wait_extra", "eu_write_planes",
    "eu_save_state", "eu_load_state", "eu_domain_plan", "eu_domain_create", "eu_domain_destroy",
    "eu_domain_last_error", "eu_domain_upload_aos", "eu_domain_download_aos", "eu_domain_step_n",
    "eu_domain_get_time", "eu_init_params", "eu_batch_param_gradients", "eu_adjoint_dts",
)

_lib = None


class EulerError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{ERRORS.get(code, code)}] {msg}")
        self.code = code


def load(path: str = LIB_PATH):
    """Load libeuler2d.so (build it first with large_sys_eq_opt_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} is missing: the CUDA library must be built (python -c 'import __graft_entry__ as g; "
            "g.build()'); there is no CPU fallback")
    L = C.CDLL(path)
    H = C.c_void_p
    L.eu_create.argtypes = [C.POINTER(EuCase), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(H)]
    L.eu_destroy.argtypes = [H]
    L.eu_destroy.restype = None
    L.eu_last_error.argtypes = [H]
    L.eu_last_error.restype = C.c_char_p
    L.eu_abi_version.restype = C.c_int
    L.eu_get_case_config.argtypes = [C.c_char_p, C.c_int, C.POINTER(EuCase)]
    L.eu_init_reference_case.argtypes = [H, C.c_char_p]
    L.eu_init_blast.argtypes = [H] + [C.c_double] * 7
    L.eu_init_shock_bubble.argtypes = [H] + [C.c_double] * 8
    L.eu_upload_aos.argtypes = [H, _dp]
    L.eu_download_aos.argtypes = [H, _dp]
    L.eu_compute_dt.argtypes = [H, C.c_double, _dp]
    L.eu_advance.argtypes = [H, C.c_double]
    L.eu_step_n.argtypes = [H, C.c_longlong, _dp]
    L.eu_run.argtypes = [H, C.c_double, C.c_int, SNAP_CB, C.c_void_p, C.POINTER(EuRunInfo)]
    L.eu_get_time.argtypes = [H, _dp, C.POINTER(C.c_longlong), _dp]
    L.eu_totals.argtypes = [H, _dp]
    L.eu_compute_dt_host.argtypes = [H, _dp, C.c_double, _dp]
    L.eu_advance_host.argtypes = [H, _dp, _dp, _dp, C.c_double]
    L.eu_step_host.argtypes = [H, _dp, _dp, C.c_double, C.c_double, C.c_double, _dp]
    L.eu_time_steps.argtypes = [H, C.c_int, C.c_int, C.POINTER(C.c_float)]
    L.eu_host_alloc.argtypes = [C.c_size_t, C.POINTER(C.c_void_p)]
    L.eu_host_free.argtypes = [C.c_void_p]
    L.eu_host_free.restype = None
    L.eu_device_info.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int)]
    L.eu_apply_boundary.argtypes = [H]
    L.eu_set_dt_log.argtypes = [H, C.c_longlong]
    L.eu_get_dt_log.argtypes = [H, _dp, C.c_longlong]
    L.eu_set_device.argtypes = [C.c_int]
    L.eu_set_option.argtypes = [H, C.c_char_p, C.c_longlong]
    L.eu_get_option.argtypes = [H, C.c_char_p, C.POINTER(C.c_longlong)]
    L.eu_read_planes.argtypes = [H, C.c_int, C.c_void_p, C.c_size_t, C.POINTER(C.c_longlong),
                                 C.POINTER(C.c_longlong)]
    L.eu_advance_first_order.argtypes = [H, C.c_double]
    L.eu_advance_first_order_host.argtypes = [H, _dp, _dp, C.c_double]
    L.eu_totals_noalloc.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    L.eu_adjoint_forward.argtypes = [H, C.c_longlong, _dp, C.c_int]
    L.eu_adjoint_backward.argtypes = [H, _dp, _dp]
    L.eu_adjoint_timing.argtypes = [H, C.POINTER(C.c_float)]
    L.eu_adjoint_dts.argtypes = [H, _dp, C.c_longlong, C.POINTER(C.c_longlong)]
    L.eu_autotune.argtypes = [H, C.c_int, C.POINTER(C.c_longlong)]
    B = C.c_void_p
    L.eu_batch_create.argtypes = [C.c_int, C.POINTER(EuCase), C.POINTER(C.c_int), C.c_int, C.c_int, C.POINTER(B)]
    L.eu_batch_destroy.argtypes = [B]
    L.eu_batch_destroy.restype = None
    L.eu_batch_last_error.argtypes = [B]
    L.eu_batch_last_error.restype = C.c_char_p
    L.eu_batch_handle.argtypes = [B, C.c_int]
    L.eu_batch_handle.restype = C.c_void_p
    L.eu_batch_start.argtypes = [B]
    L.eu_batch_step.argtypes = [B, C.c_longlong, C.POINTER(C.c_int)]
    L.eu_batch_run.argtypes = [B, C.c_longlong, C.POINTER(C.c_longlong)]
    L.eu_batch_time_steps.argtypes = [B, C.c_int, C.POINTER(C.c_float)]
    L.eu_batch_autotune.argtypes = [B, C.c_int, C.POINTER(C.c_longlong)]
    L.eu_batch_adjoint_forward.argtypes = [B, C.POINTER(C.c_longlong), C.POINTER(_dp), C.c_int]
    L.eu_batch_adjoint_backward.argtypes = [B, C.POINTER(_dp), C.POINTER(_dp)]
    L.eu_batch_set_wait_extra.argtypes = [B, C.c_int]
    L.eu_write_planes.argtypes = [H, C.c_int, C.c_void_p, C.c_size_t]
    L.eu_save_state.argtypes = [H, C.c_char_p]
    L.eu_load_state.argtypes = [H, C.c_char_p]
    L.eu_init_params.argtypes = [H, C.POINTER(EuCaseParams)]
    L.eu_batch_param_gradients.argtypes = [B, C.POINTER(EuCaseParams), C.POINTER(C.c_longlong), C.POINTER(_dp),
                                           C.c_int, _dp, _dp]
    D = C.c_void_p
    L.eu_domain_plan.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int)]
    L.eu_domain_create.argtypes = [C.POINTER(EuCase), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int,
                                   C.POINTER(D)]
    L.eu_domain_destroy.argtypes = [D]
    L.eu_domain_destroy.restype = None
    L.eu_domain_last_error.argtypes = [D]
    L.eu_domain_last_error.restype = C.c_char_p
    L.eu_domain_upload_aos.argtypes = [D, _dp]
    L.eu_domain_download_aos.argtypes = [D, _dp]
    L.eu_domain_step_n.argtypes = [D, C.c_longlong, C.c_double]
    L.eu_domain_get_time.argtypes = [D, _dp, C.POINTER(C.c_longlong)]
    _lib = L
    return L


def domain_plan(ny: int, nslabs: int):
    """First interior row of each slab (and ny) of the slab decomposition."""
    L = load()
    out = (C.c_int * (nslabs + 1))()
    rc = L.eu_domain_plan(int(ny), int(nslabs), out)
    if rc:
        raise EulerError(rc, L.eu_last_error(None).decode())
    return [int(x) for x in out]


class Domain:
    """One grid split into slabs of whole rows on the current device, each a
    handle with a 2-row halo exchanged every step (eu_domain_*); results equal
    a single Solver's bit for bit."""

    def __init__(self, cfg: CaseConfig, precision="fp64", solver="hllc", bc=(0, 0, 0, 0), nslabs=2):
        self._L = L = load()
        self.cfg = cfg
        c = EuCase(cfg.nx, cfg.ny, cfg.ng, cfg.x_min, cfg.x_max, cfg.y_min, cfg.y_max, cfg.cfl, cfg.t_end)
        b = (C.c_int * 4)(*bc)
        d = C.c_void_p()
        prec = FP32 if precision in ("fp32", FP32) else FP64
        rc = L.eu_domain_create(C.byref(c), prec, SOLVERS[solver], 0, b, int(nslabs), C.byref(d))
        if rc:
            raise EulerError(rc, L.eu_domain_last_error(None).decode())
        self._d = d

    def _check(self, rc):
        if rc:
            raise EulerError(rc, self._L.eu_domain_last_error(self._d).decode())

    def upload(self, U: np.ndarray):
        U = np.ascontiguousarray(U, dtype=np.float64)
        self._check(self._L.eu_domain_upload_aos(self._d, _p(U)))

    def download(self) -> np.ndarray:
        U = np.zeros((self.cfg.ny + 4, self.cfg.nx + 4, 4))
        self._check(self._L.eu_domain_download_aos(self._d, _p(U)))
        return U

    def step_n(self, n: int, t_end: float = float("inf")):
        self._check(self._L.eu_domain_step_n(self._d, int(n), float(t_end)))

    def time(self):
        t = C.c_double()
        n = C.c_longlong()
        self._check(self._L.eu_domain_get_time(self._d, C.byref(t), C.byref(n)))
        return t.value, n.value

    def close(self):
        if getattr(self, "_d", None):
            self._L.eu_domain_destroy(self._d)
            self._d = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def case_config(name: str, n: int = 1) -> CaseConfig:
    """get_n_case_config through the C ABI (src/test_cases.cpp:184-195)."""
    L = load()
    c = EuCase()
    rc = L.eu_get_case_config(name.encode(), int(n), C.byref(c))
    if rc:
        raise EulerError(rc, L.eu_last_error(None).decode())
    return CaseConfig(c.nx, c.ny, c.ng, c.x_min, c.x_max, c.y_min, c.y_max, c.cfl, c.t_end)


def set_device(device: int):
    L = load()
    rc = L.eu_set_device(int(device))
    if rc:
        raise EulerError(rc, L.eu_last_error(None).decode())


def device_info():
    L = load()
    buf = C.create_string_buffer(256)
    sm = C.c_int(0)
    rc = L.eu_device_info(buf, 256, C.byref(sm))
    if rc:
        raise EulerError(rc, L.eu_last_error(None).decode())
    return buf.value.decode(), sm.value


class PinnedGrid:
    """A Grid2D-shaped float64 array in page-locked host memory."""

    def __init__(self, nx: int, ny: int):
        L = load()
        self.shape = (ny + 4, nx + 4, 4)
        nbytes = 8 * int(np.prod(self.shape))
        self._ptr = C.c_void_p()
        rc = L.eu_host_alloc(nbytes, C.byref(self._ptr))
        if rc:
            raise EulerError(rc, L.eu_last_error(None).decode())
        buf = (C.c_double * (nbytes // 8)).from_address(self._ptr.value)
        self.array = np.frombuffer(buf, dtype=np.float64).reshape(self.shape)

    def __del__(self):
        if getattr(self, "_ptr", None) and self._ptr.value and _lib is not None:
            self.array = None
            _lib.eu_host_free(self._ptr)
            self._ptr = None


class Solver:
    """One device-resident grid (a handle of the C ABI)."""

    def __init__(self, cfg: CaseConfig, precision="fp64", solver="hllc", bc=(0, 0, 0, 0)):
        L = load()
        self.cfg = cfg
        self.precision = precision
        self.solver = solver
        self.bc = tuple(int(b) for b in bc)
        c = EuCase(cfg.nx, cfg.ny, cfg.ng, cfg.x_min, cfg.x_max, cfg.y_min, cfg.y_max, cfg.cfl, cfg.t_end)
        b4 = (C.c_int * 4)(*self.bc)
        h = C.c_void_p()
        prec = FP32 if precision in ("fp32", FP32) else FP64
        s = SOLVERS[solver] if isinstance(solver, str) else int(solver)
        rc = L.eu_create(C.byref(c), prec, s, 0, b4, C.byref(h))
        if rc:
            raise EulerError(rc, L.eu_last_error(None).decode())
        self._h = h
        self._L = L
        self.shape = (cfg.ny + 4, cfg.nx + 4, 4)

    @classmethod
    def _view(cls, L, h, cfg, precision, solver, bc):
        """A non-owning Solver over a handle owned by a Batch."""
        s = cls.__new__(cls)
        s.cfg, s.precision, s.solver, s.bc = cfg, precision, solver, tuple(bc)
        s._h = C.c_void_p(h)
        s._L = L
        s.shape = (cfg.ny + 4, cfg.nx + 4, 4)
        s._owned = False
        return s

    @classmethod
    def for_problem(cls, prob: Problem, precision="fp64", solver="hllc"):
        s = cls(prob.cfg, precision, solver, prob.bc)
        s.init(prob)
        return s

    def close(self):
        if getattr(self, "_h", None):
            if getattr(self, "_owned", True):
                self._L.eu_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc:
            raise EulerError(rc, self._L.eu_last_error(self._h).decode())

    # -- setup --------------------------------------------------------------
    def init(self, prob: Problem):
        p = prob.params
        if isinstance(p, BlastParams):
            self._check(self._L.eu_init_blast(self._h, p.cx, p.cy, p.r, p.rho_in, p.p_in, p.rho_out, p.p_out))
        elif isinstance(p, ShockBubbleParams):
            self._check(self._L.eu_init_shock_bubble(self._h, p.rho0, p.p0, p.mach, p.shock_x, p.bub_cx,
                                                     p.bub_cy, p.bub_r, p.rho_bubble))
        else:
            raise TypeError(type(p))

    def init_reference_case(self, name: str):
        self._check(self._L.eu_init_reference_case(self._h, name.encode()))

    # -- state ---------------------------------------------------------------
    def upload(self, U: np.ndarray):
        U = np.ascontiguousarray(U, dtype=np.float64)
        assert U.shape == self.shape, (U.shape, self.shape)
        self._check(self._L.eu_upload_aos(self._h, _p(U)))

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        out = np.empty(self.shape) if out is None else out
        self._check(self._L.eu_download_aos(self._h, _p(out)))
        return out

    def apply_boundary(self):
        self._check(self._L.eu_apply_boundary(self._h))

    def set_dt_log(self, capacity: int):
        self._check(self._L.eu_set_dt_log(self._h, int(capacity)))

    def dt_log(self, n: int) -> np.ndarray:
        out = np.zeros(int(n))
        self._check(self._L.eu_get_dt_log(self._h, _p(out), int(n)))
        return out

    def set_option(self, name: str, value: int):
        self._check(self._L.eu_set_option(self._h, name.encode(), int(value)))

    def get_option(self, name: str) -> int:
        v = C.c_longlong()
        self._check(self._L.eu_get_option(self._h, name.encode(), C.byref(v)))
        return v.value

    def _plane_len(self, which: int) -> int:
        pitch, plane = C.c_longlong(), C.c_longlong()
        self._check(self._L.eu_read_planes(self._h, int(which), None, 0, C.byref(pitch), C.byref(plane)))
        return plane.value

    def read_planes(self, which: int) -> np.ndarray:
        """Raw device planes (diagnostics): array [4, rows, pitch] of the
        handle's precision; state buffers hold interior (i, j) at [.., j+2, i+6],
        the x-sweep output at [.., j+2, i+8]."""
        pitch, plane = C.c_longlong(), C.c_longlong()
        self._check(self._L.eu_read_planes(self._h, int(which), None, 0, C.byref(pitch), C.byref(plane)))
        dt = np.float32 if self.precision in ("fp32", FP32) else np.float64
        out = np.empty(4 * plane.value, dtype=dt)
        self._check(self._L.eu_read_planes(self._h, int(which), out.ctypes.data_as(C.c_void_p), out.nbytes, None, None))
        rows = self.cfg.ny + 4
        return out.reshape(4, plane.value)[:, :rows * pitch.value].reshape(4, rows, pitch.value)

    def totals(self) -> np.ndarray:
        out = np.zeros(4)
        self._check(self._L.eu_totals(self._h, _p(out)))
        return out

    # -- discrete adjoint ----------------------------------------------------------
    def adjoint_forward(self, dts, ckpt_k: int = 32, nsteps: int | None = None):
        """Run len(dts) frozen-dt steps from the current state, keeping
        checkpoints every ckpt_k steps for adjoint_backward.  dts None:
        nsteps CFL steps (sizes chosen on the device, then held fixed by the
        backward; adjoint_dts() returns them)."""
        if dts is None:
            self._check(self._L.eu_adjoint_forward(self._h, int(nsteps), None, int(ckpt_k)))
            return
        d = np.ascontiguousarray(dts, dtype=np.float64)
        self._check(self._L.eu_adjoint_forward(self._h, len(d), _p(d), int(ckpt_k)))

    def adjoint_dts(self) -> np.ndarray:
        """Step sizes of the last adjoint_forward (given or CFL-chosen)."""
        n = C.c_longlong()
        self._check(self._L.eu_adjoint_dts(self._h, None, 0, C.byref(n)))
        out = np.zeros(n.value)
        self._check(self._L.eu_adjoint_dts(self._h, _p(out), n.value, C.byref(n)))
        return out

    def adjoint_backward(self, dJ_dUN: np.ndarray) -> np.ndarray:
        """dJ/dU_0 for dJ/dU_N (both (ny+4, nx+4, 4) float64; ghosts zero)."""
        g = np.ascontiguousarray(dJ_dUN, dtype=np.float64)
        assert g.shape == self.shape
        out = np.zeros(self.shape)
        self._check(self._L.eu_adjoint_backward(self._h, _p(g), _p(out)))
        return out

    def adjoint_timing(self):
        ms = (C.c_float * 2)()
        self._check(self._L.eu_adjoint_timing(self._h, ms))
        return float(ms[0]), float(ms[1])

    def time(self):
        t = C.c_double()
        n = C.c_longlong()
        dt = C.c_double()
        self._check(self._L.eu_get_time(self._h, C.byref(t), C.byref(n), C.byref(dt)))
        return t.value, n.value, dt.value

    # -- hot path ------------------------------------------------------------
    def compute_dt(self, cfl: float | None = None) -> float:
        dt = C.c_double()
        self._check(self._L.eu_compute_dt(self._h, self.cfg.cfl if cfl is None else cfl, C.byref(dt)))
        return dt.value

    def advance(self, dt: float):
        self._check(self._L.eu_advance(self._h, float(dt)))

    def advance_first_order(self, dt: float):
        self._check(self._L.eu_advance_first_order(self._h, float(dt)))

    def advance_first_order_host(self, Uold: np.ndarray, dt: float) -> np.ndarray:
        Uold = np.ascontiguousarray(Uold, dtype=np.float64)
        Unew = np.empty(self.shape)
        self._check(self._L.eu_advance_first_order_host(self._h, _p(Uold), _p(Unew), float(dt)))
        return Unew

    def step_n(self, n: int, dts=None):
        if dts is None:
            self._check(self._L.eu_step_n(self._h, int(n), None))
        else:
            d = np.ascontiguousarray(dts, dtype=np.float64)
            assert len(d) >= n
            self._check(self._L.eu_step_n(self._h, int(n), _p(d)))

    def run(self, t_end: float | None = None, nsnap: int = 0, callback=None):
        """Device-resident time loop; callback(k, step, t, grid) per snapshot."""
        t_end = self.cfg.t_end if t_end is None else t_end
        info = EuRunInfo()

        def _cb(user, k, step, t, aos, nx, ny):
            arr = np.ctypeslib.as_array(aos, shape=self.shape).copy()
            try:
                return int(bool(callback(k, step, t, arr)))
            except Exception:  # noqa: BLE001 - a raising callback aborts the run
                return 1

        cb = SNAP_CB(_cb) if callback is not None else SNAP_CB()
        self._check(self._L.eu_run(self._h, float(t_end), int(nsnap), cb, None, C.byref(info)))
        return dict(t=info.t, steps=info.steps, status=info.status, snapshots=info.nsnap_written)

    # -- drop-in calls on host grids ----------------------------------------
    def compute_dt_host(self, U: np.ndarray, cfl: float) -> float:
        U = np.ascontiguousarray(U, dtype=np.float64)
        dt = C.c_double()
        self._check(self._L.eu_compute_dt_host(self._h, _p(U), cfl, C.byref(dt)))
        return dt.value

    def advance_host(self, Uold: np.ndarray, dt: float, want_tmp=True):
        Uold = np.ascontiguousarray(Uold, dtype=np.float64)
        Unew = np.empty(self.shape)
        Utmp = np.empty(self.shape) if want_tmp else None
        self._check(self._L.eu_advance_host(self._h, _p(Uold), _p(Utmp) if want_tmp else None, _p(Unew),
                                            float(dt)))
        return Utmp, Unew

    def step_host(self, U: np.ndarray, Unext: np.ndarray, cfl: float, t: float, t_end: float) -> float:
        dt = C.c_double()
        self._check(self._L.eu_step_host(self._h, _p(U), _p(Unext), cfl, t, t_end, C.byref(dt)))
        return dt.value

    # -- measurement ---------------------------------------------------------
    def write_planes(self, which: int, data: np.ndarray):
        a = np.ascontiguousarray(data)
        self._check(self._L.eu_write_planes(self._h, int(which), a.ctypes.data_as(C.c_void_p), a.nbytes))

    def save_state(self, path: str):
        self._check(self._L.eu_save_state(self._h, str(path).encode()))

    def load_state(self, path: str):
        self._check(self._L.eu_load_state(self._h, str(path).encode()))

    def init_params(self, prob: Problem):
        """The differentiable initial state of prob's parameters (eu_init_params)."""
        p = case_params(prob)
        self._check(self._L.eu_init_params(self._h, C.byref(p)))

    def autotune(self, steps: int = 20):
        """Measure and set the fastest segment lengths; returns (seg_x, seg_y)."""
        out = (C.c_longlong * 2)()
        self._check(self._L.eu_autotune(self._h, int(steps), out))
        return int(out[0]), int(out[1])

    def time_steps(self, nsteps: int, use_graph=True):
        ms = (C.c_float * 3)()
        self._check(self._L.eu_time_steps(self._h, int(nsteps), int(bool(use_graph)), ms))
        return float(ms[0]), float(ms[1]), float(ms[2])


class Batch:
    """An uneven ensemble: one grid per Problem (own size, boundaries,
    parameters, CFL, t_end and dt), advanced by one persistent launch per
    step.  ``instances[i]`` is a non-owning Solver view of instance i."""

    def __init__(self, problems, precision="fp32", solver="hllc"):
        L = load()
        n = len(problems)
        cases = (EuCase * n)(*[EuCase(p.cfg.nx, p.cfg.ny, p.cfg.ng, p.cfg.x_min, p.cfg.x_max, p.cfg.y_min,
                                      p.cfg.y_max, p.cfg.cfl, p.cfg.t_end) for p in problems])
        bcs = (C.c_int * (4 * n))(*[int(b) for p in problems for b in p.bc])
        prec = FP32 if precision in ("fp32", FP32) else FP64
        sid = SOLVERS[solver] if isinstance(solver, str) else int(solver)
        b = C.c_void_p()
        rc = L.eu_batch_create(n, cases, bcs, prec, sid, C.byref(b))
        if rc:
            raise EulerError(rc, L.eu_batch_last_error(None).decode())
        self._b, self._L, self.problems = b, L, list(problems)
        self.instances = [Solver._view(L, L.eu_batch_handle(b, i), p.cfg, precision, solver, p.bc)
                          for i, p in enumerate(problems)]
        for inst, p in zip(self.instances, problems):
            inst.init(p)

    def _check(self, rc):
        if rc:
            raise EulerError(rc, self._L.eu_batch_last_error(self._b).decode())

    @property
    def cells(self) -> int:
        return sum(p.cfg.nx * p.cfg.ny for p in self.problems)

    def start(self):
        self._check(self._L.eu_batch_start(self._b))

    def step(self, nsteps: int) -> bool:
        done = C.c_int()
        self._check(self._L.eu_batch_step(self._b, int(nsteps), C.byref(done)))
        return bool(done.value)

    def run(self, max_steps: int = 1 << 40) -> int:
        n = C.c_longlong()
        self._check(self._L.eu_batch_run(self._b, int(max_steps), C.byref(n)))
        return n.value

    def time_steps(self, nsteps: int) -> float:
        ms = C.c_float()
        self._check(self._L.eu_batch_time_steps(self._b, int(nsteps), C.byref(ms)))
        return float(ms.value)

    def set_wait_extra(self, n: int):
        self._check(self._L.eu_batch_set_wait_extra(self._b, int(n)))

    def autotune(self, steps: int = 4):
        out = (C.c_longlong * 2)()
        self._check(self._L.eu_batch_autotune(self._b, int(steps), out))
        return int(out[0]), int(out[1])

    def _dt_lists(self, dts_list, nsteps):
        """(step counts, dt pointer array or None, kept arrays) of the
        batched adjoint calls; dts_list None: nsteps CFL steps each."""
        n = len(self.instances)
        if dts_list is None:
            return (C.c_longlong * n)(*[int(nsteps)] * n), None, []
        arrs = [np.ascontiguousarray(d, dtype=np.float64) for d in dts_list]
        return (C.c_longlong * n)(*[len(a) for a in arrs]), (_dp * n)(*[_p(a) for a in arrs]), arrs

    def adjoint_forward(self, dts_list, ckpt_k: int = 0, nsteps: int | None = None):
        """Checkpointed forward of every instance with its own frozen dts
        (dts_list None: at most nsteps CFL steps each, up to its t_end).
        ckpt_k 0: every state resident when the instances' buffers fit in
        half the free device memory, else checkpoints every sqrt(nsteps)."""
        ns, ptrs, self._keep = self._dt_lists(dts_list, nsteps)
        self._check(self._L.eu_batch_adjoint_forward(self._b, ns, ptrs, int(ckpt_k)))

    def param_gradients(self, problems, dts_list, ckpt_k: int = 0, nsteps: int | None = None):
        """J and the gradients with respect to each instance's two scalar
        parameters, all on the device (eu_batch_param_gradients).  dts_list
        None: at most nsteps CFL steps per instance, up to its t_end, whose
        sizes the instances' adjoint_dts() return afterwards.  Returns
        (J array of n, dJ array of n x 2)."""
        n = len(self.instances)
        params = (EuCaseParams * n)(*[case_params(p) for p in problems])
        ns, pd, dts = self._dt_lists(dts_list, nsteps)
        J = np.zeros(n)
        dJ = np.zeros(2 * n)
        self._check(self._L.eu_batch_param_gradients(self._b, params, ns, pd, int(ckpt_k), _p(J), _p(dJ)))
        return J, dJ.reshape(n, 2)

    def adjoint_backward(self, grads_N):
        """dJ/dU_0 of every instance from its dJ/dU_N (concurrently)."""
        n = len(self.instances)
        ins = [np.ascontiguousarray(g, dtype=np.float64) for g in grads_N]
        outs = [np.zeros(v.shape) for v in self.instances]
        pin = (_dp * n)(*[_p(a) for a in ins])
        pout = (_dp * n)(*[_p(a) for a in outs])
        self._check(self._L.eu_batch_adjoint_backward(self._b, pin, pout))
        return outs

    def close(self):
        if getattr(self, "_b", None):
            for v in self.instances:
                v._h = None
            self._L.eu_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

