"""ctypes loader for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module: it is the checker for the CUDA path, never part of it.

Two libraries are exposed with the same Python surface:
  * ``Oracle("port")``      -- oracle/euler2d_oracle.c, the C restatement of
                               the reference CPU solver (builds anywhere);
  * ``Oracle("reference")`` -- oracle/_ref/libref_euler2d.so, the unmodified
                               reference sources behind ref_harness.cpp
                               (only where the reference tree was present at
                               build time; transmissive boundaries only).
Grids are numpy float64 arrays of shape (ny+4, nx+4, 4): the Grid2D AoS
layout of head/cpu/grid_cpu.hpp:10-89.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle_euler2d.so")
REF_SO = os.path.join(HERE, "_ref", "libref_euler2d.so")


def _reference_tree() -> str:
    """Location of the reference sources: $EULER2D_REFERENCE when set, else
    the REF default of oracle/Makefile (the recipe that compiles them where
    they lie).  An empty string when neither names a directory."""
    env = os.environ.get("EULER2D_REFERENCE")
    if env:
        return env
    try:
        r = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "refdir"],
                           capture_output=True, text=True, timeout=30)
        return r.stdout.strip() if r.returncode == 0 else ""
    except (OSError, subprocess.SubprocessError):
        return ""


REFERENCE_TREE = _reference_tree()

SOLVERS = {"hll": 0, "hllc": 1, "exact": 2, "force": 3}
BC = {"transmissive": 0, "reflective": 1, "halo": 2}

_dp = C.POINTER(C.c_double)
_llp = C.POINTER(C.c_longlong)


class OrcGrid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int),
                ("x_min", C.c_double), ("x_max", C.c_double),
                ("y_min", C.c_double), ("y_max", C.c_double),
                ("bc", C.c_int * 4)]


def build(reference: bool | None = None) -> None:
    """Compile the restatement (always), the loader of the reference's GPU
    image (where nvcc is), and the reference CPU build plus the reference's
    GPU device image (when the reference tree exists or ``reference`` is
    True)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc"):
        env = dict(os.environ)
        if not shutil.which("nvcc"):
            env["NVCC"] = "/usr/local/cuda/bin/nvcc"
        subprocess.run(["make", "-s", "-C", HERE, "refgpu_harness"], check=True, env=env)
    want_ref = bool(REFERENCE_TREE) and os.path.isdir(REFERENCE_TREE) if reference is None else reference
    if want_ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REFERENCE_TREE}"], check=True,
                       stderr=subprocess.DEVNULL)


OPC_SO = os.path.join(HERE, "_build", "libopcount_euler2d.so")
REFGPU_SO = os.path.join(HERE, "_build", "libref_gpu_harness.so")
REFGPU_IMAGE = os.path.join(HERE, "_ref", "ref_solver_gpu.cubin")


def reference_gpu_available() -> bool:
    """The reference's own GPU device image and its loader are both built."""
    return os.path.exists(REFGPU_SO) and os.path.exists(REFGPU_IMAGE)


def reference_gpu_run(U: np.ndarray, g: "Grid", solver="hllc", cfl=0.8, warmup=0, nsteps=1):
    """The reference's own CUDA kernels (src/gpu/solver_gpu.cu, unmodified,
    compiled into oracle/_ref/ref_solver_gpu.cubin) stepped by the loop of
    scripts/gpu/main_gpu.cu (oracle/ref_gpu_harness.cu): `warmup` untimed and
    `nsteps` timed free CFL steps from U, which is advanced in place.
    Transmissive boundaries only (the reference kernels clamp their
    stencils).  Returns dict(wall_ms, dt_ms, x_ms, y_ms, dts) over the timed
    steps."""
    lib = C.CDLL(REFGPU_SO)
    lib.refgpu_last_error.restype = C.c_char_p
    lib.refgpu_run.restype = C.c_int
    lib.refgpu_run.argtypes = [C.c_char_p, _dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                               C.c_int, C.c_double, C.c_int, C.c_int, _dp, _dp]
    assert U.dtype == np.float64 and U.flags.c_contiguous and U.shape == g.shape
    assert all(b in ("transmissive", 0) for b in g.bc), "the reference GPU kernels are transmissive only"
    ms = np.zeros(4)
    dts = np.zeros(max(nsteps, 1))
    s = SOLVERS[solver] if isinstance(solver, str) else int(solver)
    rc = lib.refgpu_run(REFGPU_IMAGE.encode(), _p(U), g.nx, g.ny, g.x_min, g.x_max, g.y_min, g.y_max, s, cfl,
                        int(warmup), int(nsteps), _p(ms), _p(dts))
    if rc:
        raise RuntimeError("reference GPU run failed: " + lib.refgpu_last_error().decode())
    return dict(wall_ms=float(ms[0]), dt_ms=float(ms[1]), x_ms=float(ms[2]), y_ms=float(ms[3]), dts=dts[:nsteps])
SFD_SO = os.path.join(HERE, "_build", "libshadowfd_euler2d.so")


def frozen_fd(U0: np.ndarray, g: "Grid", dts, solver, dirs, eps: float, mask: np.ndarray, threads: int = 0):
    """Branch-frozen central differences of J = sum(rho^2 over mask) after
    len(dts) frozen-dt steps of the restatement (oracle/shadow_fd.cpp): the
    runs from U0 +- eps d take the unperturbed run's branch decisions.
    dirs: sequence of (rho, p) direction fields of shape (2, ny, nx).
    Returns dict(J0, Jp, Jm, fd, flips, U) with one entry per direction in
    fd / flips (decisions on which the +eps and -eps runs would differ) and
    U the unperturbed run's final grid."""
    lib = C.CDLL(SFD_SO)
    lib.sfd_max_dirs.restype = C.c_int
    lib.sfd_frozen_fd.restype = C.c_int
    lib.sfd_frozen_fd.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                  C.POINTER(C.c_int), _dp, C.c_longlong, C.c_int, _dp, C.c_int, C.c_double,
                                  C.POINTER(C.c_ubyte), _dp, C.POINTER(C.c_ulonglong), _dp]
    nd = len(dirs)
    assert 1 <= nd <= lib.sfd_max_dirs()
    assert U0.dtype == np.float64 and U0.flags.c_contiguous and U0.shape == g.shape
    D = np.ascontiguousarray(np.stack([np.asarray(d, dtype=np.float64).reshape(2, g.ny, g.nx) for d in dirs]))
    M = np.ascontiguousarray(mask.reshape(g.ny, g.nx).astype(np.uint8))
    dts = np.ascontiguousarray(np.asarray(dts, dtype=np.float64))
    J = np.zeros(1 + 2 * nd)
    flips = (C.c_ulonglong * nd)()
    bc = (C.c_int * 4)(*[BC[b] if isinstance(b, str) else int(b) for b in g.bc])
    s = SOLVERS[solver] if isinstance(solver, str) else int(solver)
    if threads:
        lib.sfd_set_threads_(C.c_int(threads))
    UN = g.zeros()
    rc = lib.sfd_frozen_fd(_p(U0), g.nx, g.ny, g.x_min, g.x_max, g.y_min, g.y_max, bc, _p(dts), len(dts), s,
                           _p(D), nd, eps, M.ctypes.data_as(C.POINTER(C.c_ubyte)), _p(J), flips, _p(UN))
    if rc:
        raise RuntimeError(f"sfd_frozen_fd failed ({rc})")
    Jp, Jm = J[1::2].copy(), J[2::2].copy()
    return dict(J0=float(J[0]), Jp=Jp, Jm=Jm, fd=(Jp - Jm) / (2.0 * eps), flips=np.array(list(flips)), U=UN)


def op_counts(U: np.ndarray, g: "Grid", cfl: float, t_end: float, solver="hllc", max_steps: int = 0) -> dict:
    """Floating-point operations of the restatement's time loop
    (scripts/cpu/main_cpu.cpp:217-262: ghost fill, compute_dt,
    advance_second_order) on U, advanced in place, counted by category
    (oracle/opcount.cpp).  Returns dict(steps, counts={category: n})."""
    lib = C.CDLL(OPC_SO)
    lib.opc_ncat.restype = C.c_int
    lib.opc_cat_name.restype = C.c_char_p
    lib.opc_cat_name.argtypes = [C.c_int]
    lib.opc_run_counted.restype = C.c_longlong
    lib.opc_run_counted.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                    C.POINTER(C.c_int), C.c_double, C.c_double, C.c_int, C.c_longlong,
                                    C.POINTER(C.c_ulonglong)]
    assert U.dtype == np.float64 and U.flags.c_contiguous and U.shape == g.shape
    n = lib.opc_ncat()
    counts = (C.c_ulonglong * n)()
    bc = (C.c_int * 4)(*[BC[b] if isinstance(b, str) else int(b) for b in g.bc])
    s = SOLVERS[solver] if isinstance(solver, str) else int(solver)
    steps = lib.opc_run_counted(_p(U), g.nx, g.ny, g.x_min, g.x_max, g.y_min, g.y_max, bc, cfl, t_end, s,
                                int(max_steps), counts)
    if steps < 0:
        raise RuntimeError("compute_dt: non-positive maximum wave speed.")
    return dict(steps=int(steps), counts={lib.opc_cat_name(k).decode(): int(counts[k]) for k in range(n)})


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


class Grid:
    """Geometry of one grid: interior nx x ny, 2 ghost layers, extents, BCs
    (left, right, bottom, top)."""

    def __init__(self, nx, ny, x_min=0.0, x_max=1.0, y_min=0.0, y_max=1.0,
                 bc=("transmissive",) * 4):
        self.nx, self.ny = int(nx), int(ny)
        self.x_min, self.x_max, self.y_min, self.y_max = map(float, (x_min, x_max, y_min, y_max))
        self.bc = tuple(bc)

    @property
    def shape(self):
        return (self.ny + 4, self.nx + 4, 4)

    def zeros(self):
        return np.zeros(self.shape, dtype=np.float64)

    def c(self) -> OrcGrid:
        g = OrcGrid(self.nx, self.ny, self.x_min, self.x_max, self.y_min, self.y_max)
        for k, b in enumerate(self.bc):
            g.bc[k] = BC[b] if isinstance(b, str) else int(b)
        return g

    def ext(self):
        return (self.nx, self.ny, self.x_min, self.x_max, self.y_min, self.y_max)

    @property
    def all_transmissive(self):
        return all((b == "transmissive" or b == 0) for b in self.bc)


class Oracle:
    def __init__(self, kind: str = "port"):
        self.kind = kind
        path = PORT_SO if kind == "port" else REF_SO
        if not os.path.exists(path):
            raise FileNotFoundError(f"oracle library missing: {path} (run oracle.build())")
        self.lib = C.CDLL(path)
        L = self.lib
        if kind == "port":
            G = C.POINTER(OrcGrid)
            L.orc_apply_boundary.argtypes = [_dp, G]
            L.orc_compute_dt.argtypes = [_dp, G, C.c_double, _dp]
            L.orc_compute_dt.restype = C.c_int
            L.orc_advance_second_order.argtypes = [_dp, _dp, _dp, G, C.c_double, C.c_int, _dp, _dp]
            L.orc_advance_first_order.argtypes = [_dp, _dp, G, C.c_double, C.c_int]
            L.orc_sweep_x.argtypes = [_dp, _dp, G, C.c_double, C.c_int, _dp]
            L.orc_sweep_y.argtypes = [_dp, _dp, G, C.c_double, C.c_int, _dp]
            L.orc_riemann_flux.argtypes = [_dp, _dp, C.c_int, C.c_int, _dp]
            L.orc_run.argtypes = [_dp, G, C.c_double, C.c_double, C.c_int, C.c_longlong, C.c_int,
                                  _dp, _llp, _dp, C.c_longlong, _llp, _dp, _dp]
            L.orc_run.restype = C.c_int
            L.orc_init_blast.argtypes = [_dp, G] + [C.c_double] * 7
            L.orc_init_shock_bubble.argtypes = [_dp, G] + [C.c_double] * 8
            L.orc_init_reference_case.argtypes = [_dp, G, C.c_int]
            L.orc_set_threads.argtypes = [C.c_int]
            L.orc_get_threads.restype = C.c_int
        else:
            E = [C.c_int, C.c_int] + [C.c_double] * 4
            L.ref_apply_transmissive_boundary.argtypes = [_dp] + E
            L.ref_compute_dt.argtypes = [_dp] + E + [C.c_double, _dp]
            L.ref_compute_dt.restype = C.c_int
            L.ref_advance_second_order.argtypes = [_dp, _dp, _dp] + E + [C.c_double, C.c_int]
            L.ref_advance_first_order.argtypes = [_dp, _dp] + E + [C.c_double, C.c_int]
            L.ref_riemann_flux.argtypes = [_dp, _dp, C.c_int, C.c_int, _dp]
            L.ref_case_config.argtypes = [C.c_int, C.c_int, _dp]
            L.ref_init_case.argtypes = [C.c_int, C.c_int, _dp]
            L.ref_run.argtypes = [_dp] + E + [C.c_double, C.c_double, C.c_int, C.c_longlong,
                                              C.c_int, _dp, _llp, _dp, C.c_longlong, _llp, _dp]
            L.ref_run.restype = C.c_int

    # -- helpers ---------------------------------------------------------
    def _check_ref_grid(self, g: Grid):
        if self.kind != "port" and not g.all_transmissive:
            raise ValueError("the reference build only has transmissive boundaries")

    def set_threads(self, n: int):
        if self.kind == "port":
            self.lib.orc_set_threads(int(n))
        else:
            os.environ["OMP_NUM_THREADS"] = str(n)

    def threads(self) -> int:
        if self.kind == "port":
            return int(self.lib.orc_get_threads())
        return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))

    # -- API ---------------------------------------------------------------
    def apply_boundary(self, U: np.ndarray, g: Grid) -> None:
        assert U.flags.c_contiguous and U.dtype == np.float64 and U.shape == g.shape
        if self.kind == "port":
            gc = g.c()
            self.lib.orc_apply_boundary(_p(U), C.byref(gc))
        else:
            self._check_ref_grid(g)
            self.lib.ref_apply_transmissive_boundary(_p(U), *g.ext())

    def compute_dt(self, U: np.ndarray, g: Grid, cfl: float):
        dt = C.c_double(0.0)
        if self.kind == "port":
            gc = g.c()
            rc = self.lib.orc_compute_dt(_p(U), C.byref(gc), cfl, C.byref(dt))
        else:
            rc = self.lib.ref_compute_dt(_p(U), *g.ext(), cfl, C.byref(dt))
        if rc:
            raise RuntimeError("compute_dt: non-positive maximum wave speed.")
        return dt.value

    def advance_second_order(self, Uold, g: Grid, dt: float, solver="hll", Utmp=None, Unew=None,
                             fx=None, fy=None):
        """One split step (src/cpu/solver_cpu.cpp:400-499).  fx / fy are the
        face-flux caches of 4*(nx+1)*ny and 4*nx*(ny+1) doubles (the
        CpuWorkspace of head/cpu/solver_cpu.hpp:16-40), allocated per call
        when not given (port only)."""
        s = SOLVERS[solver] if isinstance(solver, str) else int(solver)
        Utmp = g.zeros() if Utmp is None else Utmp
        Unew = g.zeros() if Unew is None else Unew
        Uold = np.ascontiguousarray(Uold, dtype=np.float64)
        if self.kind == "port":
            gc = g.c()
            if fx is not None:
                assert fx.dtype == np.float64 and fx.size >= 4 * (g.nx + 1) * g.ny
                assert fy.dtype == np.float64 and fy.size >= 4 * g.nx * (g.ny + 1)
            self.lib.orc_advance_second_order(_p(Uold), _p(Utmp), _p(Unew), C.byref(gc), dt, s,
                                              _p(fx) if fx is not None else None,
                                              _p(fy) if fy is not None else None)
        else:
            self._check_ref_grid(g)
            self.lib.ref_advance_second_order(_p(Uold), _p(Utmp), _p(Unew), *g.ext(), dt, s)
        return Utmp, Unew

    def sweep_x(self, Uold, Utmp, g: Grid, dt: float, solver="hll"):
        """x half of the split step (interior of Utmp from Uold), no ghost fill."""
        s = SOLVERS[solver] if isinstance(solver, str) else int(solver)
        gc = g.c()
        self.lib.orc_sweep_x(_p(Uold), _p(Utmp), C.byref(gc), dt, s, None)

    def sweep_y(self, Utmp, Unew, g: Grid, dt: float, solver="hll"):
        """y half of the split step (interior of Unew from Utmp incl. its ghost rows), no ghost fill."""
        s = SOLVERS[solver] if isinstance(solver, str) else int(solver)
        gc = g.c()
        self.lib.orc_sweep_y(_p(Utmp), _p(Unew), C.byref(gc), dt, s, None)

    def advance_first_order(self, Uold, g: Grid, dt: float, solver="hll"):
        s = SOLVERS[solver] if isinstance(solver, str) else int(solver)
        Unew = g.zeros()
        Uold = np.ascontiguousarray(Uold, dtype=np.float64)
        if self.kind == "port":
            gc = g.c()
            self.lib.orc_advance_first_order(_p(Uold), _p(Unew), C.byref(gc), dt, s)
        else:
            self._check_ref_grid(g)
            self.lib.ref_advance_first_order(_p(Uold), _p(Unew), *g.ext(), dt, s)
        return Unew

    def riemann_flux(self, UL, UR, direction: int, solver="hll"):
        s = SOLVERS[solver] if isinstance(solver, str) else int(solver)
        UL = np.ascontiguousarray(UL, dtype=np.float64)
        UR = np.ascontiguousarray(UR, dtype=np.float64)
        F = np.zeros(4)
        fn = self.lib.orc_riemann_flux if self.kind == "port" else self.lib.ref_riemann_flux
        fn(_p(UL), _p(UR), int(direction), s, _p(F))
        return F

    def run(self, U, g: Grid, cfl: float, t_end: float, solver="hll", max_steps=0, nsnap=0,
            dt_cap=1 << 20, want_snapshots=False):
        """Time loop of scripts/cpu/main_cpu.cpp:206-262.  U is advanced in place.
        Returns dict(t, steps, dts, snap_step, snap_t[, snapshots])."""
        s = SOLVERS[solver] if isinstance(solver, str) else int(solver)
        t = C.c_double(0.0)
        n = C.c_longlong(0)
        cap = int(dt_cap) if max_steps <= 0 else min(int(dt_cap), int(max_steps))
        dts = np.zeros(max(cap, 1))
        ss = np.zeros(max(nsnap, 1), dtype=np.int64)
        st = np.zeros(max(nsnap, 1))
        snaps = None
        if self.kind == "port":
            gc = g.c()
            if want_snapshots and nsnap > 0:
                snaps = np.zeros((nsnap,) + g.shape)
            rc = self.lib.orc_run(_p(U), C.byref(gc), cfl, t_end, s, int(max_steps), int(nsnap),
                                  C.byref(t), C.byref(n), _p(dts), cap,
                                  ss.ctypes.data_as(_llp), _p(st),
                                  _p(snaps) if snaps is not None else None)
        else:
            self._check_ref_grid(g)
            rc = self.lib.ref_run(_p(U), *g.ext(), cfl, t_end, s, int(max_steps), int(nsnap),
                                  C.byref(t), C.byref(n), _p(dts), cap,
                                  ss.ctypes.data_as(_llp), _p(st))
        if rc:
            raise RuntimeError("compute_dt: non-positive maximum wave speed.")
        out = dict(t=t.value, steps=n.value, dts=dts[: min(n.value, cap)].copy(),
                   snap_step=ss[:nsnap].copy(), snap_t=st[:nsnap].copy())
        if snaps is not None:
            out["snapshots"] = snaps
        return out

    # -- initial states (port only) ---------------------------------------
    def init_blast(self, g: Grid, cx=1.0, cy=1.0, r=0.4, rho_in=1.0, p_in=1.0,
                   rho_out=0.125, p_out=0.1):
        U = g.zeros()
        gc = g.c()
        self.lib.orc_init_blast(_p(U), C.byref(gc), cx, cy, r, rho_in, p_in, rho_out, p_out)
        return U

    def init_shock_bubble(self, g: Grid, rho0=1.0, p0=1.0, mach=1.22, shock_x=0.005,
                          bub_cx=0.035, bub_cy=0.0445, bub_r=0.025, rho_bubble=0.138):
        U = g.zeros()
        gc = g.c()
        self.lib.orc_init_shock_bubble(_p(U), C.byref(gc), rho0, p0, mach, shock_x, bub_cx,
                                       bub_cy, bub_r, rho_bubble)
        return U

    def init_reference_case(self, g: Grid, case_id: int):
        U = g.zeros()
        if self.kind == "port":
            gc = g.c()
            self.lib.orc_init_reference_case(_p(U), C.byref(gc), int(case_id))
        else:
            raise NotImplementedError("use ref_init_case via init_reference_n")
        return U

    def reference_case(self, case_id: int, n: int):
        """(Grid, U0, cfl, t_end) of the reference's own case at scale n
        (src/test_cases.cpp:132-195).  Reference build only."""
        out = np.zeros(9)
        self.lib.ref_case_config(int(case_id), int(n), _p(out))
        g = Grid(int(out[0]), int(out[1]), out[3], out[4], out[5], out[6])
        U = g.zeros()
        self.lib.ref_init_case(int(case_id), int(n), _p(U))
        return g, U, float(out[7]), float(out[8])
