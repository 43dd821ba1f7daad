/*
 * euler2d.h -- C ABI of the GB300 (sm_103a) MUSCL-Hancock split step for the
 * 2D compressible Euler equations.
 *
 * Drop-in boundary for the reference CPU/OpenMP solver.  The reference's C++
 * surface is
 *   double compute_dt(const Grid2D&, double cfl)                 src/cpu/solver_cpu.cpp:287-309
 *   void advance_second_order(const Grid2D& Uold, Grid2D& Utmp,
 *        Grid2D& Unew, double dt, CpuWorkspace&, RiemannSolver)  src/cpu/solver_cpu.cpp:400-499
 *   void advance_first_order(...)                                src/cpu/solver_cpu.cpp:315-369
 *   CaseConfig / get_n_case_config / initial_state_at            head/test_cases.hpp:8-35
 * and its driver loop is scripts/cpu/main_cpu.cpp:206-262.  Each entry point
 * below names the reference interface it replaces.  A C++ shim with the exact
 * solver_cpu.hpp signatures sits on top of this ABI
 * (large_sys_eq_opt_gb300/shim/solver_cpu_gb300.cpp).
 *
 * Conventions
 *   - every function returns EU_OK (0) or an eu_status code; it never
 *     throws and never exits.  eu_last_error(h) (h may be NULL for errors of
 *     eu_create and the case helpers) gives a message.
 *   - host grids ("AoS") use the reference Grid2D layout
 *     (head/cpu/grid_cpu.hpp:10-89): 4 doubles per cell (rho, rhou, rhov, E),
 *     (nx+4)*(ny+4) cells including the 2-cell ghost frame, cell (i, j) at
 *     index j*(nx+4)+i.
 *   - one handle = one grid, one CUDA stream, device-resident state.  A
 *     handle is not thread-safe; several handles may be used concurrently.
 *   - no CPU fallback: without a usable sm_103a device, eu_create fails.
 */
#ifndef EULER2D_H
#define EULER2D_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EU_ABI_VERSION 1

typedef struct eu_handle eu_handle;

typedef enum {
    EU_OK = 0,
    EU_ERR_INVALID = 1,     /* bad argument or configuration */
    EU_ERR_CUDA = 2,        /* CUDA runtime/driver failure */
    EU_ERR_NOMEM = 3,       /* device or pinned allocation failed */
    EU_ERR_NONPHYSICAL = 4, /* maximum wave speed not positive / not finite
                               (the reference throws std::runtime_error,
                               src/cpu/solver_cpu.cpp:304-306) */
    EU_ERR_TIMEOUT = 5,     /* a bounded device wait expired */
    EU_ERR_STATE = 6        /* call not valid in the handle's current state */
} eu_status;

typedef enum { EU_FP64 = 0, EU_FP32 = 1 } eu_precision;

/* Same order as RiemannSolver (head/riemann.hpp:13-18). */
typedef enum { EU_HLL = 0, EU_HLLC = 1, EU_EXACT = 2, EU_FORCE = 3 } eu_solver;

/* minmod is the reference's only limiter (src/cpu/solver_cpu.cpp:22-37). */
typedef enum { EU_LIMITER_MINMOD = 0 } eu_limiter;

/* Per-side boundary; the reference has transmissive only
 * (head/cpu/boundary_cpu.hpp:5-37).  Reflective mirrors the two ghost layers
 * and negates the normal momentum. */
typedef enum { EU_BC_TRANSMISSIVE = 0, EU_BC_REFLECTIVE = 1 } eu_bc;
enum { EU_SIDE_LEFT = 0, EU_SIDE_RIGHT = 1, EU_SIDE_BOTTOM = 2, EU_SIDE_TOP = 3 };

/* CaseConfig (head/test_cases.hpp:8-18).  ng must be 2. */
typedef struct {
    int nx, ny, ng;
    double x_min, x_max, y_min, y_max;
    double cfl, t_end;
} eu_case;

typedef struct {
    double t;           /* final simulation time */
    long long steps;    /* steps taken */
    int status;         /* device status bits (0 = clean) */
    int nsnap_written;  /* snapshots delivered to the callback */
} eu_run_info;

/* Snapshot callback of eu_run: k = 1..nsnap, the step and time at which the
 * reference writes it (first step with t >= t_end*k/nsnap,
 * scripts/cpu/main_cpu.cpp:244-261) and the full grid in Grid2D AoS layout
 * (valid during the call).  Return non-zero to abort the run. */
typedef int (*eu_snapshot_cb)(void* user, int k, long long step, double t, const double* aos, int nx,
                              int ny);

/* ---- handle lifecycle ---------------------------------------------------- */
/* Replaces Grid2D x3 + CpuWorkspace::init (scripts/cpu/main_cpu.cpp:175-191,
 * head/cpu/solver_cpu.hpp:28-33).  bc: left, right, bottom, top (NULL = all
 * transmissive). */
int eu_create(const eu_case* cfg, eu_precision prec, eu_solver solver, eu_limiter limiter, const int* bc,
              eu_handle** out);
void eu_destroy(eu_handle* h);
const char* eu_last_error(const eu_handle* h);
int eu_abi_version(void);

/* ---- setup (src/test_cases.cpp, src/init.cpp) ---------------------------- */
/* get_n_case_config (src/test_cases.cpp:184-195); name "shock_bubble" or
 * "blast_wave"; unknown names fail like parse_case_id. */
int eu_get_case_config(const char* name, int n, eu_case* out);
/* initialise_grid with the reference case (src/init.cpp:29-38), on device. */
int eu_init_reference_case(eu_handle* h, const char* name);
/* Parameterised blast / shock-bubble states (src/test_cases.cpp:24-101), on device. */
int eu_init_blast(eu_handle* h, double cx, double cy, double r, double rho_in, double p_in, double rho_out,
                  double p_out);
int eu_init_shock_bubble(eu_handle* h, double rho0, double p0, double mach, double shock_x, double bub_cx,
                         double bub_cy, double bub_r, double rho_bubble);

/* ---- state transfer -------------------------------------------------------- */
int eu_upload_aos(eu_handle* h, const double* aos);   /* whole grid incl. ghosts */
int eu_download_aos(eu_handle* h, double* aos);       /* ghosts filled by the BC rule */

/* ---- the hot path ---------------------------------------------------------- */
/* compute_dt (src/cpu/solver_cpu.cpp:287-309) on the device state. */
int eu_compute_dt(eu_handle* h, double cfl, double* dt);
/* advance_second_order (src/cpu/solver_cpu.cpp:400-499) on the device state:
 * x-sweep, BC, y-sweep, BC, with the given dt. */
int eu_advance(eu_handle* h, double dt);
/* advance_first_order (src/cpu/solver_cpu.cpp:315-369): first-order
 * Godunov step with the handle's Riemann solver, ghosts of the result
 * refilled by the boundary rule. */
int eu_advance_first_order(eu_handle* h, double dt);
int eu_advance_first_order_host(eu_handle* h, const double* Uold, double* Unew, double dt);
/* n steps device-resident in a CUDA graph.  dts == NULL: each dt from the
 * fused CFL reduction (no t_end clip); otherwise the frozen list dts[0..n). */
int eu_step_n(eu_handle* h, long long n, const double* dts);
/* The time loop of scripts/cpu/main_cpu.cpp:206-262 from t = 0 on the current
 * state: dt, t_end clip and snapshot schedule on the device, steps replayed
 * from a CUDA graph, snapshots copied asynchronously and handed to cb. */
int eu_run(eu_handle* h, double t_end, int nsnap, eu_snapshot_cb cb, void* user, eu_run_info* info);
/* Current time, completed steps and the dt the next step would use. */
int eu_get_time(eu_handle* h, double* t, long long* steps, double* dt_next);
/* apply_transmissive_boundary (head/cpu/boundary_cpu.hpp:5-37) with the
 * handle's per-side rule, on the device state. */
int eu_apply_boundary(eu_handle* h);
/* Record the dt of every step (indexed by the handle's step counter; eu_run
 * restarts it at 0) into a device log of `capacity` entries; 0 disables. */
int eu_set_dt_log(eu_handle* h, long long capacity);
int eu_get_dt_log(eu_handle* h, double* out, long long n);
/* FP64 totals of rho, rhou, rhov, E over the interior (conserved audit). */
int eu_totals(eu_handle* h, double out[4]);
/* eu_totals for callers that cannot let this library allocate device memory
 * (no counterpart in the reference).  For a caller that owns all device
 * memory through its own pool -- a framework's caching allocator, or an
 * application that reserves the HBM at start-up -- and so cannot create a
 * handle (eu_create allocates); cudaMalloc/cudaFree would synchronise the
 * device and fragment that pool.  Allocates nothing: no cudaMalloc/cudaFree,
 * no allocating library.
 *   d_aos   the caller's grid in device memory of the current device, Grid2D
 *           AoS layout with ghosts ((nx+4)*(ny+4)*4 doubles), 16-byte aligned;
 *           only interior cells are read.
 *   d_out   4 doubles of the caller's device memory (8-byte aligned) that
 *           receive the totals; they need not start at zero.
 *   stream  cudaStream_t to enqueue on (NULL = the default stream).  The call
 *           returns once the work is enqueued; d_out is ready when the stream
 *           reaches it.
 * Scratch: a fixed 1 MiB array inside the library (8 doubles per interior
 * row).  ny > 16384 is rejected with EU_ERR_INVALID; nothing in the scratch
 * has to start at zero.  Every call looks the scratch's address up with
 * cudaGetSymbolAddress in the current context (so a device reset cannot
 * leave a stale address).  With lazy module loading, the CUDA default, the
 * first call on a device loads the library's device image, 1 MiB array
 * included: that one call may take device memory.  A caller that hands all
 * HBM to its own pool makes one warm-up call first (or sets
 * CUDA_MODULE_LOADING=EAGER), and makes the first call before any stream
 * capture begins.  All calls on one device share the scratch, so two calls
 * whose work overlaps (different streams or host threads, unordered) race
 * and give wrong totals: order them on one stream or with events. */
int eu_totals_noalloc(const double* d_aos, int nx, int ny, double* d_out, void* stream);

/* ---- discrete adjoint (no counterpart in the reference) ---------------------- */
/* Gradient of a scalar objective J(U_N) of the state after nsteps steps with
 * the frozen step sizes dts[0..nsteps), with respect to the current state
 * U_0, through the discrete adjoint of the split step (transposed
 * reconstruction with minmod subgradients, transposed Riemann-flux
 * Jacobians, the exact solver through implicit differentiation at the
 * converged p*, transposed boundary rule).
 * eu_adjoint_forward runs the nsteps steps from the current state, keeping a
 * checkpoint every ckpt_k steps (plus the last segment's intermediate
 * states); the handle's state becomes U_N and its time advances by sum(dts).
 * With dts NULL the steps take CFL step sizes as eu_step_n does (chosen on
 * the device from each state) and the backward differentiates with those
 * sizes held fixed; eu_adjoint_dts returns them.  ckpt_k in [0, 1024]; 0
 * keeps every step's state on the device (nothing recomputed by the
 * backward) when that fits in half the free device memory, else
 * checkpoints every ceil(sqrt(nsteps)) steps (the batched calls decide
 * this once for all instances).
 * eu_adjoint_backward takes dJ/dU_N and returns dJ/dU_0 (both host grids in
 * Grid2D AoS layout; ghost entries of the input are ignored, those of the
 * output are zero), recomputing each earlier segment's states from its
 * checkpoint.  It can be called repeatedly after one forward pass.  The
 * arithmetic is the handle's precision.  Needs nx, ny >= 2. */
int eu_adjoint_forward(eu_handle* h, long long nsteps, const double* dts, int ckpt_k);
int eu_adjoint_backward(eu_handle* h, const double* dJ_dUN, double* dJ_dU0);
/* The step sizes of the last eu_adjoint_forward (given or CFL-chosen):
 * *nsteps = their number, the first min(cap, *nsteps) copied to dts. */
int eu_adjoint_dts(eu_handle* h, double* dts, long long cap, long long* nsteps);
/* Device time (CUDA events) of the last eu_adjoint_forward (ms[0], its steps
 * only) and eu_adjoint_backward (ms[1], recomputation + adjoint sweeps). */
int eu_adjoint_timing(eu_handle* h, float ms[2]);

/* ---- uneven ensembles (no counterpart in the reference) ---------------------- */
/* n independent grids (own size, boundaries, case, parameters, CFL and
 * t_end) advanced together: every step is one persistent launch over a work
 * list of all instances' sweep tasks, and each instance keeps its own
 * device-computed dt.  Each instance's results are bit-for-bit those of its
 * own handle.  eu_batch_handle(b, i) gives the instance's handle for the
 * setup, state transfer, totals and option calls above (do not destroy it;
 * do not step it on its own while the batch is stepping). */
typedef struct eu_batch eu_batch;
int eu_batch_create(int n, const eu_case* cfgs, const int* bcs /* 4 per instance or NULL */, eu_precision prec,
                    eu_solver solver, eu_batch** out);
void eu_batch_destroy(eu_batch* b);
const char* eu_batch_last_error(const eu_batch* b);
eu_handle* eu_batch_handle(eu_batch* b, int i);
/* t = 0 on every instance: ghosts filled, first dt from the CFL reduction,
 * each instance stops at its own cfg.t_end (the reference loop's clip). */
int eu_batch_start(eu_batch* b);
/* nsteps ensemble steps (finished instances idle); *all_done (may be NULL)
 * reports whether every instance reached its t_end. */
int eu_batch_step(eu_batch* b, long long nsteps, int* all_done);
/* Steps until every instance reached its t_end or max_steps were taken. */
int eu_batch_run(eu_batch* b, long long max_steps, long long* steps_taken);
/* Device time (CUDA events) of nsteps graph-replayed ensemble steps. */
int eu_batch_time_steps(eu_batch* b, int nsteps, float* ms);
/* Ensemble tile-shape autotuner: one (seg_x, seg_y) pair for all instances
 * (clipped to each grid), chosen by timing whole ensemble steps; states
 * restored afterwards. */
int eu_batch_autotune(eu_batch* b, int steps, long long chosen[2]);
/* Batched discrete adjoint: eu_adjoint_forward / eu_adjoint_backward of
 * every instance (instance i: nsteps[i] steps with its own frozen dts[i]).
 * The forward steps of all instances run as one ensemble launch per step
 * (while every instance is on the batch's solver; else each on its own
 * stream), the backwards concurrently on the instances' own streams.
 * With dts NULL (or dts[i] NULL) instance i takes CFL steps as in
 * eu_batch_step: at most nsteps[i], stopping at its own t_end.
 * Gradients with respect to scalar case parameters follow by the chain
 * rule dJ/dtheta = <dJ/dU_0, dU_0/dtheta> (large_sys_eq_opt_gb300/adjoint.py). */
int eu_batch_adjoint_forward(eu_batch* b, const long long* nsteps, const double* const* dts, int ckpt_k);
int eu_batch_adjoint_backward(eu_batch* b, const double* const* dJ_dUN, double* const* dJ_dU0);
/* Scalar case parameters of one instance (no reference counterpart; the
 * values of src/test_cases.cpp:24-101 made parameters):
 *   kind 0, blast:        v = {cx, cy, R, rho_in, p_in, rho_out, p_out}
 *   kind 1, shock-bubble: v = {rho0, p0, Mach, shock_x, bub_cx, bub_cy, bub_r,
 *                              rho_bubble} */
typedef struct {
    int kind;
    double v[8];
} eu_case_params;
/* The differentiable initial state of those parameters on the handle's grid,
 * evaluated on the device at the cell centres: the blast with its interface
 * as the one-cell linear ramp frac = clip(1/2 - (r - R)/h, 0, 1), h =
 * min(dx, dy) (the cell average of a straight interface, so that the state
 * is differentiable in R), the shock-bubble as src/test_cases.cpp:24-69. */
int eu_init_params(eu_handle* h, const eu_case_params* p);
/* Objective values and gradients with respect to two scalar parameters per
 * instance, entirely on the device: each instance starts from
 * eu_init_params(params[i]), runs nsteps[i] steps with the frozen step
 * sizes dts[i] (checkpoints every ckpt_k; dts or dts[i] NULL: CFL steps as
 * in eu_batch_step, at most nsteps[i] and up to the instance's t_end, their
 * sizes then held fixed and readable by eu_adjoint_dts on the instance's
 * handle), J_i = sum of rho^2 over the ring
 * 0.6 <= r <= 0.8 from the blast centre or 1.2 r_b <= d <= 1.6 r_b from the
 * bubble centre, and dJ_i/dtheta = <dJ/dU_0, dU_0/dtheta> with the closed-form
 * tangents of the initial state.  dJ[2i], dJ[2i+1] = dJ/dR, dJ/dp_in (blast)
 * or dJ/drho_bubble, dJ/dMach (shock-bubble).  Only these 3n numbers cross
 * the host link.  The forwards run as in eu_batch_adjoint_forward, the
 * rest of each instance's work on its own stream, enqueued by several host
 * threads. */
int eu_batch_param_gradients(eu_batch* b, const eu_case_params* params, const long long* nsteps,
                             const double* const* dts, int ckpt_k, double* J, double* dJ);
/* Test hook of the failure-detection path (no reference counterpart): with
 * n > 0 every y-sweep task waits for n more x-sweep tasks than exist, its
 * bounded wait (2 s) expires, and eu_batch_step returns EU_ERR_TIMEOUT with
 * the device context intact.  0 restores normal operation. */
int eu_batch_set_wait_extra(eu_batch* b, int n);

/* ---- drop-in calls on host grids (what the reference's callers pass) ------- */
/* compute_dt(const Grid2D&, double): upload, reduce, read back dt. */
int eu_compute_dt_host(eu_handle* h, const double* U, double cfl, double* dt);
/* advance_second_order(Uold, Utmp, Unew, dt, ws, solver) on host grids:
 * upload Uold, one step, download Unew (and Utmp when non-NULL). */
int eu_advance_host(eu_handle* h, const double* Uold, double* Utmp, double* Unew, double dt);
/* One iteration of the reference loop body on host grids
 * (scripts/cpu/main_cpu.cpp:222-241): upload U, dt = compute_dt(U, cfl)
 * clipped to t_end - t, advance, download into Unext; *dt_used returns dt. */
int eu_step_host(eu_handle* h, const double* U, double* Unext, double cfl, double t, double t_end,
                 double* dt_used);

/* ---- measurement ------------------------------------------------------------- */
/* Runs nsteps free-running CFL steps (one CUDA graph when use_graph) with
 * CUDA events on the handle's stream around every kernel.  ms[0] = total
 * elapsed, ms[1] = sum over x-sweep launches, ms[2] = sum over y-sweep
 * launches. */
int eu_time_steps(eu_handle* h, int nsteps, int use_graph, float ms[3]);
/* Pinned host memory for zero-staging transfers. */
int eu_host_alloc(size_t bytes, void** p);
void eu_host_free(void* p);
/* Launch-shape options of a handle (no reference counterpart): "seg_x"
 * (x-sweep segment length, a multiple of the box width), "seg_y" (y-sweep
 * rows per warp), "l2_promotion_x" / "l2_promotion_y" (TMA L2 promotion in
 * bytes: 0, 64, 128, 256; defaults 128 and 256), "graph_steps" (steps per
 * replayed graph), "solver" (the eu_solver of later steps: the reference
 * passes the solver to every advance_second_order call,
 * head/cpu/solver_cpu.hpp:62-80, so one handle serves every solver of a
 * geometry; the state is kept, the launch plan becomes the planner's for the
 * new solver; a completed adjoint forward pass is discarded, so
 * eu_adjoint_backward returns EU_ERR_STATE until the next forward, and a
 * batch's own ensemble steps keep the batch's solver).
 * Read-only: "tasks_x", "tasks_y", "occ_x", "occ_y", "sm_count", and
 * "ckpt_k" (the checkpoint spacing of the last adjoint forward).  Used by
 * the tile-shape autotuner. */
int eu_set_option(eu_handle* h, const char* name, long long value);
int eu_get_option(eu_handle* h, const char* name, long long* value);
/* Tile-shape autotuner (no reference counterpart): times candidate segment
 * lengths of both sweeps on this handle's grid (the best of two runs of
 * `steps` graph-replayed steps per candidate, CUDA events per kernel),
 * keeps the current lengths unless a candidate is more than 1% faster, and
 * returns the chosen ones in chosen[0] (seg_x) and chosen[1] (seg_y).  Every
 * candidate starts from the state, time and step counter of the call, and
 * they are left as they were. */
int eu_autotune(eu_handle* h, int steps, long long chosen[2]);
/* Diagnostics (no reference counterpart): copy the raw device planes of
 * state buffer 0/1 (which = 0, 1) or of the x-sweep output (which = 2) to
 * `out` (4 planes of `plane` elements in the handle's precision; interior
 * cell (i, j) of a state buffer at column i+6, row j+2; of the x-sweep output
 * at column i+8).  out == NULL only reports the pitch and plane length. */
int eu_read_planes(eu_handle* h, int which, void* out, size_t bytes, long long* pitch, long long* plane);
/* Diagnostics counterpart of eu_read_planes: overwrite the raw planes of a
 * buffer (bytes = 4 planes), e.g. to plant canary values in the unused
 * columns and padding and check that no kernel reads or writes them. */
int eu_write_planes(eu_handle* h, int which, const void* in, size_t bytes);
/* Restart files (no reference counterpart): the state (Grid2D AoS, FP64),
 * grid geometry, time and step counter; eu_load_state accepts only a file
 * of the same grid. */
int eu_save_state(eu_handle* h, const char* path);
int eu_load_state(eu_handle* h, const char* path);
/* ---- slab decomposition of one grid ------------------------------------------ */
/* One grid split into nslabs slabs of whole rows, each with a 2-row halo:
 * the semantics of the reference's domain decomposition
 * (src/cpu/solver_mpi.cpp:246-291 partition, :340-402 and :547-573 halo
 * exchange, :416-443 dt reduction) for slabs on the current device.  Per
 * step: every slab's x-sweep, then the x-sweep outputs' two boundary rows
 * copied into each neighbour's halo rows, every slab's y-sweep, then one dt
 * for all slabs (the smallest of the slabs' proposals, which equals the
 * undivided grid's CFL dt).  The results equal one handle's on the whole
 * grid bit for bit.  Slab s holds interior rows [row0[s], row0[s+1]) with
 * row0[s] = s*ny/nslabs; bc as eu_create (the outer sides only).  Needs
 * ny >= 2*nslabs. */
typedef struct eu_domain eu_domain;
int eu_domain_plan(int ny, int nslabs, int* row0 /* nslabs + 1 */);
int eu_domain_create(const eu_case* cfg, eu_precision prec, eu_solver solver, eu_limiter limiter, const int* bc,
                     int nslabs, eu_domain** out);
void eu_domain_destroy(eu_domain* d);
const char* eu_domain_last_error(const eu_domain* d);
/* The whole grid in the Grid2D AoS layout (ghosts included). */
int eu_domain_upload_aos(eu_domain* d, const double* aos);
int eu_domain_download_aos(eu_domain* d, double* aos);
/* n CFL steps (clipped to t_end, which may be +inf), as eu_step_n. */
int eu_domain_step_n(eu_domain* d, long long n, double t_end);
int eu_domain_get_time(eu_domain* d, double* t, long long* steps);

/* Device used by handles created afterwards on the calling thread. */
int eu_set_device(int device);
/* Name of device 0 and its SM count, for logs. */
int eu_device_info(char* name, int len, int* sm_count);

#ifdef __cplusplus
}
#endif
#endif /* EULER2D_H */
