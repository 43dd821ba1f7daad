// eu_internal.h -- device control block and launch descriptors shared by the
// sweep kernels and the host runtime (not part of the public C ABI).
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace eu {

constexpr int kMaxSnap = 16;

// Device-resident step control.  One per handle, in device memory.  The
// y-sweep's last warp (last-block-done, no spin) turns the step's maximum
// signal speed into the next dt, advances t, applies the t_end clip and the
// snapshot schedule of scripts/cpu/main_cpu.cpp:206-262, so dt never goes
// back to the host.
struct Ctl {
    double t;            // simulation time at the start of the next step
    double dt;           // step size the next step will use
    double t_end;        // +inf for free-running steps
    double cfl_dmin;     // cfl * min(dx, dy)
    double smax;         // last reduced maximum signal speed (diagnostic)
    const double* frozen;  // frozen dt list (mode kModeFrozen)
    double* dt_log;        // dt of every completed step (may be null)
    long long dt_log_cap;
    long long n_frozen;
    long long frozen_base;  // step index of frozen[0]
    long long max_steps; // done once step reaches this
    long long step;      // completed steps
    unsigned long long smax_bits;  // running max (bit pattern of a non-negative double)
    unsigned int arrive;           // warps finished in the current launch
    int done;            // 1 once t >= t_end, the frozen list is exhausted or on error
    int status;          // kStatus* bits
    int mode;            // kModeCfl / kModeFrozen / kModeHost
    int cur;             // state buffer (0/1) holding the latest state
    int nsnap, next_snap;
    unsigned int snap_req;   // bit k: snapshot k is the state at the start of the next step
    unsigned int snap_taken; // bit k: copied into snapshot storage
    unsigned int ytask_next; // y-sweep work list: next task to hand out (0 between launches)
    unsigned int ytask_exit; // y-sweep warps that found the list empty (0 between launches)
    int pad;
    double snap_target[kMaxSnap];
    double snap_time[kMaxSnap];
    long long snap_step[kMaxSnap];
};

enum { kModeCfl = 0, kModeFrozen = 1, kModeHost = 2 };
enum { kStatusOk = 0, kStatusNonPhysical = 1, kStatusTimeout = 2, kStatusNonFinite = 4 };

// Column of interior cell i in the state buffers S0/S1 (ghosts at i+4, i+5
// and nx+6, nx+7; columns 0-3 unused) and in Utmp.  With these offsets
// every TMA box and every warp-wide row store of both sweeps starts on a
// 32-byte sector boundary, so DRAM never sees a partial-sector write (which
// costs an ECC read-modify-write).
constexpr int kSOff = 6;
constexpr int kTOff = 8;
// y-sweep: a cell is final 4 rows after it enters a line's stencil window
// (2 ghost rows + 2 cells of lag), so its outputs are stored in boxes of 4
// rows and row segments are multiples of 4 rows; the input boxes hold one or
// more such groups of rows.
constexpr int kYLag = 4;

// SoA plane set: field f (0 rho, 1 rhou, 2 rhov, 3 E), array row r, column c
// at base[f*plane + r*pitch + c].
template <class T> struct Planes {
    T* base;
    long long pitch;
    long long plane;
};

// Boundary kinds, as in include/euler2d.h.
enum { kBcTransmissive = 0, kBcReflective = 1 };

template <class T> struct SweepArgs {
    Planes<T> out;       // x-sweep: Utmp (interior at col+kTOff, row+2); y-sweep: Unew (col+kSOff, row+2)
    Ctl* ctl;
    int nx, ny;
    int seg;             // outputs per task along the march direction
    int nseg;            // tasks per line
    int ntasks;
    int bc_lo, bc_hi;    // x-sweep: bottom/top; y-sweep: left/right (ghost lines it writes)
    int out_index;       // y-sweep: index of the buffer it writes (becomes Ctl::cur)
    int finalize;        // y-sweep: 1 = advance t/step and compute the next dt
    int wclip;           // y-sweep: S columns >= wclip are stored directly (TMA stores clip at
                         // 16-byte granularity, so the store map ends on a 16-byte boundary)
    double d;            // dx (x-sweep) or dy (y-sweep); the step uses dt/d
    T* snap;             // x-sweep: snapshot storage, interior SoA [k][f][ny][nx]
    long long snap_plane, snap_stride;
};

// ---- ensemble (many independent grids in one persistent launch per step) ----
constexpr int kMaxInst = 256;

// One instance as the ensemble kernel sees it (device memory, 64-byte
// aligned for the tensor maps).
template <class T> struct EnsInst {
    CUtensorMap tm_x[2];   // x-sweep input, per state buffer
    CUtensorMap tm_xo;     // x-sweep output (Utmp)
    CUtensorMap tm_y;      // y-sweep input (Utmp)
    CUtensorMap tm_yo[2];  // y-sweep output, per state buffer
    SweepArgs<T> xa;       // x-sweep arguments
    SweepArgs<T> ya[2];    // y-sweep arguments writing state buffer b
};

// Work-list state of one launch: the dequeue counter and, per instance,
// the number of finished x-sweep tasks (reset before every launch).
struct EnsSched {
    unsigned int next;
    unsigned int pad[31];
    unsigned int xdone[kMaxInst];
};

template <class T> struct EnsArgs {
    const EnsInst<T>* inst;
    EnsSched* sched;
    int ninst;
    int total_x, total_y;
    int wait_extra;            // test hook: y tasks wait for this many x tasks more than exist
    int x_off[kMaxInst + 1];   // prefix sums of the instances' x-sweep tasks
    int y_off[kMaxInst + 1];   // ... and y-sweep tasks
};

using EnsembleLaunch = cudaError_t (*)(const void* args, int ctas, cudaStream_t s);

// Host-side launch entry of one sweep instantiation.
using SweepLaunch = cudaError_t (*)(const CUtensorMap* tm, const CUtensorMap* tm_out, const void* args,
                                    int ctas, cudaStream_t s);

using FirstOrderLaunch = cudaError_t (*)(const void* in, const void* out, int nx, int ny, double dtdx,
                                         double dtdy, cudaStream_t s);

struct SweepKernels {
    SweepLaunch x, y;
    FirstOrderLaunch first;  // first-order Godunov step (in/out: Planes<T>*)
    EnsembleLaunch ens;      // persistent ensemble step (args: EnsArgs<T>*)
    int (*occ_e)();          // resident CTAs per SM of the ensemble kernel
    int (*occ_x)();      // resident CTAs per SM of each kernel
    int (*occ_y)();
    int box_x;           // x-sweep box: box_x columns (32 bytes) x 32 rows, 32-byte swizzle
    int ry;              // y-sweep box: box_w_y columns x ry rows
    int box_w_y;
    int stages_x, stages_y;
    int nw;              // warps per CTA
    size_t smem_x, smem_y;
};

}  // namespace eu
