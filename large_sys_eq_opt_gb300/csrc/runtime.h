// runtime.h -- internals of the host runtime behind include/euler2d.h (not
// part of the C ABI): the handle and ensemble structures and the helpers the
// four runtime units share.
//   runtime.cpp      tensor maps, work decomposition, launches, control
//                    block, graphs, host transfers
//   api.cpp          the single-grid entry points
//   api_adjoint.cpp  checkpointed forward and adjoint sweeps (eu_adjoint_*)
//   api_batch.cpp    ensembles in one persistent launch (eu_batch_*)
#pragma once
#include <cudaTypedefs.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/euler2d.h"
#include "adjoint_kernels.h"
#include "aux_kernels.h"

namespace eu {
namespace __attribute__((visibility("hidden"))) rt {

// NVTX range for the duration of one ABI call (shows in Nsight timelines).
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
};

inline long long round_up(long long a, long long b) { return (a + b - 1) / b * b; }

}  // namespace rt
}  // namespace eu

struct eu_handle {
    eu_case cfg{};
    int prec = EU_FP64, solver = EU_HLL;
    int bc[4] = {0, 0, 0, 0};
    size_t esz = 8;
    double dx = 0, dy = 0;
    int sm_count = 152;
    cudaStream_t st = nullptr;
    long long pitch_s = 0, plane_s = 0, pitch_t = 0, plane_t = 0;
    void* S[2] = {nullptr, nullptr};
    void* Tm = nullptr;
    eu::Ctl* ctl = nullptr;   // device
    eu::Ctl* hctl = nullptr;  // pinned host mirror
    double* d_aos = nullptr;
    double* h_aos = nullptr;  // pinned staging for snapshots
    double* d_part = nullptr;
    double* d_tot = nullptr;
    double* h_tot = nullptr;
    int part_blocks = 1024;
    void* snap = nullptr;
    long long snap_plane = 0, snap_stride = 0;
    int snap_cap = 0;
    double* d_frozen = nullptr;
    long long frozen_cap = 0;
    double* d_dtlog = nullptr;
    long long dtlog_cap = 0;
    CUtensorMap tm_x[2];
    CUtensorMap tm_y;
    int tm_y_ry = 0;       // rows of tm_y's box: the y-sweep launch must expect exactly these (K.ry)
    CUtensorMap tm_xo;     // x-sweep output: Utmp boxes, rows [0, ny+2), columns [0, nx+kTOff)
    CUtensorMap tm_yo[2];  // y-sweep output: S boxes, columns [0, nx+kSOff) (right ghosts clipped)
    eu::SweepKernels K{};
    int seg_x = 0, nseg_x = 0, ntasks_x = 0, ctas_x = 0;
    int seg_y = 0, nseg_y = 0, ntasks_y = 0, ctas_y = 0;
    int cur = 0;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    int gsteps = 0;
    // TMA L2 promotion (bytes) of the sweep inputs.  The x-sweep's boxes are
    // 32-byte row pieces: promoting them to 128 B measured 1.5% faster than
    // 256 B at 8192^2 (64 B slower); the y-sweep is insensitive.
    int l2promo_x = 128, l2promo_y = 256;
    // Discrete adjoint (eu_adjoint_forward / eu_adjoint_backward): checkpoints
    // every k steps plus one segment of recomputed forward states.
    struct Adj {
        int k = 0, nseg = 0;
        long long nsteps = 0;
        std::vector<void*> ck;   // nseg+1 states: ck[s] = state after s*k steps
        std::vector<void*> R;    // k states: R[j] = state after s*k+j steps (j >= 1) of the ring segment
        std::vector<void*> Q;    // k x-sweep outputs of the ring segment
        std::vector<CUtensorMap> ck_x, ck_yo, R_x, R_yo, Q_xo, Q_y;
        int q_y_ry = 0;          // rows of the Q_y boxes (K.ry when they were encoded)
        void* lam = nullptr;     // adjoint of the state
        void* mu = nullptr;      // adjoint of the x-sweep output
        double* d_dts = nullptr;
        long long dts_cap = 0;
        std::vector<double> dts;
        eu::Ctl* hctl = nullptr;     // pinned control images, one per segment launch
        int hctl_cap = 0;
        int ring_seg = -1;
        bool ready = false;
        bool cfl = false;            // forward chose its dts (CFL, logged into d_dts)
        double t0 = 0.0;
        long long step0 = 0;
        cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};   // 4: cross-stream hand-off
        float ms_fwd = 0.f, ms_bwd = 0.f;
    } adj;
    std::string err;
};

// Ensemble of independent grids advanced by one persistent launch per step.
struct eu_batch {
    int n = 0, prec = EU_FP32, solver = EU_HLLC;
    std::vector<eu_handle*> h;   // one handle per instance (state, maps, control block)
    cudaStream_t st = nullptr;
    eu::SweepKernels K{};
    void* d_inst = nullptr;      // EnsInst<T>[n]
    eu::EnsSched* d_sched = nullptr;
    std::vector<unsigned char> args;   // host image of EnsArgs<T>
    int ctas = 0;
    bool dirty = true;
    cudaGraphExec_t g = nullptr;
    int gsteps = 0;
    int wait_extra = 0;
    void* d_adj = nullptr;       // descriptors of the shared adjoint launches
    size_t adj_cap = 0;
    cudaEvent_t adj_ev = nullptr;
    std::string err;
};

namespace eu {
namespace __attribute__((visibility("hidden"))) rt {

extern thread_local std::string g_err;   // eu_last_error(NULL)

SweepKernels kernels_for(int prec, int solver);

// Error reporting: record the message on the handle (or the thread) and
// return the status code.
int fail(eu_handle* h, int code, const std::string& msg);
int cuda_fail(eu_handle* h, cudaError_t e, const char* what);
int bfail(eu_batch* b, int code, const std::string& msg);

#define EU_CUDA(h, call)                                        \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return cuda_fail((h), e_, #call); \
    } while (0)

template <class T> Planes<T> planes_s(const eu_handle* h, int b) {
    return Planes<T>{static_cast<T*>(h->S[b]), h->pitch_s, h->plane_s};
}

template <class T> Planes<T> planes_t(const eu_handle* h) {
    return Planes<T>{static_cast<T*>(h->Tm), h->pitch_t, h->plane_t};
}

// Tensor maps and work decomposition.
int encode(eu_handle* h, CUtensorMap* m, void* base, long long width, long long pitch, long long plane,
           int box_w, int box_h, CUtensorMapSwizzle swz, int promo, long long height = -1);
long long wclip_of(const eu_handle* h);
int encode_all(eu_handle* h);
void plan(eu_handle* h);

template <class T> SweepArgs<T> x_args(const eu_handle* h, int cur) {
    SweepArgs<T> a{};
    a.out = planes_t<T>(h);
    a.ctl = h->ctl;
    a.nx = h->cfg.nx;
    a.ny = h->cfg.ny;
    a.seg = h->seg_x;
    a.nseg = h->nseg_x;
    a.ntasks = h->ntasks_x;
    a.bc_lo = h->bc[EU_SIDE_BOTTOM];
    a.bc_hi = h->bc[EU_SIDE_TOP];
    a.out_index = cur;
    a.finalize = 0;
    a.d = h->dx;
    a.snap = static_cast<T*>(h->snap);
    a.snap_plane = h->snap_plane;
    a.snap_stride = h->snap_stride;
    return a;
}

template <class T> SweepArgs<T> y_args(const eu_handle* h, int cur) {
    SweepArgs<T> a{};
    a.out = planes_s<T>(h, 1 - cur);
    a.ctl = h->ctl;
    a.nx = h->cfg.nx;
    a.ny = h->cfg.ny;
    a.seg = h->seg_y;
    a.nseg = h->nseg_y;
    a.ntasks = h->ntasks_y;
    a.bc_lo = h->bc[EU_SIDE_LEFT];
    a.bc_hi = h->bc[EU_SIDE_RIGHT];
    a.out_index = 1 - cur;
    a.finalize = 1;
    a.wclip = (int)wclip_of(h);
    a.d = h->dy;
    return a;
}

// Launches on the handle's stream.
cudaError_t launch_x(eu_handle* h, int cur);
cudaError_t launch_y(eu_handle* h, int cur);
cudaError_t launch_step(eu_handle* h, int cur);
cudaError_t launch_dt(eu_handle* h, int b);
cudaError_t unpack_state(eu_handle* h, int b, double* d_aos);
cudaError_t unpack_tmp(eu_handle* h, double* d_aos);
cudaError_t fill_ghosts(eu_handle* h, int b);
cudaError_t pack_state(eu_handle* h, int b, const double* d_aos);

// Sizes, control block, graphs, host transfers.
long long aos_bytes(const eu_handle* h);
size_t state_bytes(const eu_handle* h);
size_t tmp_bytes(const eu_handle* h);
void ctl_reset(eu_handle* h, int mode, double t_end, long long max_steps);
int ctl_push(eu_handle* h);
int ctl_pull_sync(eu_handle* h);
int status_code(eu_handle* h);
int graph_for(eu_handle* h, int cur, cudaGraphExec_t* out);
void drop_graphs(eu_handle* h);
int ensure_aos(eu_handle* h);
int ensure_snapshots(eu_handle* h, int nsnap);
int upload_to(eu_handle* h, int b, const double* aos);
int download_from_state(eu_handle* h, int b, double* aos);

// Discrete adjoint (api_adjoint.cpp).
void adj_free(eu_handle* h);
constexpr int kMaxCkptK = 1024;
template <class T> EnsInst<T> adj_ens_inst(const eu_handle* h, long long n);
int adj_fwd_setup(eu_handle* h, long long nsteps, const double* dts, int ckpt_k, double t_end);
int adj_fwd_done(eu_handle* h);
int adj_fwd_steps(eu_handle* h);
int adj_auto_k(eu_handle* const* hs, const long long* nsteps, int n);
int adj_fwd_enqueue(eu_handle* h, long long nsteps, const double* dts, int ckpt_k, double t_end);
int adj_fwd_finish(eu_handle* h);
int adj_bwd_enqueue(eu_handle* h, const double* dJ_dUN, double* dJ_dU0);
int adj_bwd_sweeps(eu_handle* h);
int adj_bwd_finish(eu_handle* h, double* dJ_dU0);

// Ensembles (api_batch.cpp).
int batch_build(eu_batch* b);
cudaError_t batch_launch(eu_batch* b);
int batch_graph(eu_batch* b, int steps, cudaGraphExec_t* out);
int batch_pull(eu_batch* b, int* all_done);

}  // namespace rt

// Message for eu_last_error(NULL), for entry points defined in other units.
void set_global_error(const char* msg);

}  // namespace eu
