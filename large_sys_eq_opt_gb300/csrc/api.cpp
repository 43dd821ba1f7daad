// api.cpp -- host runtime behind include/euler2d.h.
//
// One handle owns: two SoA state buffers (S0/S1, ping-pong), the x-sweep
// output buffer Utmp, the device control block (Ctl), three TMA descriptors
// (S0 and S1 boxed for the x-sweep, Utmp boxed for the y-sweep), a CUDA
// stream, and lazily built CUDA graphs of whole steps.  The host never
// touches a state value on the hot path: dt, t_end clipping and the snapshot
// schedule live in Ctl and are advanced by the y-sweep's last warp.
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

using namespace eu;

namespace {

thread_local std::string g_err;

// NVTX range for the duration of one ABI call (shows in Nsight timelines).
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
};

long long round_up(long long a, long long b) { return (a + b - 1) / b * b; }

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }();
    return fn;
}

SweepKernels kernels_for(int prec, int solver) {
    if (prec == EU_FP32) {
        switch (solver) {
            case EU_HLLC: return sweep_kernels_32_1();
            case EU_EXACT: return sweep_kernels_32_2();
            case EU_FORCE: return sweep_kernels_32_3();
            default: return sweep_kernels_32_0();
        }
    }
    switch (solver) {
        case EU_HLLC: return sweep_kernels_64_1();
        case EU_EXACT: return sweep_kernels_64_2();
        case EU_FORCE: return sweep_kernels_64_3();
        default: return sweep_kernels_64_0();
    }
}

}  // namespace

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
    Ctl* ctl = nullptr;   // device
    Ctl* hctl = nullptr;  // pinned host mirror
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
    CUtensorMap tm_xo;     // x-sweep output: Utmp boxes, rows [0, ny+2), columns [0, nx+kTOff)
    CUtensorMap tm_yo[2];  // y-sweep output: S boxes, columns [0, nx+kSOff) (right ghosts clipped)
    SweepKernels K{};
    int seg_x = 0, nseg_x = 0, ntasks_x = 0, ctas_x = 0;
    int seg_y = 0, nseg_y = 0, ntasks_y = 0, ctas_y = 0;
    int cur = 0;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    int gsteps = 0;
    int l2promo_x = 256, l2promo_y = 256;   // TMA L2 promotion (bytes) of the sweep inputs
    // Discrete adjoint (eu_adjoint_forward / eu_adjoint_backward): checkpoints
    // every k steps plus one segment of recomputed forward states.
    struct Adj {
        int k = 0, nseg = 0;
        long long nsteps = 0;
        std::vector<void*> ck;   // nseg+1 states: ck[s] = state after s*k steps
        std::vector<void*> R;    // k states: R[j] = state after s*k+j steps (j >= 1) of the ring segment
        std::vector<void*> Q;    // k x-sweep outputs of the ring segment
        std::vector<CUtensorMap> ck_x, ck_yo, R_x, R_yo, Q_xo, Q_y;
        void* lam = nullptr;     // adjoint of the state
        void* mu = nullptr;      // adjoint of the x-sweep output
        double* d_dts = nullptr;
        long long dts_cap = 0;
        std::vector<double> dts;
        Ctl* hctl = nullptr;     // pinned control images, one per segment launch
        int hctl_cap = 0;
        int ring_seg = -1;
        bool ready = false;
        double t0 = 0.0;
        long long step0 = 0;
        cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
        float ms_fwd = 0.f, ms_bwd = 0.f;
    } adj;
    std::string err;
};

// Ensemble of independent grids advanced by one persistent launch per step.
struct eu_batch {
    int n = 0, prec = EU_FP32, solver = EU_HLLC;
    std::vector<eu_handle*> h;   // one handle per instance (state, maps, control block)
    cudaStream_t st = nullptr;
    SweepKernels K{};
    void* d_inst = nullptr;      // EnsInst<T>[n]
    EnsSched* d_sched = nullptr;
    std::vector<unsigned char> args;   // host image of EnsArgs<T>
    int ctas = 0;
    bool dirty = true;
    cudaGraphExec_t g = nullptr;
    int gsteps = 0;
    int wait_extra = 0;
    std::string err;
};

namespace {

int fail(eu_handle* h, int code, const std::string& msg) {
    // A failed runtime call (e.g. an allocation) stays the thread's "last
    // error" until read; clear it so that the next launch check of any
    // handle does not report it again.
    (void)cudaGetLastError();
    if (h) h->err = msg;
    else g_err = msg;
    return code;
}

int cuda_fail(eu_handle* h, cudaError_t e, const char* what) {
    return fail(h, e == cudaErrorMemoryAllocation ? EU_ERR_NOMEM : EU_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

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

CUtensorMapL2promotion promo_of(int bytes) {
    switch (bytes) {
        case 0: return CU_TENSOR_MAP_L2_PROMOTION_NONE;
        case 64: return CU_TENSOR_MAP_L2_PROMOTION_L2_64B;
        case 128: return CU_TENSOR_MAP_L2_PROMOTION_L2_128B;
        default: return CU_TENSOR_MAP_L2_PROMOTION_L2_256B;
    }
}

int encode(eu_handle* h, CUtensorMap* m, void* base, long long width, long long pitch, long long plane,
           int box_w, int box_h, CUtensorMapSwizzle swz, int promo, long long height = -1) {
    auto fn = encode_fn();
    if (!fn) return fail(h, EU_ERR_CUDA, "cuTensorMapEncodeTiled entry point unavailable");
    const cuuint64_t dims[3] = {(cuuint64_t)width, (cuuint64_t)(height > 0 ? height : h->cfg.ny + 4), 4};
    const cuuint64_t strides[2] = {(cuuint64_t)(pitch * h->esz), (cuuint64_t)(plane * h->esz)};
    const cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)box_h, 4};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = fn(m, h->prec == EU_FP32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                          3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          swz, promo_of(promo),
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(h, EU_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return EU_OK;
}

// Width of the y-sweep store map: the interior's end (column nx+kSOff)
// rounded down to 16 bytes, because TMA stores clip at that granularity and
// must not reach the right ghost columns.
long long wclip_of(const eu_handle* h) {
    const long long per16 = 16 / (long long)h->esz;
    return std::max<long long>((h->cfg.nx + kSOff) / per16 * per16, per16);
}

int encode_all(eu_handle* h) {
    for (int b = 0; b < 2; ++b)
        if (int rc = encode(h, &h->tm_x[b], h->S[b], h->cfg.nx + kSOff + 2, h->pitch_s, h->plane_s, h->K.box_x, 32,
                            CU_TENSOR_MAP_SWIZZLE_32B, h->l2promo_x))
            return rc;
    // x-sweep stores: width nx+4 and height ny+2 clip everything past the
    // last interior column / row, so no box spills into the top ghost rows.
    if (int rc = encode(h, &h->tm_xo, h->Tm, h->cfg.nx + kTOff, h->pitch_t, h->plane_t, h->K.box_x, 32,
                        CU_TENSOR_MAP_SWIZZLE_32B, 256, h->cfg.ny + 2))
        return rc;
    for (int b = 0; b < 2; ++b)
        if (int rc = encode(h, &h->tm_yo[b], h->S[b], wclip_of(h), h->pitch_s, h->plane_s, 32, h->K.ry,
                            CU_TENSOR_MAP_SWIZZLE_NONE, 256))
            return rc;
    return encode(h, &h->tm_y, h->Tm, h->pitch_t, h->pitch_t, h->plane_t, h->K.box_w_y, h->K.ry,
                  CU_TENSOR_MAP_SWIZZLE_NONE, h->l2promo_y);
}

// Work decomposition.  Every warp is one task: a segment of one group of 32
// lines.  Measured on GB300 (8192^2 and 2048^2, FP32 HLLC), launches of many
// short tasks beat near-single-wave launches of long ones even though each
// task recomputes a 4-cell warm-up (plus one box in the x-sweep): CTAs refill
// the SMs as they retire, the tail shrinks to one short task, and fewer
// lines are in flight at once.  The default aims at about eight tasks per
// resident warp slot with segments clamped to [32, 128] rows (y) and
// [32, 256] columns (x); eu_set_option overrides it.
void plan(eu_handle* h) {
    const int nx = h->cfg.nx, ny = h->cfg.ny;
    const long long slots_x = (long long)h->sm_count * h->K.nw * h->K.occ_x();
    const long long slots_y = (long long)h->sm_count * h->K.nw * h->K.occ_y();
    const int CX = h->K.box_x;
    const int rgroups = (ny + 31) / 32;
    long long want = ((long long)rgroups * nx + 8 * slots_x - 1) / (8 * slots_x);
    want = std::min<long long>(std::max<long long>(want, 32), 256);
    int seg = (int)round_up(std::min<long long>(want, nx), CX);
    h->seg_x = seg;
    h->nseg_x = (nx + seg - 1) / seg;
    h->ntasks_x = rgroups * h->nseg_x;
    h->ctas_x = (h->ntasks_x + h->K.nw - 1) / h->K.nw;
    const int groups = (nx + kSOff + 31) / 32;
    want = ((long long)groups * ny + 8 * slots_y - 1) / (8 * slots_y);
    want = std::min<long long>(std::max<long long>(want, 32), 128);
    h->seg_y = (int)round_up(std::min<long long>(want, ny), h->K.ry);  // whole output boxes
    h->nseg_y = groups;  // tasks per row segment
    h->ntasks_y = groups * ((ny + h->seg_y - 1) / h->seg_y);
    h->ctas_y = (h->ntasks_y + h->K.nw - 1) / h->K.nw;
}

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

cudaError_t launch_x(eu_handle* h, int cur) {
    if (h->prec == EU_FP32) {
        const SweepArgs<float> a = x_args<float>(h, cur);
        return h->K.x(&h->tm_x[cur], &h->tm_xo, &a, h->ctas_x, h->st);
    }
    const SweepArgs<double> a = x_args<double>(h, cur);
    return h->K.x(&h->tm_x[cur], &h->tm_xo, &a, h->ctas_x, h->st);
}

cudaError_t launch_y(eu_handle* h, int cur) {
    if (h->prec == EU_FP32) {
        const SweepArgs<float> a = y_args<float>(h, cur);
        return h->K.y(&h->tm_y, &h->tm_yo[1 - cur], &a, h->ctas_y, h->st);
    }
    const SweepArgs<double> a = y_args<double>(h, cur);
    return h->K.y(&h->tm_y, &h->tm_yo[1 - cur], &a, h->ctas_y, h->st);
}

cudaError_t launch_step(eu_handle* h, int cur) {
    cudaError_t e = launch_x(h, cur);
    if (e != cudaSuccess) return e;
    return launch_y(h, cur);
}

cudaError_t launch_dt(eu_handle* h, int b) {
    if (h->prec == EU_FP32) return eu::launch_dt<float>(planes_s<float>(h, b), h->cfg.nx, h->cfg.ny, h->ctl, h->st);
    return eu::launch_dt<double>(planes_s<double>(h, b), h->cfg.nx, h->cfg.ny, h->ctl, h->st);
}

cudaError_t unpack_state(eu_handle* h, int b, double* d_aos) {
    if (h->prec == EU_FP32)
        return launch_unpack_aos<float>(planes_s<float>(h, b), kSOff, h->cfg.nx, h->cfg.ny, h->bc, d_aos, h->st);
    return launch_unpack_aos<double>(planes_s<double>(h, b), kSOff, h->cfg.nx, h->cfg.ny, h->bc, d_aos, h->st);
}

cudaError_t unpack_tmp(eu_handle* h, double* d_aos) {
    if (h->prec == EU_FP32)
        return launch_unpack_aos<float>(planes_t<float>(h), kTOff, h->cfg.nx, h->cfg.ny, h->bc, d_aos, h->st);
    return launch_unpack_aos<double>(planes_t<double>(h), kTOff, h->cfg.nx, h->cfg.ny, h->bc, d_aos, h->st);
}

cudaError_t fill_ghosts(eu_handle* h, int b) {
    if (h->prec == EU_FP32) return launch_fill_ghosts<float>(planes_s<float>(h, b), h->cfg.nx, h->cfg.ny, h->bc, h->st);
    return launch_fill_ghosts<double>(planes_s<double>(h, b), h->cfg.nx, h->cfg.ny, h->bc, h->st);
}

cudaError_t pack_state(eu_handle* h, int b, const double* d_aos) {
    if (h->prec == EU_FP32) return launch_pack_aos<float>(d_aos, planes_s<float>(h, b), h->cfg.nx, h->cfg.ny, h->st);
    return launch_pack_aos<double>(d_aos, planes_s<double>(h, b), h->cfg.nx, h->cfg.ny, h->st);
}

long long aos_bytes(const eu_handle* h) { return 32LL * (h->cfg.nx + 4) * (h->cfg.ny + 4); }

// Control block defaults for a fresh sequence of steps.
void ctl_reset(eu_handle* h, int mode, double t_end, long long max_steps) {
    Ctl& c = *h->hctl;
    std::memset(&c, 0, sizeof(Ctl));
    c.t = 0.0;
    c.dt = 0.0;
    c.t_end = t_end;
    c.cfl_dmin = h->cfg.cfl * std::min(h->dx, h->dy);
    c.mode = mode;
    c.max_steps = max_steps;
    c.cur = h->cur;
    c.dt_log = h->d_dtlog;
    c.dt_log_cap = h->dtlog_cap;
}

int ctl_push(eu_handle* h) {
    EU_CUDA(h, cudaMemcpyAsync(h->ctl, h->hctl, sizeof(Ctl), cudaMemcpyHostToDevice, h->st));
    return EU_OK;
}

int ctl_pull_sync(eu_handle* h) {
    EU_CUDA(h, cudaMemcpyAsync(h->hctl, h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    h->cur = h->hctl->cur;
    return EU_OK;
}

int status_code(eu_handle* h) {
    const int s = h->hctl->status;
    if (s & kStatusTimeout) return fail(h, EU_ERR_TIMEOUT, "a bounded device wait expired");
    if (s & kStatusNonPhysical) return fail(h, EU_ERR_NONPHYSICAL, "compute_dt: non-positive maximum wave speed.");
    return EU_OK;
}

// Graph of `steps` consecutive steps starting from buffer `cur`.
int build_graph(eu_handle* h, int cur, int steps, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    EU_CUDA(h, cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (int s = 0; s < steps && e == cudaSuccess; ++s) e = launch_step(h, (cur + s) & 1);
    cudaError_t e2 = cudaStreamEndCapture(h->st, &g);
    if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(h, e, "step capture"); }
    if (e2 != cudaSuccess) return cuda_fail(h, e2, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaGraphInstantiate");
    return EU_OK;
}

int graph_for(eu_handle* h, int cur, cudaGraphExec_t* out) {
    if (!h->gexec[cur]) {
        int rc = build_graph(h, cur, h->gsteps, &h->gexec[cur]);
        if (rc) return rc;
    }
    *out = h->gexec[cur];
    return EU_OK;
}

void drop_graphs(eu_handle* h) {
    for (auto& g : h->gexec)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}

int ensure_aos(eu_handle* h) {
    if (!h->d_aos) EU_CUDA(h, cudaMalloc(&h->d_aos, aos_bytes(h)));
    return EU_OK;
}

int ensure_snapshots(eu_handle* h, int nsnap) {
    if (nsnap <= h->snap_cap) return EU_OK;
    if (h->snap) { cudaFree(h->snap); h->snap = nullptr; h->snap_cap = 0; }
    h->snap_plane = (long long)h->cfg.nx * h->cfg.ny;
    h->snap_stride = 4 * h->snap_plane;
    EU_CUDA(h, cudaMalloc(&h->snap, (size_t)nsnap * h->snap_stride * h->esz));
    h->snap_cap = nsnap;
    drop_graphs(h);  // graphs bake the snapshot pointer into the x-sweep args
    if (!h->h_aos) EU_CUDA(h, cudaMallocHost(&h->h_aos, aos_bytes(h)));
    return ensure_aos(h);
}

int upload_to(eu_handle* h, int b, const double* aos) {
    int rc = ensure_aos(h);
    if (rc) return rc;
    EU_CUDA(h, cudaMemcpyAsync(h->d_aos, aos, aos_bytes(h), cudaMemcpyHostToDevice, h->st));
    EU_CUDA(h, pack_state(h, b, h->d_aos));
    return EU_OK;
}

int download_from_state(eu_handle* h, int b, double* aos) {
    int rc = ensure_aos(h);
    if (rc) return rc;
    EU_CUDA(h, unpack_state(h, b, h->d_aos));
    EU_CUDA(h, cudaMemcpyAsync(aos, h->d_aos, aos_bytes(h), cudaMemcpyDeviceToHost, h->st));
    return EU_OK;
}

// ---------------------------------------------------------------------------
// discrete adjoint: buffers, forward segments, adjoint sweeps
// ---------------------------------------------------------------------------
AdjLaunch adj_launcher(int prec, int solver) {
    static const AdjLaunch f32[4] = {adjoint_sweep_32_0, adjoint_sweep_32_1, adjoint_sweep_32_2, adjoint_sweep_32_3};
    static const AdjLaunch f64[4] = {adjoint_sweep_64_0, adjoint_sweep_64_1, adjoint_sweep_64_2, adjoint_sweep_64_3};
    return prec == EU_FP32 ? f32[solver] : f64[solver];
}

size_t state_bytes(const eu_handle* h) { return (size_t)(4 * h->plane_s) * h->esz; }
size_t tmp_bytes(const eu_handle* h) { return (size_t)(4 * h->plane_t) * h->esz; }

// TMA maps of a state buffer (x-sweep input, y-sweep output) and of an
// x-sweep output buffer (x-sweep output, y-sweep input), as encode_all.
int enc_state(eu_handle* h, void* b, CUtensorMap* xin, CUtensorMap* yout) {
    if (int rc = encode(h, xin, b, h->cfg.nx + kSOff + 2, h->pitch_s, h->plane_s, h->K.box_x, 32,
                        CU_TENSOR_MAP_SWIZZLE_32B, h->l2promo_x))
        return rc;
    return encode(h, yout, b, wclip_of(h), h->pitch_s, h->plane_s, 32, h->K.ry, CU_TENSOR_MAP_SWIZZLE_NONE, 256);
}
int enc_tmp(eu_handle* h, void* b, CUtensorMap* xout, CUtensorMap* yin) {
    if (int rc = encode(h, xout, b, h->cfg.nx + kTOff, h->pitch_t, h->plane_t, h->K.box_x, 32,
                        CU_TENSOR_MAP_SWIZZLE_32B, 256, h->cfg.ny + 2))
        return rc;
    return encode(h, yin, b, h->pitch_t, h->pitch_t, h->plane_t, h->K.box_w_y, h->K.ry, CU_TENSOR_MAP_SWIZZLE_NONE,
                  h->l2promo_y);
}

void adj_free(eu_handle* h) {
    auto& A = h->adj;
    for (void* p : A.ck) cudaFree(p);
    for (void* p : A.R) cudaFree(p);
    for (void* p : A.Q) cudaFree(p);
    A.ck.clear(); A.R.clear(); A.Q.clear();
    A.ck_x.clear(); A.ck_yo.clear(); A.R_x.clear(); A.R_yo.clear(); A.Q_xo.clear(); A.Q_y.clear();
    cudaFree(A.lam); cudaFree(A.mu); cudaFree(A.d_dts);
    A.lam = A.mu = nullptr;
    A.d_dts = nullptr;
    A.dts_cap = 0;
    cudaFreeHost(A.hctl);
    A.hctl = nullptr;
    A.hctl_cap = 0;
    for (auto& e : A.ev)
        if (e) { cudaEventDestroy(e); e = nullptr; }
    A.k = A.nseg = 0;
    A.ready = false;
    A.ring_seg = -1;
}

int adj_alloc_buf(eu_handle* h, size_t bytes, void** p) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, bytes, h->st);
    if (e != cudaSuccess) return fail(h, EU_ERR_NOMEM, std::string("adjoint buffers: ") + cudaGetErrorString(e));
    return EU_OK;
}

// Buffers for nsteps steps with checkpoints every k steps.
int adj_prepare(eu_handle* h, long long nsteps, int k) {
    auto& A = h->adj;
    const int nseg = (int)((nsteps + k - 1) / k);
    if (A.k != k || A.nseg < nseg) {
        EU_CUDA(h, cudaStreamSynchronize(h->st));
        adj_free(h);
        A.ck.assign(nseg + 1, nullptr);
        A.R.assign(k, nullptr);
        A.Q.assign(k, nullptr);
        A.ck_x.resize(nseg + 1); A.ck_yo.resize(nseg + 1);
        A.R_x.resize(k); A.R_yo.resize(k);
        A.Q_xo.resize(k); A.Q_y.resize(k);
        for (int i = 0; i <= nseg; ++i) {
            if (int rc = adj_alloc_buf(h, state_bytes(h), &A.ck[i])) return rc;
            if (int rc = enc_state(h, A.ck[i], &A.ck_x[i], &A.ck_yo[i])) return rc;
        }
        for (int j = 1; j < k; ++j) {
            if (int rc = adj_alloc_buf(h, state_bytes(h), &A.R[j])) return rc;
            if (int rc = enc_state(h, A.R[j], &A.R_x[j], &A.R_yo[j])) return rc;
        }
        for (int j = 0; j < k; ++j) {
            if (int rc = adj_alloc_buf(h, tmp_bytes(h), &A.Q[j])) return rc;
            if (int rc = enc_tmp(h, A.Q[j], &A.Q_xo[j], &A.Q_y[j])) return rc;
        }
        if (int rc = adj_alloc_buf(h, state_bytes(h), &A.lam)) return rc;
        if (int rc = adj_alloc_buf(h, state_bytes(h), &A.mu)) return rc;
        for (auto& e : A.ev) EU_CUDA(h, cudaEventCreate(&e));
        A.k = k;
        A.nseg = nseg;
    }
    A.nseg = nseg;
    if (nsteps > A.dts_cap) {
        cudaFree(A.d_dts);
        A.d_dts = nullptr;
        A.dts_cap = 0;
        EU_CUDA(h, cudaMalloc(&A.d_dts, sizeof(double) * (size_t)nsteps));
        A.dts_cap = nsteps;
    }
    if (A.hctl_cap < nseg + 1) {
        EU_CUDA(h, cudaStreamSynchronize(h->st));
        cudaFreeHost(A.hctl);
        A.hctl = nullptr;
        A.hctl_cap = 0;
        EU_CUDA(h, cudaMallocHost(&A.hctl, sizeof(Ctl) * (size_t)(nseg + 1)));
        A.hctl_cap = nseg + 1;
    }
    A.nsteps = nsteps;
    return EU_OK;
}

// Forward steps s*k .. s*k+len-1 from ck[s] with the frozen dts: the x-sweep
// of step j writes Q[j], the y-sweep writes R[j+1] (ck[s+1] for the last).
template <class T> cudaError_t adj_segment_t(eu_handle* h, int s) {
    auto& A = h->adj;
    const long long n0 = (long long)s * A.k;
    const int len = (int)std::min<long long>(A.k, A.nsteps - n0);
    Ctl& c = A.hctl[s];
    std::memset(&c, 0, sizeof(Ctl));
    c.t_end = INFINITY;
    c.cfl_dmin = h->cfg.cfl * std::min(h->dx, h->dy);
    c.mode = kModeFrozen;
    c.frozen = A.d_dts;
    c.n_frozen = A.nsteps;
    c.frozen_base = 0;
    c.step = n0;
    c.dt = A.dts[n0];
    c.max_steps = LLONG_MAX;
    cudaError_t e = cudaMemcpyAsync(h->ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, h->st);
    for (int j = 0; j < len && e == cudaSuccess; ++j) {
        SweepArgs<T> ax = x_args<T>(h, 0);
        ax.out = Planes<T>{static_cast<T*>(A.Q[j]), h->pitch_t, h->plane_t};
        ax.snap = nullptr;
        const CUtensorMap* xin = j == 0 ? &A.ck_x[s] : &A.R_x[j];
        e = h->K.x(xin, &A.Q_xo[j], &ax, h->ctas_x, h->st);
        if (e != cudaSuccess) break;
        const bool last = j == len - 1;
        void* dst = last ? A.ck[s + 1] : A.R[j + 1];
        SweepArgs<T> ay = y_args<T>(h, 0);
        ay.out = Planes<T>{static_cast<T*>(dst), h->pitch_s, h->plane_s};
        ay.out_index = 0;
        e = h->K.y(&A.Q_y[j], last ? &A.ck_yo[s + 1] : &A.R_yo[j + 1], &ay, h->ctas_y, h->st);
    }
    return e;
}
cudaError_t adj_segment(eu_handle* h, int s) {
    return h->prec == EU_FP32 ? adj_segment_t<float>(h, s) : adj_segment_t<double>(h, s);
}

// Adjoint of step n = s*k + j (the ring holds segment s): y-sweep adjoint
// lam -> mu on the x-sweep output Q[j], then x-sweep adjoint mu -> lam on the
// step's input state.
cudaError_t adj_step(eu_handle* h, int s, int j) {
    auto& A = h->adj;
    const long long n = (long long)s * A.k + j;
    const AdjLaunch L = adj_launcher(h->prec, h->solver);
    AdjSweepArgs y{};
    y.P = A.Q[j]; y.p_pitch = h->pitch_t; y.p_plane = h->plane_t; y.p_coff = kTOff;
    y.A = A.lam; y.a_pitch = h->pitch_s; y.a_plane = h->plane_s; y.a_coff = kSOff;
    y.G = A.mu; y.g_pitch = h->pitch_s; y.g_plane = h->plane_s; y.g_coff = kSOff;
    y.nx = h->cfg.nx; y.ny = h->cfg.ny;
    y.lam_d = A.dts[n] / h->dy;
    y.bc_lo = h->bc[EU_SIDE_BOTTOM]; y.bc_hi = h->bc[EU_SIDE_TOP];
    cudaError_t e = L(1, y, h->st);
    if (e != cudaSuccess) return e;
    AdjSweepArgs x{};
    x.P = j == 0 ? A.ck[s] : A.R[j]; x.p_pitch = h->pitch_s; x.p_plane = h->plane_s; x.p_coff = kSOff;
    x.A = A.mu; x.a_pitch = h->pitch_s; x.a_plane = h->plane_s; x.a_coff = kSOff;
    x.G = A.lam; x.g_pitch = h->pitch_s; x.g_plane = h->plane_s; x.g_coff = kSOff;
    x.nx = h->cfg.nx; x.ny = h->cfg.ny;
    x.lam_d = A.dts[n] / h->dx;
    x.bc_lo = h->bc[EU_SIDE_LEFT]; x.bc_hi = h->bc[EU_SIDE_RIGHT];
    return L(0, x, h->st);
}

// Enqueue the checkpointed forward on the handle's stream (no host wait).
int adj_fwd_enqueue(eu_handle* h, long long nsteps, const double* dts, int ckpt_k) {
    if (!h) return fail(nullptr, EU_ERR_INVALID, "null handle");
    if (nsteps < 1 || !dts) return fail(h, EU_ERR_INVALID, "eu_adjoint_forward: need nsteps >= 1 and a dt list");
    if (ckpt_k < 1 || ckpt_k > 1024) return fail(h, EU_ERR_INVALID, "eu_adjoint_forward: ckpt_k must be in [1, 1024]");
    if (h->cfg.nx < 2 || h->cfg.ny < 2) return fail(h, EU_ERR_INVALID, "eu_adjoint_forward: the adjoint needs nx, ny >= 2");
    for (long long i = 0; i < nsteps; ++i)
        if (!(dts[i] > 0.0) || !(dts[i] < INFINITY))
            return fail(h, EU_ERR_INVALID, "eu_adjoint_forward: every dt must be positive and finite");
    auto& A = h->adj;
    A.ready = false;
    if (int rc = adj_prepare(h, nsteps, ckpt_k)) return rc;
    A.dts.assign(dts, dts + nsteps);
    A.t0 = h->hctl->t;
    A.step0 = h->hctl->step;
    EU_CUDA(h, cudaMemcpyAsync(A.d_dts, A.dts.data(), sizeof(double) * (size_t)nsteps, cudaMemcpyHostToDevice, h->st));
    EU_CUDA(h, fill_ghosts(h, h->cur));   // scripts/cpu/main_cpu.cpp:222
    EU_CUDA(h, cudaMemcpyAsync(A.ck[0], h->S[h->cur], state_bytes(h), cudaMemcpyDeviceToDevice, h->st));
    EU_CUDA(h, cudaEventRecord(A.ev[0], h->st));
    for (int s = 0; s < A.nseg; ++s) EU_CUDA(h, adj_segment(h, s));
    EU_CUDA(h, cudaEventRecord(A.ev[1], h->st));
    A.ring_seg = A.nseg - 1;
    EU_CUDA(h, cudaMemcpyAsync(h->S[h->cur], A.ck[A.nseg], state_bytes(h), cudaMemcpyDeviceToDevice, h->st));
    EU_CUDA(h, cudaMemcpyAsync(&A.hctl[A.nseg], h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
    return EU_OK;
}

// Wait for the forward; status, timing, the handle's time and step.
int adj_fwd_finish(eu_handle* h) {
    auto& A = h->adj;
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    EU_CUDA(h, cudaEventElapsedTime(&A.ms_fwd, A.ev[0], A.ev[1]));
    const Ctl probe = A.hctl[A.nseg];
    double t = A.t0;
    for (double d : A.dts) t += d;
    ctl_reset(h, kModeHost, INFINITY, LLONG_MAX);
    h->hctl->t = t;
    h->hctl->step = A.step0 + A.nsteps;
    if (int rc = ctl_push(h)) return rc;
    if (probe.status & kStatusTimeout) return fail(h, EU_ERR_TIMEOUT, "a bounded device wait expired");
    if (probe.status & kStatusNonFinite) return fail(h, EU_ERR_NONPHYSICAL, "non-finite state in the forward steps");
    A.ready = true;
    return EU_OK;
}

int adj_bwd_enqueue(eu_handle* h, const double* dJ_dUN, double* dJ_dU0) {
    if (!h) return fail(nullptr, EU_ERR_INVALID, "null handle");
    if (!dJ_dUN || !dJ_dU0) return fail(h, EU_ERR_INVALID, "eu_adjoint_backward: null argument");
    auto& A = h->adj;
    if (!A.ready) return fail(h, EU_ERR_STATE, "eu_adjoint_backward: call eu_adjoint_forward first");
    if (int rc = ensure_aos(h)) return rc;
    EU_CUDA(h, cudaMemcpyAsync(h->d_aos, dJ_dUN, aos_bytes(h), cudaMemcpyHostToDevice, h->st));
    if (h->prec == EU_FP32) EU_CUDA(h, launch_pack_aos<float>(h->d_aos, Planes<float>{static_cast<float*>(A.lam), h->pitch_s, h->plane_s}, h->cfg.nx, h->cfg.ny, h->st));
    else EU_CUDA(h, launch_pack_aos<double>(h->d_aos, Planes<double>{static_cast<double*>(A.lam), h->pitch_s, h->plane_s}, h->cfg.nx, h->cfg.ny, h->st));
    EU_CUDA(h, cudaEventRecord(A.ev[2], h->st));
    for (int s = A.nseg - 1; s >= 0; --s) {
        if (A.ring_seg != s) {
            EU_CUDA(h, adj_segment(h, s));
            A.ring_seg = s;
        }
        const int len = (int)std::min<long long>(A.k, A.nsteps - (long long)s * A.k);
        for (int j = len - 1; j >= 0; --j) EU_CUDA(h, adj_step(h, s, j));
    }
    EU_CUDA(h, cudaEventRecord(A.ev[3], h->st));
    const int bcz[4] = {0, 0, 0, 0};
    if (h->prec == EU_FP32) EU_CUDA(h, launch_unpack_aos<float>(Planes<float>{static_cast<float*>(A.lam), h->pitch_s, h->plane_s}, kSOff, h->cfg.nx, h->cfg.ny, bcz, h->d_aos, h->st));
    else EU_CUDA(h, launch_unpack_aos<double>(Planes<double>{static_cast<double*>(A.lam), h->pitch_s, h->plane_s}, kSOff, h->cfg.nx, h->cfg.ny, bcz, h->d_aos, h->st));
    EU_CUDA(h, cudaMemcpyAsync(dJ_dU0, h->d_aos, aos_bytes(h), cudaMemcpyDeviceToHost, h->st));
    return EU_OK;
}

int adj_bwd_finish(eu_handle* h, double* dJ_dU0) {
    auto& A = h->adj;
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    EU_CUDA(h, cudaEventElapsedTime(&A.ms_bwd, A.ev[2], A.ev[3]));
    // the gradient is with respect to the interior; ghost entries are zero
    const int tnx = h->cfg.nx + 4, tny = h->cfg.ny + 4;
    for (int j = 0; j < tny; ++j)
        for (int i = 0; i < tnx; ++i)
            if (i < 2 || i >= tnx - 2 || j < 2 || j >= tny - 2) std::memset(dJ_dU0 + 4 * ((size_t)j * tnx + i), 0, 32);
    return EU_OK;
}

template <class T> Planes<T> planes_of(const eu_handle* h, void* b) {
    return Planes<T>{static_cast<T*>(b), h->pitch_s, h->plane_s};
}

// ---------------------------------------------------------------------------
// ensemble: descriptors, launches
// ---------------------------------------------------------------------------
int bfail(eu_batch* b, int code, const std::string& msg) {
    (void)cudaGetLastError();
    if (b) b->err = msg;
    else g_err = msg;
    return code;
}

template <class T> int batch_build_t(eu_batch* b) {
    std::vector<EnsInst<T>> inst((size_t)b->n);
    EnsArgs<T> A;
    std::memset(&A, 0, sizeof(A));
    A.inst = static_cast<const EnsInst<T>*>(b->d_inst);
    A.sched = b->d_sched;
    A.ninst = b->n;
    int tx = 0, ty = 0;
    for (int i = 0; i < b->n; ++i) {
        eu_handle* h = b->h[(size_t)i];
        EnsInst<T>& I = inst[(size_t)i];
        I.tm_x[0] = h->tm_x[0];
        I.tm_x[1] = h->tm_x[1];
        I.tm_xo = h->tm_xo;
        I.tm_y = h->tm_y;
        I.tm_yo[0] = h->tm_yo[0];
        I.tm_yo[1] = h->tm_yo[1];
        I.xa = x_args<T>(h, 0);
        I.xa.snap = nullptr;
        I.ya[0] = y_args<T>(h, 1);   // y_args(h, cur) writes buffer 1 - cur
        I.ya[1] = y_args<T>(h, 0);
        A.x_off[i] = tx;
        A.y_off[i] = ty;
        tx += h->ntasks_x;
        ty += h->ntasks_y;
    }
    A.x_off[b->n] = tx;
    A.y_off[b->n] = ty;
    A.total_x = tx;
    A.total_y = ty;
    A.wait_extra = b->wait_extra;
    cudaError_t e = cudaMemcpyAsync(b->d_inst, inst.data(), sizeof(EnsInst<T>) * (size_t)b->n,
                                    cudaMemcpyHostToDevice, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return bfail(b, EU_ERR_CUDA, std::string("ensemble descriptors: ") + cudaGetErrorString(e));
    b->args.assign(reinterpret_cast<unsigned char*>(&A), reinterpret_cast<unsigned char*>(&A) + sizeof(A));
    if (b->g) { cudaGraphExecDestroy(b->g); b->g = nullptr; }
    b->dirty = false;
    return EU_OK;
}
int batch_build(eu_batch* b) { return b->prec == EU_FP32 ? batch_build_t<float>(b) : batch_build_t<double>(b); }

cudaError_t batch_launch(eu_batch* b) {
    cudaError_t e = cudaMemsetAsync(b->d_sched, 0, sizeof(EnsSched), b->st);
    if (e != cudaSuccess) return e;
    return b->K.ens(b->args.data(), b->ctas, b->st);
}

int batch_graph(eu_batch* b, int steps, cudaGraphExec_t* out) {
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal);
    for (int s = 0; s < steps && e == cudaSuccess; ++s) e = batch_launch(b);
    cudaError_t e2 = cudaStreamEndCapture(b->st, &gr);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, gr, 0);
    if (gr) cudaGraphDestroy(gr);
    if (e != cudaSuccess) return bfail(b, EU_ERR_CUDA, std::string("ensemble graph: ") + cudaGetErrorString(e));
    return EU_OK;
}

// Pull every instance's control block; report the first bad status.
int batch_pull(eu_batch* b, int* all_done) {
    int done = 1;
    for (int i = 0; i < b->n; ++i) {
        eu_handle* h = b->h[(size_t)i];
        if (ctl_pull_sync(h)) return bfail(b, EU_ERR_CUDA, h->err);
        const int st = h->hctl->status;
        if (st & kStatusTimeout) return bfail(b, EU_ERR_TIMEOUT, "instance " + std::to_string(i) + ": a bounded device wait expired");
        if (st & kStatusNonPhysical)
            return bfail(b, EU_ERR_NONPHYSICAL, "instance " + std::to_string(i) + ": non-positive maximum wave speed");
        if (st & kStatusNonFinite)
            return bfail(b, EU_ERR_NONPHYSICAL, "instance " + std::to_string(i) + ": non-finite state");
        done &= h->hctl->done ? 1 : 0;
    }
    if (all_done) *all_done = done;
    return EU_OK;
}

}  // namespace

namespace eu {
// Message for eu_last_error(NULL), for entry points defined in other units.
void set_global_error(const char* msg) { g_err = msg; }
}  // namespace eu

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int eu_abi_version(void) { return EU_ABI_VERSION; }

const char* eu_last_error(const eu_handle* h) { return h ? h->err.c_str() : g_err.c_str(); }

int eu_device_info(char* name, int len, int* sm_count) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return fail(nullptr, EU_ERR_CUDA, "no CUDA device");
    cudaDeviceProp p;
    EU_CUDA(nullptr, cudaGetDeviceProperties(&p, 0));
    if (name && len > 0) std::snprintf(name, (size_t)len, "%s (sm_%d%d)", p.name, p.major, p.minor);
    if (sm_count) *sm_count = p.multiProcessorCount;
    return EU_OK;
}

int eu_create(const eu_case* cfg, eu_precision prec, eu_solver solver, eu_limiter limiter, const int* bc,
              eu_handle** out) {
    if (!cfg || !out) return fail(nullptr, EU_ERR_INVALID, "eu_create: null argument");
    *out = nullptr;
    if (cfg->nx < 1 || cfg->ny < 1) return fail(nullptr, EU_ERR_INVALID, "eu_create: nx and ny must be >= 1");
    if (cfg->ng != 2) return fail(nullptr, EU_ERR_INVALID, "eu_create: ghost width ng must be 2");
    if (!(cfg->x_max > cfg->x_min) || !(cfg->y_max > cfg->y_min))
        return fail(nullptr, EU_ERR_INVALID, "eu_create: empty domain");
    if (prec != EU_FP64 && prec != EU_FP32) return fail(nullptr, EU_ERR_INVALID, "eu_create: bad precision");
    if (solver < EU_HLL || solver > EU_FORCE) return fail(nullptr, EU_ERR_INVALID, "eu_create: bad solver");
    if (limiter != EU_LIMITER_MINMOD) return fail(nullptr, EU_ERR_INVALID, "eu_create: only minmod is provided");
    if ((long long)cfg->nx * cfg->ny > (1LL << 31) - 1 || cfg->nx > (1 << 28) || cfg->ny > (1 << 28))
        return fail(nullptr, EU_ERR_INVALID, "eu_create: grid too large");
    int b4[4] = {0, 0, 0, 0};
    if (bc)
        for (int k = 0; k < 4; ++k) {
            if (bc[k] != EU_BC_TRANSMISSIVE && bc[k] != EU_BC_REFLECTIVE)
                return fail(nullptr, EU_ERR_INVALID, "eu_create: bad boundary kind");
            b4[k] = bc[k];
        }
    if ((b4[0] || b4[1]) && cfg->nx < 2) return fail(nullptr, EU_ERR_INVALID, "reflective x sides need nx >= 2");
    if ((b4[2] || b4[3]) && cfg->ny < 2) return fail(nullptr, EU_ERR_INVALID, "reflective y sides need ny >= 2");

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(nullptr, EU_ERR_CUDA, "eu_create: no CUDA device (this library has no CPU path)");
    int dev = 0, major = 0, minor = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (major != 10 || minor != 3)
        return fail(nullptr, EU_ERR_CUDA,
                    "eu_create: kernels are built for sm_103a; device is sm_" + std::to_string(major) +
                        std::to_string(minor));

    eu_handle* h = new eu_handle();
    h->cfg = *cfg;
    h->prec = prec;
    h->solver = solver;
    std::memcpy(h->bc, b4, sizeof(b4));
    h->esz = prec == EU_FP32 ? 4 : 8;
    h->dx = (cfg->x_max - cfg->x_min) / (double)cfg->nx;  // head/cpu/grid_cpu.hpp:19-20
    h->dy = (cfg->y_max - cfg->y_min) / (double)cfg->ny;
    cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, dev);
    h->K = kernels_for(prec, solver);
    h->gsteps = 2;
    plan(h);

    auto bail = [&](int rc) {
        eu_destroy(h);
        return rc;
    };
    const long long align = 128 / (long long)h->esz;
    h->pitch_s = round_up(cfg->nx + kSOff + 2, align);
    h->pitch_t = round_up(cfg->nx + kTOff, align);
    h->plane_s = round_up(h->pitch_s * (cfg->ny + 4), 256 / (long long)h->esz);
    h->plane_t = round_up(h->pitch_t * (cfg->ny + 4), 256 / (long long)h->esz);
    cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) { g_err = std::string("cudaStreamCreate: ") + cudaGetErrorString(e); return bail(EU_ERR_CUDA); }
    for (int b = 0; b < 2; ++b) {
        e = cudaMalloc(&h->S[b], (size_t)(4 * h->plane_s) * h->esz);
        if (e == cudaSuccess) e = cudaMemsetAsync(h->S[b], 0, (size_t)(4 * h->plane_s) * h->esz, h->st);
        if (e != cudaSuccess) { (void)cudaGetLastError(); g_err = std::string("state buffer: ") + cudaGetErrorString(e); return bail(EU_ERR_NOMEM); }
    }
    e = cudaMalloc(&h->Tm, (size_t)(4 * h->plane_t) * h->esz);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->Tm, 0, (size_t)(4 * h->plane_t) * h->esz, h->st);
    if (e == cudaSuccess) e = cudaMalloc(&h->ctl, sizeof(Ctl));
    if (e == cudaSuccess) e = cudaMallocHost(&h->hctl, sizeof(Ctl));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_part, sizeof(double) * 8 * h->part_blocks);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_tot, sizeof(double) * 4);
    if (e == cudaSuccess) e = cudaMallocHost(&h->h_tot, sizeof(double) * 4);
    if (e != cudaSuccess) { (void)cudaGetLastError(); g_err = std::string("allocation: ") + cudaGetErrorString(e); return bail(EU_ERR_NOMEM); }
    ctl_reset(h, kModeHost, INFINITY, LLONG_MAX);
    if (ctl_push(h)) { g_err = h->err; return bail(EU_ERR_CUDA); }
    if (encode_all(h)) {
        g_err = h->err;
        return bail(EU_ERR_CUDA);
    }
    e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess) { g_err = std::string("eu_create: ") + cudaGetErrorString(e); return bail(EU_ERR_CUDA); }
    *out = h;
    return EU_OK;
}

void eu_destroy(eu_handle* h) {
    if (!h) return;
    if (h->st) cudaStreamSynchronize(h->st);
    drop_graphs(h);
    cudaFree(h->S[0]);
    cudaFree(h->S[1]);
    cudaFree(h->Tm);
    cudaFree(h->ctl);
    cudaFreeHost(h->hctl);
    cudaFree(h->d_aos);
    cudaFreeHost(h->h_aos);
    cudaFree(h->d_part);
    cudaFree(h->d_tot);
    cudaFreeHost(h->h_tot);
    cudaFree(h->snap);
    cudaFree(h->d_frozen);
    cudaFree(h->d_dtlog);
    adj_free(h);
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
}

// --- setup ------------------------------------------------------------------
int eu_get_case_config(const char* name, int n, eu_case* out) {
    if (!name || !out) return fail(nullptr, EU_ERR_INVALID, "eu_get_case_config: null argument");
    if (n < 1) return fail(nullptr, EU_ERR_INVALID, "get_n_case_config: n must be >= 1.");
    const std::string s(name);
    // src/test_cases.cpp:132-162
    if (s == "shock_bubble") *out = eu_case{500, 197, 2, 0.0, 0.225, 0.0, 0.089, 0.4, 0.0011741};
    else if (s == "blast_wave") *out = eu_case{500, 500, 2, 0.0, 1.0, 0.0, 1.0, 0.4, 0.2};
    else
        return fail(nullptr, EU_ERR_INVALID,
                    "Unknown case name: " + s + ". Supported cases are: shock_bubble, blast_wave.");
    out->nx *= n;  // src/test_cases.cpp:184-195
    out->ny *= n;
    return EU_OK;
}

int eu_init_blast(eu_handle* h, double cx, double cy, double r, double rho_in, double p_in, double rho_out,
                  double p_out) {
    if (!h) return fail(nullptr, EU_ERR_INVALID, "null handle");
    const GridGeom g{h->cfg.nx, h->cfg.ny, h->cfg.x_min, h->cfg.x_max, h->cfg.y_min, h->cfg.y_max};
    const BlastDesc b{cx, cy, r, rho_in, p_in, rho_out, p_out};
    if (h->prec == EU_FP32) EU_CUDA(h, launch_init_blast<float>(planes_s<float>(h, h->cur), g, b, h->st));
    else EU_CUDA(h, launch_init_blast<double>(planes_s<double>(h, h->cur), g, b, h->st));
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    return EU_OK;
}

int eu_init_shock_bubble(eu_handle* h, double rho0, double p0, double mach, double shock_x, double bub_cx,
                         double bub_cy, double bub_r, double rho_bubble) {
    if (!h) return fail(nullptr, EU_ERR_INVALID, "null handle");
    const GridGeom g{h->cfg.nx, h->cfg.ny, h->cfg.x_min, h->cfg.x_max, h->cfg.y_min, h->cfg.y_max};
    const ShockBubbleDesc d{rho0, p0, mach, shock_x, bub_cx, bub_cy, bub_r, rho_bubble};
    if (h->prec == EU_FP32) EU_CUDA(h, launch_init_shock_bubble<float>(planes_s<float>(h, h->cur), g, d, h->st));
    else EU_CUDA(h, launch_init_shock_bubble<double>(planes_s<double>(h, h->cur), g, d, h->st));
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    return EU_OK;
}

int eu_init_reference_case(eu_handle* h, const char* name) {
    if (!h || !name) return fail(h, EU_ERR_INVALID, "null argument");
    const std::string s(name);
    // src/test_cases.cpp:24-33 and :79-89
    if (s == "shock_bubble") return eu_init_shock_bubble(h, 1.29, 1.01325e5, 1.22, 0.005, 0.035, 0.0445, 0.025, 0.214);
    if (s == "blast_wave") return eu_init_blast(h, 0.5, 0.5, 0.1, 1.0, 100.0, 1.0, 1.0);
    return fail(h, EU_ERR_INVALID, "Unknown case name: " + s + ". Supported cases are: shock_bubble, blast_wave.");
}

// --- transfer -------------------------------------------------------------
int eu_upload_aos(eu_handle* h, const double* aos) {
    if (!h || !aos) return fail(h, EU_ERR_INVALID, "null argument");
    int rc = upload_to(h, h->cur, aos);
    if (rc) return rc;
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    return EU_OK;
}

int eu_download_aos(eu_handle* h, double* aos) {
    if (!h || !aos) return fail(h, EU_ERR_INVALID, "null argument");
    int rc = download_from_state(h, h->cur, aos);
    if (rc) return rc;
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    return EU_OK;
}

// --- hot path -----------------------------------------------------------------
int eu_compute_dt(eu_handle* h, double cfl, double* dt) {
    if (!h || !dt) return fail(h, EU_ERR_INVALID, "null argument");
    if (!(cfl > 0.0)) return fail(h, EU_ERR_INVALID, "cfl must be positive");
    Ctl& c = *h->hctl;
    c.mode = kModeHost;
    c.cfl_dmin = cfl * std::min(h->dx, h->dy);
    c.done = 0;
    c.status = 0;
    c.smax_bits = 0;
    c.arrive = 0;
    c.max_steps = LLONG_MAX;
    int rc = ctl_push(h);
    if (rc) return rc;
    EU_CUDA(h, launch_dt(h, h->cur));
    rc = ctl_pull_sync(h);
    if (rc) return rc;
    rc = status_code(h);
    if (rc) return rc;
    *dt = c.dt;
    return EU_OK;
}

int eu_advance(eu_handle* h, double dt) {
    Range range_("eu_advance");
    if (!h) return fail(nullptr, EU_ERR_INVALID, "null handle");
    if (!(dt >= 0.0) || !std::isfinite(dt)) return fail(h, EU_ERR_INVALID, "dt must be finite and >= 0");
    Ctl& c = *h->hctl;
    c.mode = kModeHost;
    c.dt = dt;
    c.done = 0;
    c.status = 0;
    c.smax_bits = 0;
    c.arrive = 0;
    c.max_steps = LLONG_MAX;
    c.snap_req = 0;
    c.nsnap = 0;
    c.cur = h->cur;
    int rc = ctl_push(h);
    if (rc) return rc;
    EU_CUDA(h, launch_step(h, h->cur));
    rc = ctl_pull_sync(h);
    if (rc) return rc;
    return h->hctl->status & kStatusTimeout ? status_code(h) : EU_OK;
}

int eu_advance_first_order(eu_handle* h, double dt) {
    if (!h) return fail(nullptr, EU_ERR_INVALID, "null handle");
    if (!(dt >= 0.0) || !std::isfinite(dt)) return fail(h, EU_ERR_INVALID, "dt must be finite and >= 0");
    const int nxt = 1 - h->cur;
    if (h->prec == EU_FP32) {
        const Planes<float> a = planes_s<float>(h, h->cur), b = planes_s<float>(h, nxt);
        EU_CUDA(h, h->K.first(&a, &b, h->cfg.nx, h->cfg.ny, dt / h->dx, dt / h->dy, h->st));
    } else {
        const Planes<double> a = planes_s<double>(h, h->cur), b = planes_s<double>(h, nxt);
        EU_CUDA(h, h->K.first(&a, &b, h->cfg.nx, h->cfg.ny, dt / h->dx, dt / h->dy, h->st));
    }
    EU_CUDA(h, fill_ghosts(h, nxt));  // src/cpu/solver_cpu.cpp:368
    Ctl& c = *h->hctl;
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    h->cur = nxt;
    c.cur = nxt;
    c.t += dt;
    c.step += 1;
    return ctl_push(h);
}

int eu_advance_first_order_host(eu_handle* h, const double* Uold, double* Unew, double dt) {
    if (!h || !Uold || !Unew) return fail(h, EU_ERR_INVALID, "null argument");
    int rc = upload_to(h, h->cur, Uold);
    if (rc) return rc;
    if ((rc = eu_advance_first_order(h, dt))) return rc;
    if ((rc = download_from_state(h, h->cur, Unew))) return rc;
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    return EU_OK;
}

int eu_step_n(eu_handle* h, long long n, const double* dts) {
    Range range_("eu_step_n");
    if (!h) return fail(nullptr, EU_ERR_INVALID, "null handle");
    if (n < 0) return fail(h, EU_ERR_INVALID, "n must be >= 0");
    if (n == 0) return EU_OK;
    Ctl& c = *h->hctl;
    const double t0 = c.t;
    const long long s0 = c.step;
    ctl_reset(h, dts ? kModeFrozen : kModeCfl, INFINITY, s0 + n);
    c.t = t0;
    c.step = s0;
    if (dts) {
        if (n > h->frozen_cap) {
            cudaFree(h->d_frozen);
            h->d_frozen = nullptr;
            h->frozen_cap = 0;
            EU_CUDA(h, cudaMalloc(&h->d_frozen, sizeof(double) * (size_t)n));
            h->frozen_cap = n;
        }
        EU_CUDA(h, cudaMemcpyAsync(h->d_frozen, dts, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, h->st));
        c.frozen = h->d_frozen;
        c.n_frozen = n;
        c.frozen_base = s0;
        c.dt = dts[0];
    }
    int rc = ctl_push(h);
    if (rc) return rc;
    EU_CUDA(h, fill_ghosts(h, h->cur));  // scripts/cpu/main_cpu.cpp:222
    if (!dts) EU_CUDA(h, launch_dt(h, h->cur));
    const int K = h->gsteps;
    const long long reps = (n + K - 1) / K;
    cudaGraphExec_t g = nullptr;
    int cur = h->cur;
    for (long long r = 0; r < reps; ++r) {
        // Replays of a K-step graph; steps past the end are no-ops (Ctl::done).
        rc = graph_for(h, cur, &g);
        if (rc) return rc;
        EU_CUDA(h, cudaGraphLaunch(g, h->st));
        cur = (cur + K) & 1;
    }
    rc = ctl_pull_sync(h);
    if (rc) return rc;
    return status_code(h);
}

int eu_run(eu_handle* h, double t_end, int nsnap, eu_snapshot_cb cb, void* user, eu_run_info* info) {
    Range range_("eu_run");
    if (!h) return fail(nullptr, EU_ERR_INVALID, "null handle");
    if (nsnap < 0 || nsnap > kMaxSnap) return fail(h, EU_ERR_INVALID, "nsnap must be in [0, 16]");
    if (!(t_end >= 0.0)) return fail(h, EU_ERR_INVALID, "t_end must be >= 0");
    const bool want = cb && nsnap > 0;
    int rc = EU_OK;
    if (want && (rc = ensure_snapshots(h, nsnap))) return rc;
    ctl_reset(h, kModeCfl, t_end, LLONG_MAX);
    Ctl& c = *h->hctl;
    c.nsnap = want ? nsnap : 0;  // without storage no snapshot is ever requested
    for (int k = 0; k < nsnap; ++k) c.snap_target[k] = t_end * (double)(k + 1) / (double)nsnap;  // main_cpu.cpp:210-215
    if ((rc = ctl_push(h))) return rc;
    EU_CUDA(h, fill_ghosts(h, h->cur));  // scripts/cpu/main_cpu.cpp:222
    EU_CUDA(h, launch_dt(h, h->cur));
    if ((rc = ctl_pull_sync(h))) return rc;
    int delivered = 0;
    bool aborted = false;
    while (!c.done) {
        cudaGraphExec_t g = nullptr;
        if ((rc = graph_for(h, h->cur, &g))) return rc;
        EU_CUDA(h, cudaGraphLaunch(g, h->st));
        if ((rc = ctl_pull_sync(h))) return rc;
        // hand over every snapshot whose copy is complete
        while (want && !aborted && delivered < c.next_snap) {
            const int k = delivered;
            const long long sstep = c.snap_step[k];
            if (!(c.step > sstep || c.done)) break;
            int kb = k;
            while (kb > 0 && c.snap_step[kb - 1] == sstep) --kb;
            if (c.step > sstep) {
                const long long plane = h->snap_plane;
                if (h->prec == EU_FP32)
                    EU_CUDA(h, launch_unpack_snapshot<float>(static_cast<float*>(h->snap) + kb * h->snap_stride, plane,
                                                             h->cfg.nx, h->cfg.ny, h->bc, h->d_aos, h->st));
                else
                    EU_CUDA(h, launch_unpack_snapshot<double>(static_cast<double*>(h->snap) + kb * h->snap_stride,
                                                              plane, h->cfg.nx, h->cfg.ny, h->bc, h->d_aos, h->st));
            } else {
                EU_CUDA(h, unpack_state(h, h->cur, h->d_aos));
            }
            EU_CUDA(h, cudaMemcpyAsync(h->h_aos, h->d_aos, aos_bytes(h), cudaMemcpyDeviceToHost, h->st));
            EU_CUDA(h, cudaStreamSynchronize(h->st));
            if (cb(user, k + 1, sstep, c.snap_time[k], h->h_aos, h->cfg.nx, h->cfg.ny)) aborted = true;
            ++delivered;
        }
        if (aborted || c.status) break;
    }
    if (info) {
        info->t = c.t;
        info->steps = c.step;
        info->status = c.status;
        info->nsnap_written = delivered;
    }
    if (aborted) return fail(h, EU_ERR_STATE, "run aborted by the snapshot callback");
    return status_code(h);
}

int eu_get_time(eu_handle* h, double* t, long long* steps, double* dt_next) {
    if (!h) return fail(nullptr, EU_ERR_INVALID, "null handle");
    int rc = ctl_pull_sync(h);
    if (rc) return rc;
    if (t) *t = h->hctl->t;
    if (steps) *steps = h->hctl->step;
    if (dt_next) *dt_next = h->hctl->dt;
    return EU_OK;
}

int eu_totals(eu_handle* h, double out[4]) {
    if (!h || !out) return fail(h, EU_ERR_INVALID, "null argument");
    if (h->prec == EU_FP32)
        EU_CUDA(h, launch_totals<float>(planes_s<float>(h, h->cur), kSOff, h->cfg.nx, h->cfg.ny, h->d_part,
                                        h->part_blocks, h->d_tot, h->st));
    else
        EU_CUDA(h, launch_totals<double>(planes_s<double>(h, h->cur), kSOff, h->cfg.nx, h->cfg.ny, h->d_part,
                                         h->part_blocks, h->d_tot, h->st));
    EU_CUDA(h, cudaMemcpyAsync(h->h_tot, h->d_tot, 4 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    std::memcpy(out, h->h_tot, 4 * sizeof(double));
    return EU_OK;
}

// --- drop-in calls on host grids -----------------------------------------------
// --- discrete adjoint -----------------------------------------------------------
int eu_adjoint_forward(eu_handle* h, long long nsteps, const double* dts, int ckpt_k) {
    Range range_("eu_adjoint_forward");
    if (int rc = adj_fwd_enqueue(h, nsteps, dts, ckpt_k)) return rc;
    return adj_fwd_finish(h);
}

int eu_adjoint_backward(eu_handle* h, const double* dJ_dUN, double* dJ_dU0) {
    Range range_("eu_adjoint_backward");
    if (int rc = adj_bwd_enqueue(h, dJ_dUN, dJ_dU0)) return rc;
    return adj_bwd_finish(h, dJ_dU0);
}

int eu_adjoint_timing(eu_handle* h, float ms[2]) {
    if (!h || !ms) return fail(h, EU_ERR_INVALID, "eu_adjoint_timing: null argument");
    ms[0] = h->adj.ms_fwd;
    ms[1] = h->adj.ms_bwd;
    return EU_OK;
}

int eu_compute_dt_host(eu_handle* h, const double* U, double cfl, double* dt) {
    if (!h || !U || !dt) return fail(h, EU_ERR_INVALID, "null argument");
    int rc = upload_to(h, h->cur, U);
    if (rc) return rc;
    return eu_compute_dt(h, cfl, dt);
}

int eu_advance_host(eu_handle* h, const double* Uold, double* Utmp, double* Unew, double dt) {
    if (!h || !Uold || !Unew) return fail(h, EU_ERR_INVALID, "null argument");
    int rc = upload_to(h, h->cur, Uold);
    if (rc) return rc;
    if ((rc = eu_advance(h, dt))) return rc;
    if (Utmp) {
        EU_CUDA(h, unpack_tmp(h, h->d_aos));
        EU_CUDA(h, cudaMemcpyAsync(Utmp, h->d_aos, aos_bytes(h), cudaMemcpyDeviceToHost, h->st));
    }
    if ((rc = download_from_state(h, h->cur, Unew))) return rc;
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    return EU_OK;
}

int eu_step_host(eu_handle* h, const double* U, double* Unext, double cfl, double t, double t_end,
                 double* dt_used) {
    Range range_("eu_step_host");
    if (!h || !U || !Unext) return fail(h, EU_ERR_INVALID, "null argument");
    int rc = upload_to(h, h->cur, U);
    if (rc) return rc;
    ctl_reset(h, kModeCfl, t_end, LLONG_MAX);
    Ctl& c = *h->hctl;
    c.cfl_dmin = cfl * std::min(h->dx, h->dy);
    c.t = t;
    if ((rc = ctl_push(h))) return rc;
    EU_CUDA(h, fill_ghosts(h, h->cur));         // apply_transmissive_boundary(U)
    EU_CUDA(h, launch_dt(h, h->cur));           // dt = compute_dt(U), clipped to t_end - t
    EU_CUDA(h, cudaMemcpyAsync(&h->hctl->dt, &h->ctl->dt, sizeof(double), cudaMemcpyDeviceToHost, h->st));
    EU_CUDA(h, launch_step(h, h->cur));
    const int nxt = 1 - h->cur;
    if ((rc = download_from_state(h, nxt, Unext))) return rc;
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    if (dt_used) *dt_used = h->hctl->dt;
    rc = ctl_pull_sync(h);
    if (rc) return rc;
    return status_code(h);
}

// --- measurement ----------------------------------------------------------------
int eu_time_steps(eu_handle* h, int nsteps, int use_graph, float ms[3]) {
    if (!h || !ms || nsteps < 1) return fail(h, EU_ERR_INVALID, "bad argument");
    Ctl& c = *h->hctl;
    const double t0 = c.t;
    const long long s0 = c.step;
    ctl_reset(h, kModeCfl, INFINITY, LLONG_MAX);
    c.t = t0;
    c.step = s0;
    int rc = ctl_push(h);
    if (rc) return rc;
    EU_CUDA(h, fill_ghosts(h, h->cur));
    EU_CUDA(h, launch_dt(h, h->cur));
    std::vector<cudaEvent_t> ev(2 * (size_t)nsteps + 1, nullptr);
    for (auto& e : ev) EU_CUDA(h, cudaEventCreate(&e));
    auto cleanup = [&]() { for (auto& e : ev) if (e) cudaEventDestroy(e); };
    cudaError_t e = cudaSuccess;
    int cur = h->cur;
    if (use_graph) {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t gx = nullptr;
        e = cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal);
        for (int s = 0; s < nsteps && e == cudaSuccess; ++s) {
            const int cc = (cur + s) & 1;
            if (s == 0) e = cudaEventRecordWithFlags(ev[0], h->st, cudaEventRecordExternal);
            if (e == cudaSuccess) e = launch_x(h, cc);
            if (e == cudaSuccess) e = cudaEventRecordWithFlags(ev[2 * s + 1], h->st, cudaEventRecordExternal);
            if (e == cudaSuccess) e = launch_y(h, cc);
            if (e == cudaSuccess) e = cudaEventRecordWithFlags(ev[2 * s + 2], h->st, cudaEventRecordExternal);
        }
        cudaError_t e2 = cudaStreamEndCapture(h->st, &g);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&gx, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e == cudaSuccess) e = cudaGraphLaunch(gx, h->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
        if (gx) cudaGraphExecDestroy(gx);
    } else {
        e = cudaEventRecord(ev[0], h->st);
        for (int s = 0; s < nsteps && e == cudaSuccess; ++s) {
            const int cc = (cur + s) & 1;
            e = launch_x(h, cc);
            if (e == cudaSuccess) e = cudaEventRecord(ev[2 * s + 1], h->st);
            if (e == cudaSuccess) e = launch_y(h, cc);
            if (e == cudaSuccess) e = cudaEventRecord(ev[2 * s + 2], h->st);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    }
    if (e != cudaSuccess) { cleanup(); return cuda_fail(h, e, "eu_time_steps"); }
    float tot = 0, tx = 0, ty = 0, v = 0;
    cudaEventElapsedTime(&tot, ev[0], ev[2 * nsteps]);
    for (int s = 0; s < nsteps; ++s) {
        cudaEventElapsedTime(&v, ev[2 * s], ev[2 * s + 1]);
        tx += v;
        cudaEventElapsedTime(&v, ev[2 * s + 1], ev[2 * s + 2]);
        ty += v;
    }
    cleanup();
    ms[0] = tot;
    ms[1] = tx;
    ms[2] = ty;
    rc = ctl_pull_sync(h);
    if (rc) return rc;
    return status_code(h);
}

// Measured choice of the launch shape: each trial sets one candidate
// segment length per sweep and times `steps` graph-replayed steps with CUDA
// events around every kernel; the x- and y-sweep times are kept apart, so
// one pass over the trials tunes both sweeps.  The state, time and step
// counter are restored afterwards.
int eu_autotune(eu_handle* h, int steps, long long chosen[2]) {
    Range range_("eu_autotune");
    if (!h || steps < 1) return fail(h, EU_ERR_INVALID, "eu_autotune: bad argument");
    const int CX = h->K.box_x, RY = h->K.ry;
    std::vector<int> cx, cy;
    for (int v : {CX, 2 * CX, 4 * CX, 32, 64, 128, 256})
        if (v % CX == 0 && v <= round_up(h->cfg.nx, CX) && std::find(cx.begin(), cx.end(), v) == cx.end()) cx.push_back(v);
    for (int v : {RY, 2 * RY, 4 * RY, 32, 64, 128})
        if (v % RY == 0 && v <= round_up(h->cfg.ny, RY) && std::find(cy.begin(), cy.end(), v) == cy.end()) cy.push_back(v);
    if (cx.empty()) cx.push_back(CX);
    if (cy.empty()) cy.push_back(RY);
    void* saved = nullptr;
    EU_CUDA(h, cudaMalloc(&saved, state_bytes(h)));
    const int cur0 = h->cur;
    const Ctl ctl0 = *h->hctl;
    cudaError_t e = cudaMemcpyAsync(saved, h->S[cur0], state_bytes(h), cudaMemcpyDeviceToDevice, h->st);
    const int seg_x0 = h->seg_x, seg_y0 = h->seg_y;
    int best_x = seg_x0, best_y = seg_y0;
    float tbx = INFINITY, tby = INFINITY;
    int rc = EU_OK;
    const size_t trials = std::max(cx.size(), cy.size());
    for (size_t t = 0; t < trials && rc == EU_OK && e == cudaSuccess; ++t) {
        const int sx = cx[std::min(t, cx.size() - 1)], sy = cy[std::min(t, cy.size() - 1)];
        rc = eu_set_option(h, "seg_x", sx);
        if (rc == EU_OK) rc = eu_set_option(h, "seg_y", sy);
        float ms[3];
        if (rc == EU_OK) rc = eu_time_steps(h, 2, 1, ms);
        if (rc == EU_OK) rc = eu_time_steps(h, steps, 1, ms);
        if (rc != EU_OK) break;
        if (t < cx.size() && ms[1] < tbx) { tbx = ms[1]; best_x = sx; }
        if (t < cy.size() && ms[2] < tby) { tby = ms[2]; best_y = sy; }
    }
    if (rc == EU_OK) rc = eu_set_option(h, "seg_x", best_x);
    if (rc == EU_OK) rc = eu_set_option(h, "seg_y", best_y);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->S[cur0], saved, state_bytes(h), cudaMemcpyDeviceToDevice, h->st);
    h->cur = cur0;
    *h->hctl = ctl0;
    if (e == cudaSuccess && ctl_push(h) != EU_OK) e = cudaErrorUnknown;
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    cudaFree(saved);
    if (rc != EU_OK) return rc;
    if (e != cudaSuccess) return cuda_fail(h, e, "eu_autotune");
    if (chosen) { chosen[0] = best_x; chosen[1] = best_y; }
    return EU_OK;
}

int eu_apply_boundary(eu_handle* h) {
    if (!h) return fail(nullptr, EU_ERR_INVALID, "null handle");
    EU_CUDA(h, fill_ghosts(h, h->cur));
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    return EU_OK;
}

int eu_set_dt_log(eu_handle* h, long long capacity) {
    if (!h || capacity < 0) return fail(h, EU_ERR_INVALID, "bad argument");
    cudaFree(h->d_dtlog);
    h->d_dtlog = nullptr;
    h->dtlog_cap = 0;
    if (capacity > 0) {
        EU_CUDA(h, cudaMalloc(&h->d_dtlog, sizeof(double) * (size_t)capacity));
        EU_CUDA(h, cudaMemsetAsync(h->d_dtlog, 0, sizeof(double) * (size_t)capacity, h->st));
        h->dtlog_cap = capacity;
    }
    h->hctl->dt_log = h->d_dtlog;
    h->hctl->dt_log_cap = h->dtlog_cap;
    return ctl_push(h);
}

int eu_get_dt_log(eu_handle* h, double* out, long long n) {
    if (!h || !out || n < 0 || n > h->dtlog_cap) return fail(h, EU_ERR_INVALID, "bad argument");
    if (n == 0) return EU_OK;
    EU_CUDA(h, cudaMemcpyAsync(out, h->d_dtlog, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, h->st));
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    return EU_OK;
}

int eu_set_option(eu_handle* h, const char* name, long long value) {
    if (!h || !name) return fail(h, EU_ERR_INVALID, "null argument");
    const std::string k(name);
    if (k == "l2_promotion_x" || k == "l2_promotion_y") {
        if (value != 0 && value != 64 && value != 128 && value != 256)
            return fail(h, EU_ERR_INVALID, "L2 promotion must be 0, 64, 128 or 256 bytes");
        (k == "l2_promotion_x" ? h->l2promo_x : h->l2promo_y) = (int)value;
        if (int rc = encode_all(h)) return rc;
    } else if (k == "seg_x") {
        if (value < h->K.box_x || value % h->K.box_x) return fail(h, EU_ERR_INVALID, "seg_x must be a multiple of the box width");
        h->seg_x = (int)value;
        h->nseg_x = (h->cfg.nx + h->seg_x - 1) / h->seg_x;
        h->ntasks_x = ((h->cfg.ny + 31) / 32) * h->nseg_x;
        h->ctas_x = (h->ntasks_x + h->K.nw - 1) / h->K.nw;
    } else if (k == "seg_y") {
        if (value < h->K.ry || value % h->K.ry) return fail(h, EU_ERR_INVALID, "seg_y must be a multiple of the box height");
        h->seg_y = (int)value;
        h->ntasks_y = h->nseg_y * ((h->cfg.ny + h->seg_y - 1) / h->seg_y);
        h->ctas_y = (h->ntasks_y + h->K.nw - 1) / h->K.nw;
    } else if (k == "graph_steps") {
        if (value < 1 || value > 4096) return fail(h, EU_ERR_INVALID, "graph_steps must be in [1, 4096]");
        h->gsteps = (int)value;
    } else {
        return fail(h, EU_ERR_INVALID, "unknown option " + k);
    }
    drop_graphs(h);
    return EU_OK;
}

int eu_get_option(eu_handle* h, const char* name, long long* value) {
    if (!h || !name || !value) return fail(h, EU_ERR_INVALID, "null argument");
    const std::string k(name);
    if (k == "l2_promotion_x") *value = h->l2promo_x;
    else if (k == "l2_promotion_y") *value = h->l2promo_y;
    else if (k == "seg_x") *value = h->seg_x;
    else if (k == "seg_y") *value = h->seg_y;
    else if (k == "graph_steps") *value = h->gsteps;
    else if (k == "tasks_x") *value = h->ntasks_x;
    else if (k == "occ_x") *value = h->K.occ_x();
    else if (k == "occ_y") *value = h->K.occ_y();
    else if (k == "sm_count") *value = h->sm_count;
    else if (k == "tasks_y") *value = h->ntasks_y;
    else return fail(h, EU_ERR_INVALID, "unknown option " + k);
    return EU_OK;
}

int eu_read_planes(eu_handle* h, int which, void* out, size_t bytes, long long* pitch, long long* plane) {
    if (!h || which < 0 || which > 2) return fail(h, EU_ERR_INVALID, "bad argument");
    void* src = which < 2 ? h->S[which] : h->Tm;
    const long long pl = which < 2 ? h->plane_s : h->plane_t;
    if (pitch) *pitch = which < 2 ? h->pitch_s : h->pitch_t;
    if (plane) *plane = pl;
    const size_t need = (size_t)(4 * pl) * h->esz;
    if (!out) return EU_OK;
    if (bytes < need) return fail(h, EU_ERR_INVALID, "buffer too small");
    EU_CUDA(h, cudaMemcpyAsync(out, src, need, cudaMemcpyDeviceToHost, h->st));
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    return EU_OK;
}

int eu_write_planes(eu_handle* h, int which, const void* in, size_t bytes) {
    if (!h || !in || which < 0 || which > 2) return fail(h, EU_ERR_INVALID, "bad argument");
    void* dst = which < 2 ? h->S[which] : h->Tm;
    const long long pl = which < 2 ? h->plane_s : h->plane_t;
    const size_t need = (size_t)(4 * pl) * h->esz;
    if (bytes != need) return fail(h, EU_ERR_INVALID, "eu_write_planes: size must equal the plane set");
    EU_CUDA(h, cudaMemcpyAsync(dst, in, need, cudaMemcpyHostToDevice, h->st));
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    drop_graphs(h);
    return EU_OK;
}

// Binary state file: header, then the Grid2D AoS grid (FP64, ghosts incl.).
struct StateHeader {
    char magic[8];          // "EU2DSTAT"
    int version, nx, ny, prec, solver, bc[4];
    double x_min, x_max, y_min, y_max, t;
    long long step;
};

int eu_save_state(eu_handle* h, const char* path) {
    if (!h || !path) return fail(h, EU_ERR_INVALID, "bad argument");
    Range range_("eu_save_state");
    std::vector<double> aos((size_t)4 * (h->cfg.nx + 4) * (h->cfg.ny + 4));
    if (int rc = eu_download_aos(h, aos.data())) return rc;
    StateHeader hd{};
    std::memcpy(hd.magic, "EU2DSTAT", 8);
    hd.version = 1;
    hd.nx = h->cfg.nx; hd.ny = h->cfg.ny; hd.prec = h->prec; hd.solver = h->solver;
    std::memcpy(hd.bc, h->bc, sizeof(hd.bc));
    hd.x_min = h->cfg.x_min; hd.x_max = h->cfg.x_max; hd.y_min = h->cfg.y_min; hd.y_max = h->cfg.y_max;
    if (int rc = ctl_pull_sync(h)) return rc;
    hd.t = h->hctl->t;
    hd.step = h->hctl->step;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(h, EU_ERR_INVALID, std::string("eu_save_state: cannot open ") + path);
    const bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1 &&
                    std::fwrite(aos.data(), sizeof(double), aos.size(), f) == aos.size();
    const bool closed = std::fclose(f) == 0;
    if (!ok || !closed) return fail(h, EU_ERR_INVALID, std::string("eu_save_state: write failed: ") + path);
    return EU_OK;
}

int eu_load_state(eu_handle* h, const char* path) {
    if (!h || !path) return fail(h, EU_ERR_INVALID, "bad argument");
    Range range_("eu_load_state");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(h, EU_ERR_INVALID, std::string("eu_load_state: cannot open ") + path);
    StateHeader hd{};
    std::vector<double> aos((size_t)4 * (h->cfg.nx + 4) * (h->cfg.ny + 4));
    bool ok = std::fread(&hd, sizeof(hd), 1, f) == 1 && std::memcmp(hd.magic, "EU2DSTAT", 8) == 0 && hd.version == 1 &&
              hd.nx == h->cfg.nx && hd.ny == h->cfg.ny && hd.x_min == h->cfg.x_min && hd.x_max == h->cfg.x_max &&
              hd.y_min == h->cfg.y_min && hd.y_max == h->cfg.y_max;
    if (ok) ok = std::fread(aos.data(), sizeof(double), aos.size(), f) == aos.size();
    std::fclose(f);
    if (!ok) return fail(h, EU_ERR_INVALID, std::string("eu_load_state: not a state file of this grid: ") + path);
    if (int rc = eu_upload_aos(h, aos.data())) return rc;
    ctl_reset(h, kModeHost, INFINITY, LLONG_MAX);
    h->hctl->t = hd.t;
    h->hctl->step = hd.step;
    if (int rc = ctl_push(h)) return rc;
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    return EU_OK;
}

int eu_set_device(int device) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice");
    return EU_OK;
}

int eu_host_alloc(size_t bytes, void** p) {
    if (!p) return fail(nullptr, EU_ERR_INVALID, "null argument");
    cudaError_t e = cudaMallocHost(p, bytes);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaMallocHost");
    return EU_OK;
}

void eu_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

// --- ensemble ------------------------------------------------------------------
int eu_batch_create(int n, const eu_case* cfgs, const int* bcs, eu_precision prec, eu_solver solver, eu_batch** out) {
    if (!out || !cfgs || n < 1 || n > kMaxInst)
        return bfail(nullptr, EU_ERR_INVALID, "eu_batch_create: need 1 <= n <= 256 instances and their cases");
    *out = nullptr;
    eu_batch* b = new eu_batch();
    b->n = n;
    b->prec = prec;
    b->solver = solver;
    auto bail = [&](int rc) {
        if (b->err.empty()) b->err = g_err;
        g_err = b->err;
        eu_batch_destroy(b);
        return rc;
    };
    for (int i = 0; i < n; ++i) {
        eu_handle* h = nullptr;
        const int rc = eu_create(&cfgs[i], prec, solver, EU_LIMITER_MINMOD, bcs ? bcs + 4 * i : nullptr, &h);
        if (rc != EU_OK) {
            b->err = "instance " + std::to_string(i) + ": " + g_err;
            return bail(rc);
        }
        b->h.push_back(h);
    }
    b->K = b->h[0]->K;
    cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
    const size_t isz = prec == EU_FP32 ? sizeof(EnsInst<float>) : sizeof(EnsInst<double>);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_inst, isz * (size_t)n);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_sched, sizeof(EnsSched));
    if (e != cudaSuccess) {
        b->err = std::string("eu_batch_create: ") + cudaGetErrorString(e);
        return bail(EU_ERR_NOMEM);
    }
    b->ctas = b->h[0]->sm_count * b->K.occ_e();
    b->gsteps = 4;
    *out = b;
    return EU_OK;
}

void eu_batch_destroy(eu_batch* b) {
    if (!b) return;
    if (b->st) cudaStreamSynchronize(b->st);
    if (b->g) cudaGraphExecDestroy(b->g);
    for (eu_handle* h : b->h) eu_destroy(h);
    cudaFree(b->d_inst);
    cudaFree(b->d_sched);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
}

const char* eu_batch_last_error(const eu_batch* b) { return b ? b->err.c_str() : g_err.c_str(); }

eu_handle* eu_batch_handle(eu_batch* b, int i) {
    if (!b || i < 0 || i >= b->n) return nullptr;
    b->dirty = true;   // the caller may change options of the instance
    return b->h[(size_t)i];
}

int eu_batch_start(eu_batch* b) {
    if (!b) return bfail(nullptr, EU_ERR_INVALID, "null batch");
    for (int i = 0; i < b->n; ++i) {
        eu_handle* h = b->h[(size_t)i];
        ctl_reset(h, kModeCfl, h->cfg.t_end, LLONG_MAX);
        if (ctl_push(h)) return bfail(b, EU_ERR_CUDA, h->err);
        cudaError_t e = fill_ghosts(h, h->cur);   // scripts/cpu/main_cpu.cpp:222
        if (e == cudaSuccess) e = launch_dt(h, h->cur);
        if (e != cudaSuccess) return bfail(b, EU_ERR_CUDA, std::string("eu_batch_start: ") + cudaGetErrorString(e));
    }
    return batch_pull(b, nullptr);
}

int eu_batch_step(eu_batch* b, long long nsteps, int* all_done) {
    Range range_("eu_batch_step");
    if (!b || nsteps < 0) return bfail(b, EU_ERR_INVALID, "bad argument");
    for (eu_handle* h : b->h)
        if (cudaStreamSynchronize(h->st) != cudaSuccess) return bfail(b, EU_ERR_CUDA, "instance stream failed");
    if (b->dirty)
        if (int rc = batch_build(b)) return rc;
    if (!b->g)
        if (int rc = batch_graph(b, b->gsteps, &b->g)) return rc;
    long long left = nsteps;
    cudaError_t e = cudaSuccess;
    while (left >= b->gsteps && e == cudaSuccess) {
        e = cudaGraphLaunch(b->g, b->st);
        left -= b->gsteps;
    }
    while (left > 0 && e == cudaSuccess) {
        e = batch_launch(b);
        --left;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return bfail(b, EU_ERR_CUDA, std::string("eu_batch_step: ") + cudaGetErrorString(e));
    return batch_pull(b, all_done);
}

int eu_batch_run(eu_batch* b, long long max_steps, long long* steps_taken) {
    if (!b || max_steps < 0) return bfail(b, EU_ERR_INVALID, "bad argument");
    long long done_steps = 0;
    int all = 0;
    while (done_steps < max_steps) {
        const long long k = std::min<long long>(max_steps - done_steps, 64);
        if (int rc = eu_batch_step(b, k, &all)) return rc;
        done_steps += k;
        if (all) break;
    }
    if (steps_taken) *steps_taken = done_steps;
    return EU_OK;
}

int eu_batch_time_steps(eu_batch* b, int nsteps, float* ms) {
    if (!b || !ms || nsteps < 1) return bfail(b, EU_ERR_INVALID, "bad argument");
    for (eu_handle* h : b->h)
        if (cudaStreamSynchronize(h->st) != cudaSuccess) return bfail(b, EU_ERR_CUDA, "instance stream failed");
    if (b->dirty)
        if (int rc = batch_build(b)) return rc;
    cudaGraphExec_t g = nullptr;
    if (int rc = batch_graph(b, nsteps, &g)) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaEventRecord(e0, b->st);
    if (e == cudaSuccess) e = cudaGraphLaunch(g, b->st);
    if (e == cudaSuccess) e = cudaEventRecord(e1, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaGraphExecDestroy(g);
    if (e != cudaSuccess) return bfail(b, EU_ERR_CUDA, std::string("eu_batch_time_steps: ") + cudaGetErrorString(e));
    return batch_pull(b, nullptr);
}

// Ensemble autotuner: one segment pair for all instances (clipped to each
// instance's grid), timed on the whole ensemble step; the instances' states
// and control blocks are restored afterwards.
int eu_batch_autotune(eu_batch* b, int steps, long long chosen[2]) {
    if (!b || steps < 1) return bfail(b, EU_ERR_INVALID, "bad argument");
    const int CX = b->K.box_x, RY = b->K.ry;
    std::vector<void*> saved((size_t)b->n, nullptr);
    std::vector<Ctl> ctl0((size_t)b->n);
    std::vector<int> cur0((size_t)b->n);
    for (int i = 0; i < b->n; ++i) {
        eu_handle* h = b->h[(size_t)i];
        if (cudaStreamSynchronize(h->st) != cudaSuccess || cudaMalloc(&saved[(size_t)i], state_bytes(h)) != cudaSuccess ||
            cudaMemcpy(saved[(size_t)i], h->S[h->cur], state_bytes(h), cudaMemcpyDeviceToDevice) != cudaSuccess) {
            for (void* p : saved) cudaFree(p);
            return bfail(b, EU_ERR_NOMEM, "eu_batch_autotune: state backup failed");
        }
        ctl0[(size_t)i] = *h->hctl;
        cur0[(size_t)i] = h->cur;
    }
    auto restore = [&]() {
        for (int i = 0; i < b->n; ++i) {
            eu_handle* h = b->h[(size_t)i];
            cudaMemcpy(h->S[cur0[(size_t)i]], saved[(size_t)i], state_bytes(h), cudaMemcpyDeviceToDevice);
            h->cur = cur0[(size_t)i];
            *h->hctl = ctl0[(size_t)i];
            if (ctl_push(h) == EU_OK) cudaStreamSynchronize(h->st);
        }
    };
    const int cx[] = {CX, 2 * CX, 32, 64, 128, 256}, cy[] = {RY, 2 * RY, 16, 32, 64, 128};
    float best = INFINITY;
    int bx = cx[2], by = cy[3];
    int rc = EU_OK;
    for (int a = 0; a < 6 && rc == EU_OK; ++a)
        for (int c = 0; c < 6 && rc == EU_OK; ++c) {
            if (cx[a] % CX || cy[c] % RY) continue;
            restore();
            for (eu_handle* h : b->h) {
                const long long sx = std::min<long long>(cx[a], round_up(h->cfg.nx, CX));
                const long long sy = std::min<long long>(cy[c], round_up(h->cfg.ny, RY));
                if ((rc = eu_set_option(h, "seg_x", sx)) || (rc = eu_set_option(h, "seg_y", sy))) break;
            }
            b->dirty = true;
            float ms = 0;
            if (rc == EU_OK) rc = eu_batch_time_steps(b, 2, &ms);
            if (rc == EU_OK) rc = eu_batch_time_steps(b, steps, &ms);
            if (rc == EU_OK && ms < best) { best = ms; bx = cx[a]; by = cy[c]; }
        }
    for (int i = 0; i < b->n && rc == EU_OK; ++i) {
        eu_handle* h = b->h[(size_t)i];
        const long long sx = std::min<long long>(bx, round_up(h->cfg.nx, CX));
        const long long sy = std::min<long long>(by, round_up(h->cfg.ny, RY));
        rc = eu_set_option(h, "seg_x", sx);
        if (rc == EU_OK) rc = eu_set_option(h, "seg_y", sy);
    }
    restore();
    for (void* p : saved) cudaFree(p);
    b->dirty = true;
    if (rc != EU_OK) return rc;
    if (chosen) { chosen[0] = bx; chosen[1] = by; }
    return EU_OK;
}

// Adjoints of every instance, enqueued on the instances' own streams so that
// they run concurrently, then awaited.
int eu_batch_adjoint_forward(eu_batch* b, const long long* nsteps, const double* const* dts, int ckpt_k) {
    if (!b || !nsteps || !dts) return bfail(b, EU_ERR_INVALID, "bad argument");
    if (cudaStreamSynchronize(b->st) != cudaSuccess) return bfail(b, EU_ERR_CUDA, "batch stream failed");
    for (int i = 0; i < b->n; ++i)
        if (int rc = adj_fwd_enqueue(b->h[(size_t)i], nsteps[i], dts[i], ckpt_k))
            return bfail(b, rc, "instance " + std::to_string(i) + ": " + b->h[(size_t)i]->err);
    for (int i = 0; i < b->n; ++i)
        if (int rc = adj_fwd_finish(b->h[(size_t)i]))
            return bfail(b, rc, "instance " + std::to_string(i) + ": " + b->h[(size_t)i]->err);
    return EU_OK;
}

int eu_batch_adjoint_backward(eu_batch* b, const double* const* dJ_dUN, double* const* dJ_dU0) {
    if (!b || !dJ_dUN || !dJ_dU0) return bfail(b, EU_ERR_INVALID, "bad argument");
    for (int i = 0; i < b->n; ++i)
        if (int rc = adj_bwd_enqueue(b->h[(size_t)i], dJ_dUN[i], dJ_dU0[i]))
            return bfail(b, rc, "instance " + std::to_string(i) + ": " + b->h[(size_t)i]->err);
    for (int i = 0; i < b->n; ++i)
        if (int rc = adj_bwd_finish(b->h[(size_t)i], dJ_dU0[i]))
            return bfail(b, rc, "instance " + std::to_string(i) + ": " + b->h[(size_t)i]->err);
    return EU_OK;
}

// Test hook of the failure-detection path: with n > 0 every y-sweep task
// waits for n more x-sweep tasks than exist -- a count nothing reaches -- so
// its bounded wait expires (2 s), the instance's status records the
// time-out and eu_batch_step returns EU_ERR_TIMEOUT with the context intact.
int eu_batch_set_wait_extra(eu_batch* b, int n) {
    if (!b || n < 0) return bfail(b, EU_ERR_INVALID, "bad argument");
    b->wait_extra = n;
    b->dirty = true;
    return EU_OK;
}

}  // extern "C"
