// runtime.cpp -- the host runtime's shared machinery: tensor maps, work
// decomposition, kernel launches, the device control block, CUDA graphs of
// whole steps and the host <-> device transfers of Grid2D states.
#include "runtime.h"

using namespace eu;

namespace eu {
namespace __attribute__((visibility("hidden"))) rt {

thread_local std::string g_err;

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

CUtensorMapL2promotion promo_of(int bytes) {
    switch (bytes) {
        case 0: return CU_TENSOR_MAP_L2_PROMOTION_NONE;
        case 64: return CU_TENSOR_MAP_L2_PROMOTION_L2_64B;
        case 128: return CU_TENSOR_MAP_L2_PROMOTION_L2_128B;
        default: return CU_TENSOR_MAP_L2_PROMOTION_L2_256B;
    }
}

int encode(eu_handle* h, CUtensorMap* m, void* base, long long width, long long pitch, long long plane,
           int box_w, int box_h, CUtensorMapSwizzle swz, int promo, long long height) {
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
        if (int rc = encode(h, &h->tm_yo[b], h->S[b], wclip_of(h), h->pitch_s, h->plane_s, 32, kYLag,
                            CU_TENSOR_MAP_SWIZZLE_NONE, 256))
            return rc;
    if (int rc = encode(h, &h->tm_y, h->Tm, h->pitch_t, h->pitch_t, h->plane_t, h->K.box_w_y, h->K.ry,
                        CU_TENSOR_MAP_SWIZZLE_NONE, h->l2promo_y))
        return rc;
    h->tm_y_ry = h->K.ry;
    return EU_OK;
}

// Work decomposition.  A task is a segment of one group of 32 lines (the
// x-sweep runs one per warp, the y-sweep's warps take them from a work
// list).  Measured on GB300 (8192^2 and 2048^2, FP32 HLLC), launches of many
// short tasks beat near-single-wave launches of long ones even though each
// task recomputes a 4-cell warm-up (plus one box in the x-sweep): CTAs refill
// the SMs as they retire, the tail shrinks to one short task, and fewer
// lines are in flight at once.  The default aims at about eight tasks per
// resident warp slot with segments clamped to [32, 128] rows (y) and
// [32, 256] columns (x).  The FP32 exact solver is the exception: its faces
// on and near waves run the Newton iteration for p* (with an FP64 step)
// while the rest take the identical-states route, so a step lasts about as
// long as the warps whose lines run along a wave, and short tasks shorten
// that critical path.  It aims at about 64 tasks per slot with segments
// down to 8 rows and 16 columns (blast, ms per step: 8192^2 3.2 -> 2.3,
// 2048^2 0.76 -> 0.64).  The FP64 exact solver is bound by the FP64 pipe
// throughout and keeps the default.  eu_set_option overrides the plan.
void plan(eu_handle* h) {
    const int nx = h->cfg.nx, ny = h->cfg.ny;
    const bool fine = h->solver == EU_EXACT && h->prec == EU_FP32;
    const long long per_slot = fine ? 64 : 8;
    const long long min_x = fine ? 16 : 32, min_y = fine ? 8 : 32;
    const long long slots_x = (long long)h->sm_count * h->K.nw * h->K.occ_x();
    const long long slots_y = (long long)h->sm_count * h->K.nw * h->K.occ_y();
    const int CX = h->K.box_x;
    const int rgroups = (ny + 31) / 32;
    long long want = ((long long)rgroups * nx + per_slot * slots_x - 1) / (per_slot * slots_x);
    want = std::min<long long>(std::max<long long>(want, min_x), 256);
    int seg = (int)round_up(std::min<long long>(want, nx), CX);
    h->seg_x = seg;
    h->nseg_x = (nx + seg - 1) / seg;
    h->ntasks_x = rgroups * h->nseg_x;
    h->ctas_x = (h->ntasks_x + h->K.nw - 1) / h->K.nw;
    const int groups = (nx + kSOff + 31) / 32;
    want = ((long long)groups * ny + per_slot * slots_y - 1) / (per_slot * slots_y);
    want = std::min<long long>(std::max<long long>(want, min_y), 128);
    // whole output boxes; with 8-row input boxes a segment of 8m + 4 rows
    // (+ 4 warm-up rows) fills its last box (8192^2 HLLC: 116 rows 0.525 ms,
    // 112 rows 0.534 ms per y-sweep)
    if (h->K.ry > kYLag && !fine) want = round_up(std::max<long long>(want - kYLag, 1), h->K.ry) + kYLag;
    h->seg_y = (int)round_up(std::min<long long>(want, ny), kYLag);
    h->nseg_y = groups;  // tasks per row segment
    h->ntasks_y = groups * ((ny + h->seg_y - 1) / h->seg_y);
    h->ctas_y = (h->ntasks_y + h->K.nw - 1) / h->K.nw;
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
    // a box of other rows than the kernel's stage buffers would overrun them
    if (h->tm_y_ry != h->K.ry) return cudaErrorInvalidValue;
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

size_t state_bytes(const eu_handle* h) { return (size_t)(4 * h->plane_s) * h->esz; }
size_t tmp_bytes(const eu_handle* h) { return (size_t)(4 * h->plane_t) * h->esz; }

}  // namespace rt

void set_global_error(const char* msg) { rt::g_err = msg; }

}  // namespace eu
