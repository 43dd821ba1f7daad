// api_batch.cpp -- ensembles of independent grids (instances with their
// own sizes, boundaries, parameters and dt) advanced by one persistent
// launch per step (csrc/sweeps.cuh, ensemble_kernel), and their batched
// adjoint.
#include "runtime.h"

using namespace eu;

namespace eu {
namespace __attribute__((visibility("hidden"))) rt {

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

}  // namespace rt
}  // namespace eu

using namespace eu::rt;

extern "C" {

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
