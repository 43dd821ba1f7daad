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
        if (h->tm_y_ry != b->K.ry) return bfail(b, EU_ERR_INVALID, "ensemble: an instance's y map has another box height");
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

namespace {
bool batch_adj_shared(const eu_batch* b);
int batch_adj_steps(eu_batch* b);
}  // namespace

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
    cudaFree(b->d_adj);
    if (b->adj_ev) cudaEventDestroy(b->adj_ev);
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
    const int CX = b->K.box_x, RY = kYLag;        // y segments: whole output boxes
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

// Checkpointed forwards of every instance: set up on the instances' own
// streams, the steps as shared ensemble launches (or each instance's own
// launches), then awaited.  The backwards (next) run on the instances' own
// streams, concurrently.
int eu_batch_adjoint_forward(eu_batch* b, const long long* nsteps, const double* const* dts, int ckpt_k) {
    if (!b || !nsteps) return bfail(b, EU_ERR_INVALID, "bad argument");
    if (cudaStreamSynchronize(b->st) != cudaSuccess) return bfail(b, EU_ERR_CUDA, "batch stream failed");
    const int K = ckpt_k == 0 ? adj_auto_k(b->h.data(), nsteps, b->n) : ckpt_k;
    for (int i = 0; i < b->n; ++i)
        if (int rc = adj_fwd_setup(b->h[(size_t)i], nsteps[i], dts ? dts[i] : nullptr,
                                   ckpt_k == 0 ? (int)std::min<long long>(K, std::max(1LL, nsteps[i])) : ckpt_k,
                                   b->h[(size_t)i]->cfg.t_end))
            return bfail(b, rc, "instance " + std::to_string(i) + ": " + b->h[(size_t)i]->err);
    if (batch_adj_shared(b)) {
        if (int rc = batch_adj_steps(b)) return rc;
    } else {
        for (int i = 0; i < b->n; ++i)
            if (int rc = adj_fwd_steps(b->h[(size_t)i]))
                return bfail(b, rc, "instance " + std::to_string(i) + ": " + b->h[(size_t)i]->err);
    }
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

// ---------------------------------------------------------------------------
// Batched gradients with respect to scalar case parameters, device-resident
// ---------------------------------------------------------------------------
#include <atomic>
#include <thread>

#include "grad_kernels.h"

namespace {

// Host-side derived values of one instance's parameters (see ParamState).
ParamState param_state(const eu_handle* h, const eu_case_params& p) {
    ParamState d{};
    d.kind = p.kind;
    for (int k = 0; k < 8; ++k) d.v[k] = p.v[k];
    d.h = std::min(h->dx, h->dy);
    if (p.kind == 1) {   // Rankine-Hugoniot post-shock state and its Mach derivatives (src/test_cases.cpp:35-46)
        const double g = kGammaD, rho0 = p.v[0], p0 = p.v[1], M = p.v[2], M2 = M * M;
        const double a0 = std::sqrt(g * p0 / rho0);
        const double den = (g - 1.0) * M2 + 2.0;
        d.ps[0] = rho0 * (g + 1.0) * M2 / den;
        d.ps[1] = 2.0 * a0 / (g + 1.0) * (M - 1.0 / M);
        d.ps[2] = p0 * (1.0 + 2.0 * g / (g + 1.0) * (M2 - 1.0));
        d.ps[3] = rho0 * (g + 1.0) * 4.0 * M / (den * den);
        d.ps[4] = 2.0 * a0 / (g + 1.0) * (1.0 + 1.0 / M2);
        d.ps[5] = p0 * 2.0 * g / (g + 1.0) * 2.0 * M;
    }
    return d;
}

template <class T> cudaError_t init_params_t(eu_handle* h, const ParamState& d) {
    return launch_init_param<T>(planes_s<T>(h, h->cur), h->cfg.nx, h->cfg.ny, h->cfg.x_min, h->cfg.y_min, h->dx,
                                h->dy, d, h->st);
}

// Objective and dJ/dU_N into the adjoint buffer, the backward sweeps, and the
// tangent contraction; results (J, dJ/dtheta_0, dJ/dtheta_1) at d_out.
template <class T> int grad_tail_t(eu_handle* h, const ParamState& d, double* d_out) {
    auto& A = h->adj;
    const Planes<T> L{static_cast<T*>(A.lam), h->pitch_s, h->plane_s};
    EU_CUDA(h, cudaMemsetAsync(A.lam, 0, state_bytes(h), h->st));
    EU_CUDA(h, launch_objective<T>(planes_s<T>(h, h->cur), L, h->cfg.nx, h->cfg.ny, h->cfg.x_min, h->cfg.y_min,
                                   h->dx, h->dy, d, h->d_part, h->part_blocks, d_out, h->st));
    if (int rc = adj_bwd_sweeps(h)) return rc;
    EU_CUDA(h, launch_tangent_dot<T>(L, h->cfg.nx, h->cfg.ny, h->cfg.x_min, h->cfg.y_min, h->dx, h->dy, d, h->d_part,
                                     h->part_blocks, d_out + 1, h->st));
    return EU_OK;
}

// Runs f(i) for i in [0, n) on up to `threads` host threads; the first
// failing instance's code is returned.
template <class F> int for_instances(int n, int threads, F f) {
    std::atomic<int> next{0}, rc{EU_OK};
    auto work = [&]() {
        for (int i = next++; i < n; i = next++) {
            const int r = f(i);
            int ok = EU_OK;
            if (r != EU_OK) rc.compare_exchange_strong(ok, r);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
    return rc.load();
}

#define B_CUDA(call)                                                                              \
    do {                                                                                          \
        const cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) return bfail(b, EU_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

// Device scratch of the batch's shared adjoint launches (grown, not shrunk).
int batch_adj_scratch(eu_batch* b, size_t bytes) {
    if (!b->adj_ev) B_CUDA(cudaEventCreateWithFlags(&b->adj_ev, cudaEventDisableTiming));
    if (bytes <= b->adj_cap) return EU_OK;
    B_CUDA(cudaStreamSynchronize(b->st));
    cudaFree(b->d_adj);
    b->d_adj = nullptr;
    b->adj_cap = 0;
    B_CUDA(cudaMalloc(&b->d_adj, bytes));
    b->adj_cap = bytes;
    return EU_OK;
}

// Whether the instances' adjoint steps can share launches: every instance
// on the batch's solver, with its y boxes (and its adjoint ring's) of the
// batch kernel's height.
bool batch_adj_shared(const eu_batch* b) {
    for (const eu_handle* h : b->h)
        if (h->solver != b->solver || h->tm_y_ry != b->K.ry || h->adj.q_y_ry != b->K.ry) return false;
    return b->ctas > 0;
}

// The forward steps of every instance's checkpointed forward (each set up by
// adj_fwd_setup on its own stream), as one ensemble launch per step on the
// batch stream: step s of instance i runs from the descriptors of its ring
// (adj_ens_inst), the ensemble kernel computing each tile as the single-grid
// kernels do.  An instance with fewer steps sits out the later launches
// (its control block is done), as in eu_batch_step.
template <class T> int batch_adj_steps_t(eu_batch* b) {
    const int n = b->n;
    long long nmax = 0;
    for (eu_handle* h : b->h) nmax = std::max(nmax, h->adj.nsteps);
    const size_t bytes = sizeof(EnsInst<T>) * (size_t)nmax * (size_t)n;
    if (int rc = batch_adj_scratch(b, bytes)) return rc;
    for (eu_handle* h : b->h) {
        B_CUDA(cudaEventRecord(h->adj.ev[4], h->st));
        B_CUDA(cudaStreamWaitEvent(b->st, h->adj.ev[4], 0));
    }
    std::vector<EnsInst<T>> tab((size_t)nmax * (size_t)n);
    EnsArgs<T> E;
    std::memset(&E, 0, sizeof(E));
    E.sched = b->d_sched;
    E.ninst = n;
    int tx = 0, ty = 0;
    for (int i = 0; i < n; ++i) {
        const eu_handle* h = b->h[(size_t)i];
        E.x_off[i] = tx;
        E.y_off[i] = ty;
        tx += h->ntasks_x;
        ty += h->ntasks_y;
        for (long long st = 0; st < nmax; ++st)
            tab[(size_t)st * n + i] = adj_ens_inst<T>(h, std::min(st, h->adj.nsteps - 1));
    }
    E.x_off[n] = tx;
    E.y_off[n] = ty;
    E.total_x = tx;
    E.total_y = ty;
    B_CUDA(cudaMemcpyAsync(b->d_adj, tab.data(), bytes, cudaMemcpyHostToDevice, b->st));
    for (long long st = 0; st < nmax; ++st) {
        E.inst = static_cast<const EnsInst<T>*>(b->d_adj) + (size_t)st * n;
        B_CUDA(cudaMemsetAsync(b->d_sched, 0, sizeof(EnsSched), b->st));
        B_CUDA(b->K.ens(&E, b->ctas, b->st));
    }
    B_CUDA(cudaEventRecord(b->adj_ev, b->st));
    for (eu_handle* h : b->h) {
        B_CUDA(cudaStreamWaitEvent(h->st, b->adj_ev, 0));
        if (int rc = adj_fwd_done(h)) return rc;
    }
    return EU_OK;
}
int batch_adj_steps(eu_batch* b) {
    return b->prec == EU_FP32 ? batch_adj_steps_t<float>(b) : batch_adj_steps_t<double>(b);
}

}  // namespace

extern "C" {

int eu_init_params(eu_handle* h, const eu_case_params* p) {
    if (!h || !p || (p->kind != 0 && p->kind != 1)) return fail(h, EU_ERR_INVALID, "eu_init_params: bad argument");
    const ParamState d = param_state(h, *p);
    EU_CUDA(h, h->prec == EU_FP32 ? init_params_t<float>(h, d) : init_params_t<double>(h, d));
    ctl_reset(h, kModeHost, INFINITY, LLONG_MAX);
    if (int rc = ctl_push(h)) return rc;
    drop_graphs(h);
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    return EU_OK;
}

int eu_batch_param_gradients(eu_batch* b, const eu_case_params* params, const long long* nsteps,
                             const double* const* dts, int ckpt_k, double* J, double* dJ) {
    Range range_("eu_batch_param_gradients");
    if (!b || !params || !nsteps || !J || !dJ) return bfail(b, EU_ERR_INVALID, "bad argument");
    for (int i = 0; i < b->n; ++i)
        if (params[i].kind != 0 && params[i].kind != 1) return bfail(b, EU_ERR_INVALID, "bad parameter kind");
    if (cudaStreamSynchronize(b->st) != cudaSuccess) return bfail(b, EU_ERR_CUDA, "batch stream failed");
    double *d_res = nullptr, *h_res = nullptr;
    if (cudaMalloc(&d_res, sizeof(double) * 3 * (size_t)b->n) != cudaSuccess ||
        cudaMallocHost(&h_res, sizeof(double) * 3 * (size_t)b->n) != cudaSuccess) {
        (void)cudaGetLastError();
        cudaFree(d_res);
        return bfail(b, EU_ERR_NOMEM, "eu_batch_param_gradients: result buffers");
    }
    std::vector<ParamState> ps;
    for (int i = 0; i < b->n; ++i) ps.push_back(param_state(b->h[(size_t)i], params[i]));
    const unsigned hw = std::thread::hardware_concurrency();
    const int threads = (int)std::max(1u, std::min(8u, hw ? hw : 1u));
    const int K = ckpt_k == 0 ? adj_auto_k(b->h.data(), nsteps, b->n) : ckpt_k;
    // 1. every instance's initial state and forward set-up, enqueued
    int rc = for_instances(b->n, threads, [&](int i) {
        eu_handle* h = b->h[(size_t)i];
        ctl_reset(h, kModeHost, INFINITY, LLONG_MAX);
        if (int r = ctl_push(h)) return r;
        drop_graphs(h);
        const cudaError_t e = h->prec == EU_FP32 ? init_params_t<float>(h, ps[(size_t)i]) : init_params_t<double>(h, ps[(size_t)i]);
        if (e != cudaSuccess) return cuda_fail(h, e, "parameter initial state");
        const int k = ckpt_k == 0 ? (int)std::min<long long>(K, std::max(1LL, nsteps[i])) : ckpt_k;
        return adj_fwd_setup(h, nsteps[i], dts ? dts[i] : nullptr, k, h->cfg.t_end);
    });
    // 2. the forward steps: one ensemble launch per step when the instances
    //    can share launches, else each instance's own segment launches
    bool batch_err = false;
    if (rc == EU_OK) {
        if (batch_adj_shared(b)) {
            rc = batch_adj_steps(b);
            batch_err = rc != EU_OK;
        } else {
            rc = for_instances(b->n, threads, [&](int i) { return adj_fwd_steps(b->h[(size_t)i]); });
        }
    }
    // 3. as each forward completes: objective, dJ/dU_N, backward sweeps and
    //    tangent contraction on the instance's own stream (the adjoint
    //    sweeps of many grids run faster as concurrent per-grid launches
    //    than as shared launches over all of them)
    if (rc == EU_OK)
        rc = for_instances(b->n, threads, [&](int i) {
            eu_handle* h = b->h[(size_t)i];
            if (int r = adj_fwd_finish(h)) return r;
            const int r = h->prec == EU_FP32 ? grad_tail_t<float>(h, ps[(size_t)i], d_res + 3 * i)
                                             : grad_tail_t<double>(h, ps[(size_t)i], d_res + 3 * i);
            if (r) return r;
            EU_CUDA(h, cudaMemcpyAsync(h_res + 3 * i, d_res + 3 * i, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                                       h->st));
            return (int)EU_OK;
        });
    if (cudaStreamSynchronize(b->st) != cudaSuccess && rc == EU_OK) {
        rc = bfail(b, EU_ERR_CUDA, std::string("batch stream: ") + cudaGetErrorString(cudaGetLastError()));
        batch_err = true;
    }
    for (int i = 0; i < b->n; ++i) {
        eu_handle* h = b->h[(size_t)i];
        if (cudaStreamSynchronize(h->st) != cudaSuccess && rc == EU_OK) rc = cuda_fail(h, cudaGetLastError(), "sync");
        if (rc == EU_OK) cudaEventElapsedTime(&h->adj.ms_bwd, h->adj.ev[2], h->adj.ev[3]);
    }
    if (rc == EU_OK)
        for (int i = 0; i < b->n; ++i) {
            J[i] = h_res[3 * i];
            dJ[2 * i] = h_res[3 * i + 1];
            dJ[2 * i + 1] = h_res[3 * i + 2];
        }
    cudaFree(d_res);
    cudaFreeHost(h_res);
    if (rc != EU_OK) {
        if (batch_err) return rc;
        for (int i = 0; i < b->n; ++i)
            if (!b->h[(size_t)i]->err.empty()) return bfail(b, rc, "instance " + std::to_string(i) + ": " + b->h[(size_t)i]->err);
        return bfail(b, rc, "eu_batch_param_gradients failed");
    }
    return EU_OK;
}

}  // extern "C"
