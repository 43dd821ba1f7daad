// api_adjoint.cpp -- discrete adjoint of the split step behind
// eu_adjoint_forward / eu_adjoint_backward: checkpoints every k steps, one
// ring segment of recomputed forward states, and the adjoint x/y sweeps
// (csrc/adjoint.cuh) run backwards through it.
#include "runtime.h"

using namespace eu;

namespace eu {
namespace __attribute__((visibility("hidden"))) rt {

// ---------------------------------------------------------------------------
// discrete adjoint: buffers, forward segments, adjoint sweeps
// ---------------------------------------------------------------------------
AdjLaunch adj_launcher(int prec, int solver) {
    static const AdjLaunch f32[4] = {adjoint_sweep_32_0, adjoint_sweep_32_1, adjoint_sweep_32_2, adjoint_sweep_32_3};
    static const AdjLaunch f64[4] = {adjoint_sweep_64_0, adjoint_sweep_64_1, adjoint_sweep_64_2, adjoint_sweep_64_3};
    return prec == EU_FP32 ? f32[solver] : f64[solver];
}

// TMA maps of a state buffer (x-sweep input, y-sweep output) and of an
// x-sweep output buffer (x-sweep output, y-sweep input), as encode_all.
int enc_state(eu_handle* h, void* b, CUtensorMap* xin, CUtensorMap* yout) {
    if (int rc = encode(h, xin, b, h->cfg.nx + kSOff + 2, h->pitch_s, h->plane_s, h->K.box_x, 32,
                        CU_TENSOR_MAP_SWIZZLE_32B, h->l2promo_x))
        return rc;
    return encode(h, yout, b, wclip_of(h), h->pitch_s, h->plane_s, 32, kYLag, CU_TENSOR_MAP_SWIZZLE_NONE, 256);
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

// Device bytes of the adjoint buffers for nsteps steps at spacing k
// (adj_prepare), and of those the handle holds now.
size_t adj_bytes(const eu_handle* h, long long nsteps, int k) {
    const size_t nseg = (size_t)((nsteps + k - 1) / k);
    return (nseg + 1 + (size_t)(k - 1) + 2) * state_bytes(h) + (size_t)k * tmp_bytes(h);
}
size_t adj_held_bytes(const eu_handle* h) {
    const auto& A = h->adj;
    if (A.ck.empty()) return 0;
    return (A.ck.size() + A.R.size() - 1 + 2) * state_bytes(h) + A.Q.size() * tmp_bytes(h);
}

// Checkpoint spacing for ckpt_k = 0 over n handles: every step's state
// resident (one segment each, nothing recomputed by the backward) when all
// the handles' buffers fit in half of the device memory that is free or
// already theirs, else ceil(sqrt(max nsteps)) (each segment recomputed once).
// Handle i then uses min(k, nsteps[i]).
int adj_auto_k(eu_handle* const* hs, const long long* nsteps, int n) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        (void)cudaGetLastError();
        free_b = 0;
    }
    long long nmax = 1;
    size_t need = 0, held = 0;
    for (int i = 0; i < n; ++i) {
        const long long s = std::max(1LL, nsteps[i]);
        nmax = std::max(nmax, s);
        need += adj_bytes(hs[i], s, (int)std::min<long long>(s, kMaxCkptK));
        held += adj_held_bytes(hs[i]);
    }
    if (need <= (free_b + held) / 2) return (int)std::min<long long>(nmax, kMaxCkptK);
    return (int)std::min<long long>(kMaxCkptK, (long long)std::ceil(std::sqrt((double)nmax)));
}

// Buffers for nsteps steps with checkpoints every k steps.
int adj_prepare(eu_handle* h, long long nsteps, int k) {
    auto& A = h->adj;
    const int nseg = (int)((nsteps + k - 1) / k);
    if (A.k != k || (int)A.ck.size() < nseg + 1) {
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
        A.q_y_ry = h->K.ry;
    }
    if (A.q_y_ry != h->K.ry) {   // the solver changed since the ring was built: boxes of other heights
        for (int j = 0; j < k; ++j)
            if (int rc = enc_tmp(h, A.Q[j], &A.Q_xo[j], &A.Q_y[j])) return rc;
        A.q_y_ry = h->K.ry;
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

// Control block of a frozen-dt forward from step s*k (pinned image hctl[s]).
cudaError_t adj_push_frozen(eu_handle* h, int s) {
    auto& A = h->adj;
    const long long n0 = (long long)s * A.k;
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
    return cudaMemcpyAsync(h->ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, h->st);
}

// Forward steps s*k .. s*k+len-1 from ck[s]: the x-sweep of step j writes
// Q[j], the y-sweep writes R[j+1] (ck[s+1] for the last).  With `frozen`
// the segment starts a control block that steps with the dt list d_dts;
// otherwise it continues the control block on the device (the CFL forward,
// whose y-sweeps choose and log each next dt).
template <class T> cudaError_t adj_segment_t(eu_handle* h, int s, bool frozen) {
    auto& A = h->adj;
    if (A.q_y_ry != h->K.ry) return cudaErrorInvalidValue;   // see launch_y
    const long long n0 = (long long)s * A.k;
    const int len = (int)std::min<long long>(A.k, A.nsteps - n0);
    cudaError_t e = cudaSuccess;
    if (frozen) e = adj_push_frozen(h, s);
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
cudaError_t adj_segment(eu_handle* h, int s, bool frozen = true) {
    return h->prec == EU_FP32 ? adj_segment_t<float>(h, s, frozen) : adj_segment_t<double>(h, s, frozen);
}

// Arguments of the adjoint sweeps of step n = s*k + j (the ring holds
// segment s): dir 1, the y-sweep adjoint lam -> mu on the x-sweep output
// Q[j]; dir 0, the x-sweep adjoint mu -> lam on the step's input state.
AdjSweepArgs adj_step_args(const eu_handle* h, int s, int j, int dir) {
    const auto& A = h->adj;
    const long long n = (long long)s * A.k + j;
    AdjSweepArgs a{};
    if (dir == 1) {
        a.P = A.Q[j]; a.p_pitch = h->pitch_t; a.p_plane = h->plane_t; a.p_coff = kTOff;
        a.A = A.lam; a.G = A.mu;
        a.lam_d = A.dts[n] / h->dy;
        a.bc_lo = h->bc[EU_SIDE_BOTTOM]; a.bc_hi = h->bc[EU_SIDE_TOP];
    } else {
        a.P = j == 0 ? A.ck[s] : A.R[j]; a.p_pitch = h->pitch_s; a.p_plane = h->plane_s; a.p_coff = kSOff;
        a.A = A.mu; a.G = A.lam;
        a.lam_d = A.dts[n] / h->dx;
        a.bc_lo = h->bc[EU_SIDE_LEFT]; a.bc_hi = h->bc[EU_SIDE_RIGHT];
    }
    a.a_pitch = h->pitch_s; a.a_plane = h->plane_s; a.a_coff = kSOff;
    a.g_pitch = h->pitch_s; a.g_plane = h->plane_s; a.g_coff = kSOff;
    a.nx = h->cfg.nx; a.ny = h->cfg.ny;
    return a;
}

cudaError_t adj_step(eu_handle* h, int s, int j) {
    const AdjLaunch L = adj_launcher(h->prec, h->solver);
    cudaError_t e = L(1, adj_step_args(h, s, j, 1), h->st);
    if (e != cudaSuccess) return e;
    return L(0, adj_step_args(h, s, j, 0), h->st);
}

// The ensemble kernel's view of forward step n of the handle's checkpointed
// forward (as adj_segment_t launches it): x-sweep from ck[s] or R[j] into
// Q[j], y-sweep from Q[j] into R[j+1] (ck[s+1] for a segment's last step),
// the same buffers whichever state buffer the control block names.
template <class T> EnsInst<T> adj_ens_inst(const eu_handle* h, long long n) {
    const auto& A = h->adj;
    const int s = (int)(n / A.k), j = (int)(n % A.k);
    const int len = (int)std::min<long long>(A.k, A.nsteps - (long long)s * A.k);
    const bool last = j == len - 1;
    EnsInst<T> I;
    std::memset(&I, 0, sizeof(I));
    I.tm_x[0] = I.tm_x[1] = j == 0 ? A.ck_x[s] : A.R_x[j];
    I.tm_xo = A.Q_xo[j];
    I.tm_y = A.Q_y[j];
    I.tm_yo[0] = I.tm_yo[1] = last ? A.ck_yo[s + 1] : A.R_yo[j + 1];
    I.xa = x_args<T>(h, 0);
    I.xa.out = Planes<T>{static_cast<T*>(A.Q[j]), h->pitch_t, h->plane_t};
    I.xa.snap = nullptr;
    I.ya[0] = y_args<T>(h, 0);
    I.ya[0].out = Planes<T>{static_cast<T*>(last ? A.ck[s + 1] : A.R[j + 1]), h->pitch_s, h->plane_s};
    I.ya[0].out_index = 0;
    I.ya[1] = I.ya[0];
    return I;
}
template EnsInst<float> adj_ens_inst<float>(const eu_handle*, long long);
template EnsInst<double> adj_ens_inst<double>(const eu_handle*, long long);

// The checkpointed forward, in three parts so that an ensemble can run the
// steps of all its instances in shared launches: adj_fwd_setup (buffers,
// checkpoint 0 and the control block of the first step), the steps
// (adj_segment per segment, or the ensemble kernel over adj_ens_inst
// descriptors), adj_fwd_done (timing event, control-block probe).  All on
// the handle's stream; no host wait.
// With a dt list the steps use it; without one (dts null) they take CFL
// steps as eu_step_n does -- the first dt from the initial state, each next
// one from the y-sweep's reduction, clipped to t_end -- and log them into
// d_dts, so that the backward replays exactly the steps taken.  A CFL
// forward stops early once t reaches t_end (adj_fwd_finish trims it).
int adj_fwd_setup(eu_handle* h, long long nsteps, const double* dts, int ckpt_k, double t_end) {
    if (!h) return fail(nullptr, EU_ERR_INVALID, "null handle");
    if (nsteps < 1) return fail(h, EU_ERR_INVALID, "eu_adjoint_forward: need nsteps >= 1");
    if (ckpt_k < 0 || ckpt_k > kMaxCkptK) return fail(h, EU_ERR_INVALID, "eu_adjoint_forward: ckpt_k must be in [0, 1024]");
    if (h->cfg.nx < 2 || h->cfg.ny < 2) return fail(h, EU_ERR_INVALID, "eu_adjoint_forward: the adjoint needs nx, ny >= 2");
    if (dts)
        for (long long i = 0; i < nsteps; ++i)
            if (!(dts[i] > 0.0) || !(dts[i] < INFINITY))
                return fail(h, EU_ERR_INVALID, "eu_adjoint_forward: every dt must be positive and finite");
    if (ckpt_k == 0) ckpt_k = (int)std::min<long long>(adj_auto_k(&h, &nsteps, 1), nsteps);
    auto& A = h->adj;
    A.ready = false;
    if (int rc = adj_prepare(h, nsteps, ckpt_k)) return rc;
    A.cfl = dts == nullptr;
    A.t0 = h->hctl->t;
    A.step0 = h->hctl->step;
    if (A.cfl) {
        A.dts.clear();
    } else {
        A.dts.assign(dts, dts + nsteps);
        EU_CUDA(h, cudaMemcpyAsync(A.d_dts, A.dts.data(), sizeof(double) * (size_t)nsteps, cudaMemcpyHostToDevice, h->st));
    }
    EU_CUDA(h, fill_ghosts(h, h->cur));   // scripts/cpu/main_cpu.cpp:222
    EU_CUDA(h, cudaMemcpyAsync(A.ck[0], h->S[h->cur], state_bytes(h), cudaMemcpyDeviceToDevice, h->st));
    EU_CUDA(h, cudaEventRecord(A.ev[0], h->st));
    if (A.cfl) {
        Ctl& c = A.hctl[0];
        std::memset(&c, 0, sizeof(Ctl));
        c.t = A.t0;
        c.t_end = t_end;
        c.cfl_dmin = h->cfg.cfl * std::min(h->dx, h->dy);
        c.mode = kModeCfl;
        c.max_steps = nsteps;
        c.dt_log = A.d_dts;
        c.dt_log_cap = nsteps;
        EU_CUDA(h, cudaMemcpyAsync(h->ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, h->st));
        EU_CUDA(h, launch_dt(h, h->cur));   // scripts/cpu/main_cpu.cpp:224
    } else {
        EU_CUDA(h, adj_push_frozen(h, 0));
    }
    return EU_OK;
}

int adj_fwd_done(eu_handle* h) {
    auto& A = h->adj;
    EU_CUDA(h, cudaEventRecord(A.ev[1], h->st));
    A.ring_seg = A.nseg - 1;
    EU_CUDA(h, cudaMemcpyAsync(&A.hctl[A.nseg], h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
    return EU_OK;
}

int adj_fwd_steps(eu_handle* h) {
    auto& A = h->adj;
    // segment 0's control block comes from adj_fwd_setup; a frozen forward
    // restarts it at each later segment, a CFL forward carries it on
    for (int s = 0; s < A.nseg; ++s) EU_CUDA(h, adj_segment(h, s, !A.cfl && s > 0));
    return adj_fwd_done(h);
}

int adj_fwd_enqueue(eu_handle* h, long long nsteps, const double* dts, int ckpt_k, double t_end) {
    if (int rc = adj_fwd_setup(h, nsteps, dts, ckpt_k, t_end)) return rc;
    return adj_fwd_steps(h);
}

// Wait for the forward; status, timing, the dt list of a CFL forward (and
// its length, when it reached t_end early), the final state into the
// handle's state buffer, the handle's time and step.
int adj_fwd_finish(eu_handle* h) {
    auto& A = h->adj;
    EU_CUDA(h, cudaStreamSynchronize(h->st));
    EU_CUDA(h, cudaEventElapsedTime(&A.ms_fwd, A.ev[0], A.ev[1]));
    const Ctl probe = A.hctl[A.nseg];
    if (probe.status & kStatusTimeout) return fail(h, EU_ERR_TIMEOUT, "a bounded device wait expired");
    if (probe.status & kStatusNonFinite) return fail(h, EU_ERR_NONPHYSICAL, "non-finite state in the forward steps");
    if (probe.status & kStatusNonPhysical)
        return fail(h, EU_ERR_NONPHYSICAL, "compute_dt: non-positive maximum wave speed.");
    void* fin = A.ck[A.nseg];
    if (A.cfl) {
        const long long n = probe.step;
        if (n < 1 || n > A.nsteps) return fail(h, EU_ERR_STATE, "eu_adjoint_forward: no step before t_end");
        A.dts.resize((size_t)n);
        EU_CUDA(h, cudaMemcpyAsync(A.dts.data(), A.d_dts, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, h->st));
        EU_CUDA(h, cudaStreamSynchronize(h->st));
        if (n < A.nsteps) {
            // the launches after step n found the control block done; the
            // ring holds segment s up to its step j
            const int s = (int)((n - 1) / A.k), j = (int)((n - 1) % A.k);
            fin = j == A.k - 1 ? A.ck[s + 1] : A.R[j + 1];
            A.nsteps = n;
            A.nseg = s + 1;
            A.ring_seg = s;
        }
    }
    EU_CUDA(h, cudaMemcpyAsync(h->S[h->cur], fin, state_bytes(h), cudaMemcpyDeviceToDevice, h->st));
    double t = A.t0;
    for (double d : A.dts) t += d;   // the device's own sum: t_new = t + dt per step
    ctl_reset(h, kModeHost, INFINITY, LLONG_MAX);
    h->hctl->t = t;
    h->hctl->step = A.step0 + A.nsteps;
    if (int rc = ctl_push(h)) return rc;
    A.ready = true;
    return EU_OK;
}

// The backward sweeps on the handle's stream: A.lam holds dJ/dU_N on entry
// and dJ/dU_0 on exit (planes of a state buffer), each earlier segment's
// states recomputed from its checkpoint.
int adj_bwd_sweeps(eu_handle* h) {
    auto& A = h->adj;
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
    if (int rc = adj_bwd_sweeps(h)) return rc;
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

}  // namespace rt
}  // namespace eu

using namespace eu::rt;

extern "C" {

// --- discrete adjoint -----------------------------------------------------------
int eu_adjoint_forward(eu_handle* h, long long nsteps, const double* dts, int ckpt_k) {
    Range range_("eu_adjoint_forward");
    if (int rc = adj_fwd_enqueue(h, nsteps, dts, ckpt_k, INFINITY)) return rc;
    return adj_fwd_finish(h);
}

int eu_adjoint_dts(eu_handle* h, double* dts, long long cap, long long* nsteps) {
    if (!h || !nsteps || (cap > 0 && !dts)) return fail(h, EU_ERR_INVALID, "eu_adjoint_dts: bad argument");
    const auto& A = h->adj;
    if (!A.ready) return fail(h, EU_ERR_STATE, "eu_adjoint_dts: call eu_adjoint_forward first");
    *nsteps = (long long)A.dts.size();
    const long long n = std::min<long long>(cap, *nsteps);
    if (n > 0) std::memcpy(dts, A.dts.data(), sizeof(double) * (size_t)n);
    return EU_OK;
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

}  // extern "C"
