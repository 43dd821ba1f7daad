// api.cpp -- host runtime behind include/euler2d.h.
//
// One handle owns: two SoA state buffers (S0/S1, ping-pong), the x-sweep
// output buffer Utmp, the device control block (Ctl), three TMA descriptors
// (S0 and S1 boxed for the x-sweep, Utmp boxed for the y-sweep), a CUDA
// stream, and lazily built CUDA graphs of whole steps.  The host never
// touches a state value on the hot path: dt, t_end clipping and the snapshot
// schedule live in Ctl and are advanced by the y-sweep's last warp.
//
// This unit holds the single-grid entry points; runtime.h lists the other
// units of the runtime.
#include "runtime.h"

using namespace eu;
using namespace eu::rt;

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
// one pass over the trials tunes both sweeps.  Every trial starts from the
// state, time and step counter of the call, and they are restored
// afterwards.
int eu_autotune(eu_handle* h, int steps, long long chosen[2]) {
    Range range_("eu_autotune");
    if (!h || steps < 1) return fail(h, EU_ERR_INVALID, "eu_autotune: bad argument");
    const int CX = h->K.box_x, RY = kYLag;        // y segments: whole output boxes
    // the current shape first: it is kept unless a candidate beats it by 1%
    std::vector<int> cx{h->seg_x}, cy{h->seg_y};
    for (int v : {CX, 2 * CX, 4 * CX, 32, 64, 128, 256})
        if (v % CX == 0 && v <= round_up(h->cfg.nx, CX) && std::find(cx.begin(), cx.end(), v) == cx.end()) cx.push_back(v);
    // the planner's neighbours keep its remainder modulo the input box height
    for (int v : {RY, 2 * RY, 4 * RY, 32, 64, 128, h->seg_y - 2 * RY, h->seg_y + 2 * RY})
        if (v >= RY && v % RY == 0 && v <= round_up(h->cfg.ny, RY) && std::find(cy.begin(), cy.end(), v) == cy.end())
            cy.push_back(v);
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
        // every trial starts from the same state (a solution whose cost per
        // step changes as it evolves would otherwise favour early trials)
        if (t > 0) {
            e = cudaMemcpyAsync(h->S[cur0], saved, state_bytes(h), cudaMemcpyDeviceToDevice, h->st);
            h->cur = cur0;
            *h->hctl = ctl0;
            if (e == cudaSuccess && ctl_push(h) != EU_OK) e = cudaErrorUnknown;
            if (e != cudaSuccess) break;
        }
        rc = eu_set_option(h, "seg_x", sx);
        if (rc == EU_OK) rc = eu_set_option(h, "seg_y", sy);
        float ms[3], tx = INFINITY, ty = INFINITY;
        if (rc == EU_OK) rc = eu_time_steps(h, 2, 1, ms);
        for (int rep = 0; rep < 2 && rc == EU_OK; ++rep) {   // best of two timings per shape
            rc = eu_time_steps(h, steps, 1, ms);
            tx = std::min(tx, ms[1]);
            ty = std::min(ty, ms[2]);
        }
        if (rc != EU_OK) break;
        if (t == 0) {
            tbx = 0.99f * tx;   // the current shape, with a 1% margin to beat
            tby = 0.99f * ty;
            continue;
        }
        if (t < cx.size() && tx < tbx) { tbx = tx; best_x = sx; }
        if (t < cy.size() && ty < tby) { tby = ty; best_y = sy; }
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
        if (value < kYLag || value % kYLag) return fail(h, EU_ERR_INVALID, "seg_y must be a multiple of 4 rows");
        h->seg_y = (int)value;
        h->ntasks_y = h->nseg_y * ((h->cfg.ny + h->seg_y - 1) / h->seg_y);
        h->ctas_y = (h->ntasks_y + h->K.nw - 1) / h->K.nw;
    } else if (k == "graph_steps") {
        if (value < 1 || value > 4096) return fail(h, EU_ERR_INVALID, "graph_steps must be in [1, 4096]");
        h->gsteps = (int)value;
    } else if (k == "solver") {
        // the Riemann solver of later steps (the reference passes it per
        // call, src/cpu/solver_cpu.cpp:400-405); the state is kept and the
        // launch plan is the planner's for the new solver
        if (value < EU_HLL || value > EU_FORCE) return fail(h, EU_ERR_INVALID, "solver must be 0..3");
        if (value != h->solver) {
            if (cudaStreamSynchronize(h->st) != cudaSuccess) {
                (void)cudaGetLastError();
                return fail(h, EU_ERR_CUDA, "eu_set_option(solver): stream synchronisation failed");
            }
            h->solver = (int)value;
            h->K = kernels_for(h->prec, h->solver);
            h->adj.ready = false;   // a completed adjoint forward belongs to the old solver
            // the solvers' y-sweeps load boxes of different heights (8 or 4
            // rows): re-encode the maps that carry the box
            if (h->K.ry != h->tm_y_ry)
                if (int rc = encode_all(h)) return rc;
            plan(h);
        }
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
    else if (k == "solver") *value = h->solver;
    else if (k == "tasks_x") *value = h->ntasks_x;
    else if (k == "occ_x") *value = h->K.occ_x();
    else if (k == "occ_y") *value = h->K.occ_y();
    else if (k == "sm_count") *value = h->sm_count;
    else if (k == "tasks_y") *value = h->ntasks_y;
    else if (k == "ckpt_k") *value = h->adj.k;
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

}  // extern "C"
