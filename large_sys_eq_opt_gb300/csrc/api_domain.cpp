// api_domain.cpp -- one grid split into slabs of whole rows (eu_domain_*):
// the semantics of the reference's domain decomposition
// (src/cpu/solver_mpi.cpp:246-291 partition, :340-402 / :547-573 halo
// exchange, :416-443 dt reduction) for slabs on one device.
//
// Each slab is a handle on its own rows with a 2-row frame.  A step runs
// every slab's x-sweep; then the two boundary rows of each x-sweep output
// are copied into the neighbour's frame rows (the rows the y-sweep's
// stencil reads past the slab edge); then every slab's y-sweep, whose
// finalisation proposes the slab's next dt; then one kernel gives every slab
// the smallest proposal.  A cell's update depends only on its stencil and
// dt, and every kernel's output is independent of where a line segment
// starts, so the slabs reproduce the undivided grid bit for bit.  The slabs
// share one stream; on several GPUs the row copies would become peer or
// NCCL transfers into each GPU's own memory.
#include "runtime.h"

using namespace eu;
using namespace eu::rt;

struct eu_domain {
    int n = 0;
    eu_case cfg{};
    int prec = EU_FP64;
    std::vector<int> row0;
    std::vector<eu_handle*> h;
    cudaStream_t st = nullptr;
    Ctl** d_ctls = nullptr;   // device array of the slabs' control blocks
    std::string err;
};

namespace {

int dfail(eu_domain* d, int code, const std::string& msg) {
    if (d) d->err = msg;
    else set_global_error(msg.c_str());
    return code;
}

// The plan of src/cpu/solver_mpi.cpp:246-291 along y: balanced whole rows.
void plan_rows(int ny, int n, int* row0) {
    for (int s = 0; s <= n; ++s) row0[s] = (int)((long long)s * ny / n);
}

// Frame rows of each internal boundary: the last two interior rows of the
// lower slab's x-sweep output go to the upper slab's rows 0, 1; the first
// two of the upper slab's go to the lower slab's rows ny+2, ny+3 (storage
// rows of the x-sweep output, all columns, all four planes).
cudaError_t exchange_rows(eu_domain* d) {
    for (int s = 0; s + 1 < d->n; ++s) {
        eu_handle* lo = d->h[(size_t)s];
        eu_handle* up = d->h[(size_t)s + 1];
        const size_t row = (size_t)lo->pitch_t * lo->esz;
        const int nlo = lo->cfg.ny;
        for (int f = 0; f < 4; ++f) {
            char* blo = static_cast<char*>(lo->Tm) + (size_t)f * lo->plane_t * lo->esz;
            char* bup = static_cast<char*>(up->Tm) + (size_t)f * up->plane_t * up->esz;
            cudaError_t e = cudaMemcpyAsync(bup, blo + (size_t)nlo * row, 2 * row, cudaMemcpyDeviceToDevice, d->st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(blo + (size_t)(nlo + 2) * row, bup + 2 * row, 2 * row, cudaMemcpyDeviceToDevice,
                                    d->st);
            if (e != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

}  // namespace

extern "C" {

int eu_domain_plan(int ny, int nslabs, int* row0) {
    if (!row0 || nslabs < 1 || ny < 2 * nslabs) return fail(nullptr, EU_ERR_INVALID, "eu_domain_plan: need ny >= 2*nslabs");
    plan_rows(ny, nslabs, row0);
    return EU_OK;
}

int eu_domain_create(const eu_case* cfg, eu_precision prec, eu_solver solver, eu_limiter limiter, const int* bc,
                     int nslabs, eu_domain** out) {
    if (!cfg || !out) return dfail(nullptr, EU_ERR_INVALID, "eu_domain_create: null argument");
    *out = nullptr;
    if (nslabs < 1 || nslabs > 64 || cfg->ny < 2 * nslabs)
        return dfail(nullptr, EU_ERR_INVALID, "eu_domain_create: need 1 <= nslabs <= 64 and ny >= 2*nslabs");
    eu_domain* d = new eu_domain();
    d->n = nslabs;
    d->cfg = *cfg;
    d->prec = prec;
    d->row0.resize((size_t)nslabs + 1);
    plan_rows(cfg->ny, nslabs, d->row0.data());
    auto bail = [&](int rc) {
        eu_domain_destroy(d);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&d->st, cudaStreamNonBlocking) != cudaSuccess) {
        (void)cudaGetLastError();
        return bail(dfail(nullptr, EU_ERR_CUDA, "eu_domain_create: stream creation failed"));
    }
    const double dy = (cfg->y_max - cfg->y_min) / (double)cfg->ny;   // the whole grid's (head/cpu/grid_cpu.hpp:19-20)
    for (int s = 0; s < nslabs; ++s) {
        eu_case c = *cfg;
        c.ny = d->row0[(size_t)s + 1] - d->row0[(size_t)s];
        c.y_min = cfg->y_min + dy * d->row0[(size_t)s];
        c.y_max = cfg->y_min + dy * d->row0[(size_t)s + 1];
        int b[4] = {bc ? bc[0] : 0, bc ? bc[1] : 0, bc ? bc[2] : 0, bc ? bc[3] : 0};
        if (s > 0) b[EU_SIDE_BOTTOM] = EU_BC_TRANSMISSIVE;             // halo side: overwritten each step
        if (s + 1 < nslabs) b[EU_SIDE_TOP] = EU_BC_TRANSMISSIVE;
        eu_handle* h = nullptr;
        if (int rc = eu_create(&c, prec, solver, limiter, b, &h)) return bail(dfail(nullptr, rc, g_err));
        d->h.push_back(h);
        h->dy = dy;                       // bit for bit the whole grid's spacing
        cudaStreamSynchronize(h->st);
        cudaStreamDestroy(h->st);         // every slab runs on the domain's stream
        h->st = d->st;
    }
    std::vector<Ctl*> ctls;
    for (eu_handle* h : d->h) ctls.push_back(h->ctl);
    if (cudaMalloc(&d->d_ctls, sizeof(Ctl*) * ctls.size()) != cudaSuccess ||
        cudaMemcpy(d->d_ctls, ctls.data(), sizeof(Ctl*) * ctls.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        (void)cudaGetLastError();
        return bail(dfail(nullptr, EU_ERR_NOMEM, "eu_domain_create: control-block table"));
    }
    *out = d;
    return EU_OK;
}

void eu_domain_destroy(eu_domain* d) {
    if (!d) return;
    if (d->st) cudaStreamSynchronize(d->st);
    for (eu_handle* h : d->h) {
        h->st = nullptr;                  // the shared stream is the domain's
        eu_destroy(h);
    }
    cudaFree(d->d_ctls);
    if (d->st) cudaStreamDestroy(d->st);
    delete d;
}

const char* eu_domain_last_error(const eu_domain* d) { return d ? d->err.c_str() : g_err.c_str(); }

int eu_domain_upload_aos(eu_domain* d, const double* aos) {
    if (!d || !aos) return dfail(d, EU_ERR_INVALID, "eu_domain_upload_aos: null argument");
    const size_t row = 4 * (size_t)(d->cfg.nx + 4);
    for (int s = 0; s < d->n; ++s)   // slab s's rows with their frame are one block of the grid
        if (int rc = eu_upload_aos(d->h[(size_t)s], aos + (size_t)d->row0[(size_t)s] * row))
            return dfail(d, rc, d->h[(size_t)s]->err);
    return EU_OK;
}

int eu_domain_download_aos(eu_domain* d, double* aos) {
    if (!d || !aos) return dfail(d, EU_ERR_INVALID, "eu_domain_download_aos: null argument");
    const size_t row = 4 * (size_t)(d->cfg.nx + 4);
    std::vector<double> tmp;
    for (int s = 0; s < d->n; ++s) {
        eu_handle* h = d->h[(size_t)s];
        tmp.resize(row * (size_t)(h->cfg.ny + 4));
        if (int rc = eu_download_aos(h, tmp.data())) return dfail(d, rc, h->err);
        // interior rows; the outer frame rows from the first and last slab
        const int r_lo = s == 0 ? 0 : 2, r_hi = s + 1 == d->n ? h->cfg.ny + 4 : h->cfg.ny + 2;
        std::memcpy(aos + ((size_t)d->row0[(size_t)s] + r_lo) * row, tmp.data() + (size_t)r_lo * row,
                    sizeof(double) * row * (size_t)(r_hi - r_lo));
    }
    return EU_OK;
}

int eu_domain_step_n(eu_domain* d, long long n, double t_end) {
    Range range_("eu_domain_step_n");
    if (!d || n < 0 || !(t_end > 0.0)) return dfail(d, EU_ERR_INVALID, "eu_domain_step_n: bad argument");
    if (n == 0) return EU_OK;
    for (eu_handle* h : d->h) {
        Ctl& c = *h->hctl;
        const double t0 = c.t;
        const long long s0 = c.step;
        ctl_reset(h, kModeCfl, t_end, s0 + n);
        c.t = t0;
        c.step = s0;
        if (int rc = ctl_push(h)) return dfail(d, rc, h->err);
        if (fill_ghosts(h, h->cur) != cudaSuccess || launch_dt(h, h->cur) != cudaSuccess)
            return dfail(d, EU_ERR_CUDA, "eu_domain_step_n: set-up launch failed");
    }
    if (launch_domain_dt(d->d_ctls, d->n, d->st) != cudaSuccess)
        return dfail(d, EU_ERR_CUDA, "eu_domain_step_n: dt launch failed");
    int cur = d->h[0]->cur;
    constexpr long long kChunk = 64;   // steps enqueued between checks of the stop flag
    for (long long k = 0; k < n; ++k) {
        cudaError_t e = cudaSuccess;
        for (eu_handle* h : d->h)
            if (e == cudaSuccess) e = launch_x(h, cur);
        if (e == cudaSuccess) e = exchange_rows(d);
        for (eu_handle* h : d->h)
            if (e == cudaSuccess) e = launch_y(h, cur);
        if (e == cudaSuccess) e = launch_domain_dt(d->d_ctls, d->n, d->st);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            return dfail(d, EU_ERR_CUDA, std::string("eu_domain_step_n: ") + cudaGetErrorString(e));
        }
        cur ^= 1;
        if ((k + 1) % kChunk == 0 && k + 1 < n) {   // stop early once t_end is reached (launches after it are no-ops)
            if (int rc = ctl_pull_sync(d->h[0])) return dfail(d, rc, d->h[0]->err);
            if (d->h[0]->hctl->done) break;
        }
    }
    for (eu_handle* h : d->h) {
        if (int rc = ctl_pull_sync(h)) return dfail(d, rc, h->err);
        if (int rc = status_code(h)) return dfail(d, rc, h->err);
    }
    return EU_OK;
}

int eu_domain_get_time(eu_domain* d, double* t, long long* steps) {
    if (!d) return dfail(nullptr, EU_ERR_INVALID, "eu_domain_get_time: null domain");
    const Ctl& c = *d->h[0]->hctl;
    if (t) *t = c.t;
    if (steps) *steps = c.step;
    return EU_OK;
}

}  // extern "C"
