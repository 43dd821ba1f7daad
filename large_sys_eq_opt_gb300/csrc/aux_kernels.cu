// aux_kernels.cu -- everything around the two sweeps: AoS <-> SoA transfer
// with the boundary rule applied to ghosts, device-side initial states,
// the standalone CFL reduction (first step / compute_dt), FP64 audits of the
// conserved totals, snapshot unpacking.
#include "aux_kernels.h"
#include "per_device.h"
#include "sweeps.cuh"

namespace eu {

// Source cell of ghost index g (array index in [0, n+4)) under a boundary
// pair: transmissive copies the nearest interior cell, reflective mirrors
// (head/cpu/boundary_cpu.hpp:5-37, generalised).  Returns the interior index
// and whether the normal momentum flips sign.
__device__ __forceinline__ int ghost_src(int g, int n, int bc_lo, int bc_hi, bool& flip) {
    const int i = g - 2;
    flip = false;
    if (i < 0) {
        if (bc_lo == kBcReflective) { flip = true; return -1 - i; }
        return 0;
    }
    if (i >= n) {
        if (bc_hi == kBcReflective) { flip = true; return 2 * n - 1 - i; }
        return n - 1;
    }
    return i;
}

// AoS double grid with ghosts -> S planes (every cell, ghosts included).
template <class T>
__global__ void pack_aos_kernel(const double* __restrict__ aos, Planes<T> P, int nx, int ny) {
    const long long tnx = nx + 4, total = tnx * (ny + 4);
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long r = idx / tnx, c = idx - r * tnx;
        const double2 u01 = reinterpret_cast<const double2*>(aos)[2 * idx];
        const double2 u23 = reinterpret_cast<const double2*>(aos)[2 * idx + 1];
        T* q = P.base + r * P.pitch + (c + kSOff - 2);
        q[0] = T(u01.x); q[P.plane] = T(u01.y); q[2 * P.plane] = T(u23.x); q[3 * P.plane] = T(u23.y);
    }
}

// Planes (interior at column offset coff, row offset 2) -> AoS double grid
// with ghosts filled by the boundary rule: x first, then y over all columns
// (corners take the y rule of the x ghosts), as the reference's BC pass.
template <class T>
__global__ void unpack_aos_kernel(Planes<T> P, int coff, int nx, int ny, int4 bc, double* __restrict__ aos) {
    const long long tnx = nx + 4, total = tnx * (ny + 4);
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(idx / tnx), c = (int)(idx - (long long)r * tnx);
        bool fx, fy;
        const int si = ghost_src(c, nx, bc.x, bc.y, fx);
        const int sj = ghost_src(r, ny, bc.z, bc.w, fy);
        const T* q = P.base + (long long)(sj + 2) * P.pitch + (si + coff);
        double2 u01 = make_double2((double)q[0], (double)q[P.plane]);
        double2 u23 = make_double2((double)q[2 * P.plane], (double)q[3 * P.plane]);
        if (fx) u01.y = -u01.y;
        if (fy) u23.x = -u23.x;
        reinterpret_cast<double2*>(aos)[2 * idx] = u01;
        reinterpret_cast<double2*>(aos)[2 * idx + 1] = u23;
    }
}

// Ghost frame of an S buffer from its interior (apply_transmissive_boundary,
// head/cpu/boundary_cpu.hpp:5-37, with the per-side rule).  Ghosts read only
// interior cells, so every ghost is written independently.
template <class T>
__global__ void fill_ghosts_kernel(Planes<T> P, int nx, int ny, int4 bc) {
    const long long tnx = nx + 4, total = tnx * (ny + 4);
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(idx / tnx), c = (int)(idx - (long long)r * tnx);
        if (r >= 2 && r < ny + 2 && c >= 2 && c < nx + 2) continue;
        bool fx, fy;
        const int si = ghost_src(c, nx, bc.x, bc.y, fx);
        const int sj = ghost_src(r, ny, bc.z, bc.w, fy);
        const T* q = P.base + (long long)(sj + 2) * P.pitch + (si + kSOff);
        T* o = P.base + (long long)r * P.pitch + (c + kSOff - 2);
        o[0] = q[0];
        o[P.plane] = fx ? -q[P.plane] : q[P.plane];
        o[2 * P.plane] = fy ? -q[2 * P.plane] : q[2 * P.plane];
        o[3 * P.plane] = q[3 * P.plane];
    }
}

// Interior SoA snapshot [f][ny][nx] -> AoS double grid with ghosts.
template <class T>
__global__ void unpack_snapshot_kernel(const T* __restrict__ s, long long plane, int nx, int ny, int4 bc,
                                       double* __restrict__ aos) {
    const long long tnx = nx + 4, total = tnx * (ny + 4);
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(idx / tnx), c = (int)(idx - (long long)r * tnx);
        bool fx, fy;
        const int si = ghost_src(c, nx, bc.x, bc.y, fx);
        const int sj = ghost_src(r, ny, bc.z, bc.w, fy);
        const T* q = s + (long long)sj * nx + si;
        double2 u01 = make_double2((double)q[0], (double)q[plane]);
        double2 u23 = make_double2((double)q[2 * plane], (double)q[3 * plane]);
        if (fx) u01.y = -u01.y;
        if (fy) u23.x = -u23.x;
        reinterpret_cast<double2*>(aos)[2 * idx] = u01;
        reinterpret_cast<double2*>(aos)[2 * idx + 1] = u23;
    }
}

// src/test_cases.cpp:11-18 make_conserved, without FMA contraction so the
// FP64 initial state matches the CPU oracle bit for bit.
struct Cell4 { double r, mu, mv, e; };
__device__ __forceinline__ Cell4 make_conserved_rn(double rho, double u, double v, double p) {
    const double kin = __dmul_rn(__dmul_rn(0.5, rho), __dadd_rn(__dmul_rn(u, u), __dmul_rn(v, v)));
    return Cell4{rho, __dmul_rn(rho, u), __dmul_rn(rho, v), __dadd_rn(p / kGm1D, kin)};
}

__device__ __forceinline__ double cell_centre(double lo, int idx, double d) {
    return __dadd_rn(lo, __dmul_rn(__dadd_rn((double)(idx - 2), 0.5), d));
}

template <class T>
__device__ __forceinline__ void put(Planes<T> P, int r, int c, Cell4 u) {
    T* q = P.base + (long long)r * P.pitch + (c + kSOff - 2);
    q[0] = T(u.r); q[P.plane] = T(u.mu); q[2 * P.plane] = T(u.mv); q[3 * P.plane] = T(u.e);
}

// src/test_cases.cpp:78-101 (parameterised), every cell incl. ghosts (src/init.cpp:29-38)
template <class T>
__global__ void init_blast_kernel(Planes<T> P, GridGeom g, BlastDesc b) {
    const long long tnx = g.nx + 4, total = tnx * (g.ny + 4);
    const double dx = (g.x_max - g.x_min) / (double)g.nx, dy = (g.y_max - g.y_min) / (double)g.ny;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(idx / tnx), c = (int)(idx - (long long)r * tnx);
        const double x = cell_centre(g.x_min, c, dx), y = cell_centre(g.y_min, r, dy);
        const double ddx = __dadd_rn(x, -b.cx), ddy = __dadd_rn(y, -b.cy);
        const double r2 = __dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy));
        const bool in = r2 <= __dmul_rn(b.r, b.r);
        put(P, r, c, in ? make_conserved_rn(b.rho_in, 0.0, 0.0, b.p_in)
                        : make_conserved_rn(b.rho_out, 0.0, 0.0, b.p_out));
    }
}

// src/test_cases.cpp:24-69 (parameterised)
template <class T>
__global__ void init_shock_bubble_kernel(Planes<T> P, GridGeom g, ShockBubbleDesc s) {
    const long long tnx = g.nx + 4, total = tnx * (g.ny + 4);
    const double dx = (g.x_max - g.x_min) / (double)g.nx, dy = (g.y_max - g.y_min) / (double)g.ny;
    const double gm = kGammaD;
    const double a0 = sqrt(__dmul_rn(gm, s.p0) / s.rho0);
    const double M2 = __dmul_rn(s.mach, s.mach);
    const double rho2 = __dmul_rn(s.rho0, __dmul_rn(gm + 1.0, M2)) / __dadd_rn(__dmul_rn(gm - 1.0, M2), 2.0);
    const double p2 = __dmul_rn(s.p0, __dadd_rn(1.0, __dmul_rn(2.0 * gm / (gm + 1.0), __dadd_rn(M2, -1.0))));
    const double u2 = __dmul_rn(__dmul_rn(2.0, a0) / (gm + 1.0), __dadd_rn(s.mach, -(1.0 / s.mach)));
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(idx / tnx), c = (int)(idx - (long long)r * tnx);
        const double x = cell_centre(g.x_min, c, dx), y = cell_centre(g.y_min, r, dy);
        double rho = s.rho0, u = 0.0, p = s.p0;
        if (x < s.shock_x) { rho = rho2; u = u2; p = p2; }
        const double ddx = __dadd_rn(x, -s.bub_cx), ddy = __dadd_rn(y, -s.bub_cy);
        if (__dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)) <= __dmul_rn(s.bub_r, s.bub_r)) rho = s.rho_bubble;
        put(P, r, c, make_conserved_rn(rho, u, 0.0, p));
    }
}

// Standalone CFL reduction over the interior of an S buffer
// (src/cpu/solver_cpu.cpp:287-309); the last warp computes dt on device.
template <class T>
__global__ void dt_kernel(Planes<T> P, int nx, int ny, Ctl* ctl, unsigned int nwarps) {
    const int lane = threadIdx.x & 31;
    const long long total = (long long)nx * ny;
    T smax = T(0);
    bool bad = false;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long j = idx / nx, i = idx - j * nx;
        const T* q = P.base + (j + 2) * P.pitch + (i + kSOff);
        const Cons<T> U{q[0], q[P.plane], q[2 * P.plane], q[3 * P.plane]};
        const T sp = max_signal_speed(U);
        bad |= !(sp < T(INFINITY));
        smax = Ar<T>::fmax_(smax, sp);
    }
    warp_arrive<T>(ctl, smax, bad, false, lane, nwarps, 0, 0);
}

// FP64 audit of the conserved totals: per-block Neumaier sums of the
// interior, in a fixed order, then one block folds the partials.
template <class T>
__global__ void totals_partial_kernel(Planes<T> P, int coff, int nx, int ny, double* part) {
    __shared__ double sh[4][256];
    __shared__ double shc[4][256];
    double s[4] = {0, 0, 0, 0}, comp[4] = {0, 0, 0, 0};
    const long long total = (long long)nx * ny;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long j = idx / nx, i = idx - j * nx;
        const T* q = P.base + (j + 2) * P.pitch + (i + coff);
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            const double x = (double)q[f * P.plane];
            const double t = s[f] + x;
            comp[f] += (fabs(s[f]) >= fabs(x)) ? ((s[f] - t) + x) : ((x - t) + s[f]);
            s[f] = t;
        }
    }
#pragma unroll
    for (int f = 0; f < 4; ++f) { sh[f][threadIdx.x] = s[f]; shc[f][threadIdx.x] = comp[f]; }
    __syncthreads();
    if (threadIdx.x < 4) {
        const int f = threadIdx.x;
        double a = 0.0, c = 0.0;
        for (int k = 0; k < (int)blockDim.x; ++k) {
            const double x = sh[f][k];
            const double t = a + x;
            c += (fabs(a) >= fabs(x)) ? ((a - t) + x) : ((x - t) + a);
            a = t;
            c += shc[f][k];
        }
        part[blockIdx.x * 8 + f] = a;
        part[blockIdx.x * 8 + 4 + f] = c;
    }
}

__global__ void totals_final_kernel(const double* part, int nblocks, double* out) {
    if (threadIdx.x < 4) {
        const int f = threadIdx.x;
        double a = 0.0, c = 0.0;
        for (int b = 0; b < nblocks; ++b) {
            const double x = part[b * 8 + f];
            const double t = a + x;
            c += (fabs(a) >= fabs(x)) ? ((a - t) + x) : ((x - t) + a);
            a = t;
            c += part[b * 8 + 4 + f];
        }
        out[f] = a + c;
    }
}

// One thread: the smallest proposed dt of n slabs to every slab (see
// launch_domain_dt), with their status and stop flags merged.
__global__ void domain_dt_kernel(Ctl* const* ctls, int n) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double dt = ctls[0]->dt, smax = ctls[0]->smax;
    int status = 0, done = 0;
    for (int s = 0; s < n; ++s) {
        const Ctl* c = ctls[s];
        if (c->dt < dt) dt = c->dt;
        if (c->smax > smax) smax = c->smax;
        status |= c->status;
        done |= c->done;
    }
    for (int s = 0; s < n; ++s) {
        Ctl* c = ctls[s];
        c->dt = dt;
        c->smax = smax;
        c->status = status;
        c->done = done;
    }
    __threadfence();
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
cudaError_t launch_domain_dt(Ctl* const* ctls, int n, cudaStream_t s) {
    domain_dt_kernel<<<1, 32, 0, s>>>(ctls, n);
    return cudaGetLastError();
}

static int grid_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    const long long cap = 16LL * sm_count_current();   // grid-stride loops: 16 CTAs per SM at most
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

template <class T>
cudaError_t launch_pack_aos(const double* aos, Planes<T> P, int nx, int ny, cudaStream_t s) {
    const long long n = (long long)(nx + 4) * (ny + 4);
    pack_aos_kernel<T><<<grid_for(n, 256), 256, 0, s>>>(aos, P, nx, ny);
    return cudaGetLastError();
}
template <class T>
cudaError_t launch_unpack_aos(Planes<T> P, int coff, int nx, int ny, const int bc[4], double* aos,
                              cudaStream_t s) {
    const long long n = (long long)(nx + 4) * (ny + 4);
    unpack_aos_kernel<T><<<grid_for(n, 256), 256, 0, s>>>(P, coff, nx, ny, make_int4(bc[0], bc[1], bc[2], bc[3]), aos);
    return cudaGetLastError();
}
template <class T>
cudaError_t launch_fill_ghosts(Planes<T> P, int nx, int ny, const int bc[4], cudaStream_t s) {
    const long long n = (long long)(nx + 4) * (ny + 4);
    fill_ghosts_kernel<T><<<grid_for(n, 256), 256, 0, s>>>(P, nx, ny, make_int4(bc[0], bc[1], bc[2], bc[3]));
    return cudaGetLastError();
}
template <class T>
cudaError_t launch_unpack_snapshot(const T* snap, long long plane, int nx, int ny, const int bc[4],
                                   double* aos, cudaStream_t s) {
    const long long n = (long long)(nx + 4) * (ny + 4);
    unpack_snapshot_kernel<T><<<grid_for(n, 256), 256, 0, s>>>(snap, plane, nx, ny,
                                                               make_int4(bc[0], bc[1], bc[2], bc[3]), aos);
    return cudaGetLastError();
}
template <class T>
cudaError_t launch_init_blast(Planes<T> P, GridGeom g, BlastDesc b, cudaStream_t s) {
    const long long n = (long long)(g.nx + 4) * (g.ny + 4);
    init_blast_kernel<T><<<grid_for(n, 256), 256, 0, s>>>(P, g, b);
    return cudaGetLastError();
}
template <class T>
cudaError_t launch_init_shock_bubble(Planes<T> P, GridGeom g, ShockBubbleDesc d, cudaStream_t s) {
    const long long n = (long long)(g.nx + 4) * (g.ny + 4);
    init_shock_bubble_kernel<T><<<grid_for(n, 256), 256, 0, s>>>(P, g, d);
    return cudaGetLastError();
}
template <class T>
cudaError_t launch_dt(Planes<T> P, int nx, int ny, Ctl* ctl, cudaStream_t s) {
    const int threads = 256;
    const int blocks = grid_for((long long)nx * ny, threads);
    dt_kernel<T><<<blocks, threads, 0, s>>>(P, nx, ny, ctl, (unsigned)(blocks * (threads / 32)));
    return cudaGetLastError();
}
template <class T>
cudaError_t launch_totals(Planes<T> P, int coff, int nx, int ny, double* part, int max_blocks, double* out,
                          cudaStream_t s) {
    int blocks = grid_for((long long)nx * ny, 256);
    if (blocks > max_blocks) blocks = max_blocks;
    totals_partial_kernel<T><<<blocks, 256, 0, s>>>(P, coff, nx, ny, part);
    totals_final_kernel<<<1, 32, 0, s>>>(part, blocks, out);
    return cudaGetLastError();
}

#define EU_INST(T)                                                                                   \
    template cudaError_t launch_pack_aos<T>(const double*, Planes<T>, int, int, cudaStream_t);     \
    template cudaError_t launch_unpack_aos<T>(Planes<T>, int, int, int, const int*, double*,       \
                                              cudaStream_t);                                         \
    template cudaError_t launch_fill_ghosts<T>(Planes<T>, int, int, const int*, cudaStream_t);     \
    template cudaError_t launch_unpack_snapshot<T>(const T*, long long, int, int, const int*,      \
                                                   double*, cudaStream_t);                           \
    template cudaError_t launch_init_blast<T>(Planes<T>, GridGeom, BlastDesc, cudaStream_t);        \
    template cudaError_t launch_init_shock_bubble<T>(Planes<T>, GridGeom, ShockBubbleDesc,          \
                                                     cudaStream_t);                                  \
    template cudaError_t launch_dt<T>(Planes<T>, int, int, Ctl*, cudaStream_t);                     \
    template cudaError_t launch_totals<T>(Planes<T>, int, int, int, double*, int, double*, cudaStream_t);
EU_INST(float)
EU_INST(double)

}  // namespace eu
