// adjoint_kernels.cu -- the adjoint sweep kernels for one precision and one
// Riemann solver (compiled once per (EU_PREC, EU_SOLVER) pair).
//
// One CTA of 256 threads owns a tile of NL lines x up to TC cells and runs
// the five phases of eu::adj::adjoint_tile in shared memory (20 values of
// the element type per tile cell).  x-adjoint: lines are rows, threads walk
// cells fastest (coalesced along rows).  y-adjoint: lines are columns,
// threads walk lines fastest (coalesced along rows again).  The kernels
// read plain global loads: at the adjoint's working sizes the forward
// states of a checkpoint segment sit in L2.
#include "adjoint.cuh"
#include "adjoint_kernels.h"
#include "per_device.h"

#ifndef EU_PREC
#error "EU_PREC (32 or 64) must be defined"
#endif
#ifndef EU_SOLVER
#error "EU_SOLVER (0..3) must be defined"
#endif

#define EU_NAME2(base, p, s) base##_##p##_##s
#define EU_NAME(base, p, s) EU_NAME2(base, p, s)
#define ADJ_LAUNCH EU_NAME(adjoint_sweep, EU_PREC, EU_SOLVER)

namespace eu {
namespace {

#if EU_PREC == 32
using T = float;
constexpr int NLX = 8, TCX = 64, NLY = 32, TCY = 32;
constexpr int kMinBlocks = 1;   // ~62 registers: up to 4 CTAs per SM already
#else
using T = double;
// Two CTAs per SM (<= 128 registers, a few spills) and smaller tiles:
// measured on GB300 (512^2 HLLC, 400 steps, checkpoints every 32) the
// backward takes 657 ms against 726 ms for one CTA per SM (154 registers)
// with 4x64 / 16x32 tiles, gradients bit-identical.
constexpr int NLX = 4, TCX = 32, NLY = 8, TCY = 64;
constexpr int kMinBlocks = 2;
#endif
constexpr int kThreads = 256;

template <int DIR> struct DevAcc {
    const T* P;
    long long pp, pl;
    int pc;
    const T* A;
    long long ap, al;
    int ac;
    T* G;
    long long gp, gl;
    int gc;
    int n, nlines;
    T hl, lam;
    int bc_lo, bc_hi;

    __host__ __device__ long long off(long long pitch, int coff, int line, int c) const {
        return DIR == 0 ? (long long)(line + 2) * pitch + (c + coff) : (long long)(c + 2) * pitch + (line + coff);
    }
    __host__ __device__ bool line_ok(int l) const { return l < nlines; }
    // sweep-local order: (rho, normal momentum, tangential momentum, E)
    __host__ __device__ adj::C4<T> load_state(int line, int c) const {
        const T* q = P + off(pp, pc, line, c);
        return DIR == 0 ? adj::C4<T>{q[0], q[pl], q[2 * pl], q[3 * pl]}
                        : adj::C4<T>{q[0], q[2 * pl], q[pl], q[3 * pl]};
    }
    __host__ __device__ adj::C4<T> load_adj(int line, int c) const {
        const T* q = A + off(ap, ac, line, c);
        return DIR == 0 ? adj::C4<T>{q[0], q[al], q[2 * al], q[3 * al]}
                        : adj::C4<T>{q[0], q[2 * al], q[al], q[3 * al]};
    }
    __host__ __device__ void store(int line, int c, const adj::C4<T>& u) const {
        T* q = G + off(gp, gc, line, c);
        q[0] = u.r;
        q[DIR == 0 ? gl : 2 * gl] = u.mn;
        q[DIR == 0 ? 2 * gl : gl] = u.mt;
        q[3 * gl] = u.e;
    }
};

template <int DIR, int NL, int TC>
__global__ void __launch_bounds__(kThreads, kMinBlocks) adjoint_sweep_kernel(const DevAcc<DIR> acc) {
    extern __shared__ __align__(16) unsigned char smem[];
    auto& m = *reinterpret_cast<adj::TileMem<T, NL, TC, DIR == 1>*>(smem);
    const int ntile = (acc.n + TC - 1) / TC;
    const int g = blockIdx.x / ntile, t = blockIdx.x - g * ntile;
    int c0, c1;
    adj::tile_range(acc.n, TC, t, c0, c1);
    adj::adjoint_tile<EU_SOLVER, T, NL, TC, DIR == 1>(acc, m, g * NL, c0, c1 - c0, threadIdx.x, kThreads);
}

template <int DIR, int NL, int TC> cudaError_t launch(const AdjSweepArgs& a, cudaStream_t s) {
    DevAcc<DIR> acc;
    acc.P = static_cast<const T*>(a.P);
    acc.pp = a.p_pitch; acc.pl = a.p_plane; acc.pc = a.p_coff;
    acc.A = static_cast<const T*>(a.A);
    acc.ap = a.a_pitch; acc.al = a.a_plane; acc.ac = a.a_coff;
    acc.G = static_cast<T*>(a.G);
    acc.gp = a.g_pitch; acc.gl = a.g_plane; acc.gc = a.g_coff;
    acc.n = DIR == 0 ? a.nx : a.ny;
    acc.nlines = DIR == 0 ? a.ny : a.nx;
    acc.lam = T(a.lam_d);
    acc.hl = T(0.5 * a.lam_d);
    acc.bc_lo = a.bc_lo;
    acc.bc_hi = a.bc_hi;
    constexpr size_t smem = sizeof(adj::TileMem<T, NL, TC, DIR == 1>);
    auto k = adjoint_sweep_kernel<DIR, NL, TC>;
    static PerDevice<cudaError_t> attr_cache;
    const cudaError_t attr = attr_cache.get(
        [k] { return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); });
    if (attr != cudaSuccess) return attr;
    const long long ctas = (long long)((acc.nlines + NL - 1) / NL) * ((acc.n + TC - 1) / TC);
    k<<<(unsigned)ctas, kThreads, smem, s>>>(acc);
    return cudaGetLastError();
}

}  // namespace

cudaError_t ADJ_LAUNCH(int dir, const AdjSweepArgs& a, cudaStream_t s) {
    return dir == 0 ? launch<0, NLX, TCX>(a, s) : launch<1, NLY, TCY>(a, s);
}

}  // namespace eu
