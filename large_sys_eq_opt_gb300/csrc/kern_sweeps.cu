// kern_sweeps.cu -- instantiates the two sweep kernels for one precision and
// one Riemann solver.  Compiled once per (EU_PREC, EU_SOLVER) pair so the
// eight variants build in parallel; the Riemann solver is a template
// parameter, never a per-face runtime switch.
#include "aux_kernels.h"
#include "per_device.h"
#include "sweeps.cuh"

#ifndef EU_PREC
#error "EU_PREC (32 or 64) must be defined"
#endif
#ifndef EU_SOLVER
#error "EU_SOLVER (0..3) must be defined"
#endif

#define EU_NAME2(base, p, s) base##_##p##_##s
#define EU_NAME(base, p, s) EU_NAME2(base, p, s)
#define LAUNCH_X EU_NAME(launch_x, EU_PREC, EU_SOLVER)
#define LAUNCH_Y EU_NAME(launch_y, EU_PREC, EU_SOLVER)
#define OCC_X EU_NAME(occ_x, EU_PREC, EU_SOLVER)
#define LAUNCH_F EU_NAME(launch_first, EU_PREC, EU_SOLVER)
#define OCC_Y EU_NAME(occ_y, EU_PREC, EU_SOLVER)
#define LAUNCH_E EU_NAME(launch_ens, EU_PREC, EU_SOLVER)
#define OCC_E EU_NAME(occ_e, EU_PREC, EU_SOLVER)

namespace eu {
namespace {

#if EU_PREC == 32
using T = float;
#ifndef EU_MINB_X
#define EU_MINB_X 3
#endif
constexpr int MINB_X = EU_MINB_X, MINB_Y = 4;   // x: 3 CTAs of 4 warps per SM (<= 168 registers, measured 13% faster than 4); y: 16 warps (<= 128 registers)
#else
using T = double;
constexpr int MINB_X = 2, MINB_Y = 2;
#endif
// x: boxes of 32 rows x 32 bytes x 4 fields (4 KB), 3 stages per warp.
// y: boxes of 36 columns x RY rows x 4 fields; FP32 8 rows in 2 stages per
// warp (the per-box work halved, 4 CTAs per SM still fit), FP64 and the FP32
// exact solver 4 rows in 3 (the exact solver's y-sweep spilled with 8-row
// boxes: 27.0 -> 35.9 ms per step on the developed 8192^2 blast).
constexpr int CX = 32 / sizeof(T);
constexpr int SX = 3;
#ifndef EU_Y_ROWS
#define EU_Y_ROWS (EU_PREC == 32 && EU_SOLVER != 2 ? 8 : 4)
#endif
constexpr int RY = EU_Y_ROWS, SY = RY == 8 ? 2 : 3;
constexpr int BWY = 36;                 // y-sweep box width: the warp's 32 columns + 2, rounded to 16 B
constexpr int NW = 4;
constexpr int SOL = EU_SOLVER;
constexpr size_t kStageX = 4 * 32 * CX * sizeof(T);
constexpr size_t kStageY = (4 * RY * BWY * sizeof(T) + 127) / 128 * 128;
constexpr size_t kSmemX = 1024 + NW * SX * kStageX + NW * SX * sizeof(uint64_t);
constexpr size_t kOStageY = 4 * kYLag * 32 * sizeof(T);
constexpr size_t kSmemY = 1024 + NW * (SY * kStageY + 2 * kOStageY) + NW * SY * sizeof(uint64_t);

static cudaError_t LAUNCH_X(const CUtensorMap* tm, const CUtensorMap* tm_out, const void* args, int ctas,
                            cudaStream_t s) {
    auto k = sweep_x_kernel<T, SOL, SX, NW, MINB_X>;
    static PerDevice<cudaError_t> attr_cache;
    const cudaError_t attr = attr_cache.get(
        [k] { return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemX); });
    if (attr != cudaSuccess) return attr;
    k<<<ctas, NW * 32, kSmemX, s>>>(*tm, *tm_out, *static_cast<const SweepArgs<T>*>(args));
    return cudaGetLastError();
}

static cudaError_t LAUNCH_Y(const CUtensorMap* tm, const CUtensorMap* tm_out, const void* args, int ctas,
                            cudaStream_t s) {
    auto k = sweep_y_kernel<T, SOL, RY, BWY, SY, NW, MINB_Y>;
    static PerDevice<cudaError_t> attr_cache;
    const cudaError_t attr = attr_cache.get(
        [k] { return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemY); });
    if (attr != cudaSuccess) return attr;
    // persistent: at most one CTA per resident slot (the warps share the work list)
    static PerDevice<int> slot_cache;
    const int slots = slot_cache.get([k]() {
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, NW * 32, kSmemY) != cudaSuccess || occ < 1) {
            (void)cudaGetLastError();
            occ = 1;
        }
        return sm_count_current() * occ;
    });
    k<<<ctas < slots ? ctas : slots, NW * 32, kSmemY, s>>>(*tm, *tm_out, *static_cast<const SweepArgs<T>*>(args));
    return cudaGetLastError();
}

static cudaError_t LAUNCH_F(const void* in, const void* out, int nx, int ny, double dtdx, double dtdy,
                            cudaStream_t s) {
    long long blocks = ((long long)nx * ny + 255) / 256;
    const long long cap = 32LL * sm_count_current();   // grid-stride loop: 32 CTAs per SM at most
    if (blocks > cap) blocks = cap;
    first_order_kernel<T, SOL><<<(int)blocks, 256, 0, s>>>(*static_cast<const Planes<T>*>(in),
                                                           *static_cast<const Planes<T>*>(out), nx, ny, dtdx, dtdy);
    return cudaGetLastError();
}

constexpr size_t kSmemE = ensemble_smem<T, SX, RY, BWY, SY, NW>();
// The persistent ensemble kernel holds both sweeps' code: FP32 at 3 CTAs per
// SM (<= 168 registers; at 128 it spilled 188 bytes, 64-instance ensemble
// 27.5 -> 26.4 ms per 50 steps), FP64 as its y-sweep.
#ifndef EU_MINB_E
#define EU_MINB_E (EU_PREC == 32 ? 3 : 2)
#endif
constexpr int MINB_E = EU_MINB_E;

static cudaError_t LAUNCH_E(const void* args, int ctas, cudaStream_t s) {
    auto k = ensemble_kernel<T, SOL, SX, RY, BWY, SY, NW, MINB_E>;
    static PerDevice<cudaError_t> attr_cache;
    const cudaError_t attr = attr_cache.get(
        [k] { return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemE); });
    if (attr != cudaSuccess) return attr;
    k<<<ctas, NW * 32, kSmemE, s>>>(*static_cast<const EnsArgs<T>*>(args));
    return cudaGetLastError();
}

static int OCC_E() {
    auto k = ensemble_kernel<T, SOL, SX, RY, BWY, SY, NW, MINB_E>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemE);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, NW * 32, kSmemE) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

static int OCC_X() {
    auto k = sweep_x_kernel<T, SOL, SX, NW, MINB_X>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemX);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, NW * 32, kSmemX) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

static int OCC_Y() {
    auto k = sweep_y_kernel<T, SOL, RY, BWY, SY, NW, MINB_Y>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemY);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, NW * 32, kSmemY) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

}  // namespace

SweepKernels EU_NAME(sweep_kernels, EU_PREC, EU_SOLVER)() {
    SweepKernels k;
    k.x = LAUNCH_X;
    k.y = LAUNCH_Y;
    k.occ_x = OCC_X;
    k.first = LAUNCH_F;
    k.ens = LAUNCH_E;
    k.occ_e = OCC_E;
    k.occ_y = OCC_Y;
    k.box_x = CX;
    k.ry = RY;
    k.box_w_y = BWY;
    k.stages_x = SX;
    k.stages_y = SY;
    k.nw = NW;
    k.smem_x = kSmemX;
    k.smem_y = kSmemY;
    return k;
}

}  // namespace eu
