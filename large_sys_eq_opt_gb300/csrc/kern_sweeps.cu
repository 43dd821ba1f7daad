// kern_sweeps.cu -- instantiates the two sweep kernels for one precision and
// one Riemann solver.  Compiled once per (EU_PREC, EU_SOLVER) pair so the
// eight variants build in parallel; the Riemann solver is a template
// parameter, never a per-face runtime switch.
#include "aux_kernels.h"
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

namespace eu {
namespace {

#if EU_PREC == 32
using T = float;
// x: 4 cells/lane (float4), 4 stages of 128x1x4 boxes.
// y: 2 cells/lane (float2), boxes of 68 columns x 2 rows x 4 fields, 3 stages.
constexpr int VX = 4, SX = 4;
constexpr int VY = 2, RY = 2, OFFY = 2, BWY = 68, SY = 3;
#else
using T = double;
// x: 2 cells/lane (double2), 4 stages of 64x1x4 boxes.
// y: 1 cell/lane, boxes of 36 columns x 2 rows x 4 fields, 3 stages.
constexpr int VX = 2, SX = 4;
constexpr int VY = 1, RY = 2, OFFY = 0, BWY = 36, SY = 3;
#endif
constexpr int NW = 4;
constexpr int SOL = EU_SOLVER;
constexpr size_t kStageX = 4 * 32 * VX * sizeof(T);
constexpr size_t kStageY = 4 * RY * BWY * sizeof(T);
constexpr size_t kSmemX = NW * SX * kStageX + NW * SX * sizeof(uint64_t);
constexpr size_t kSmemY = NW * SY * kStageY + NW * SY * sizeof(uint64_t);
static_assert(kStageX % 128 == 0 && kStageY % 128 == 0, "stage buffers must stay 128-byte aligned");

static cudaError_t LAUNCH_X(const CUtensorMap* tm, const void* args, int ctas, cudaStream_t s) {
    sweep_x_kernel<T, SOL, VX, SX, NW><<<ctas, NW * 32, kSmemX, s>>>(*tm, *static_cast<const SweepArgs<T>*>(args));
    return cudaGetLastError();
}

static cudaError_t LAUNCH_Y(const CUtensorMap* tm, const void* args, int ctas, cudaStream_t s) {
    sweep_y_kernel<T, SOL, VY, RY, BWY, OFFY, SY, NW>
        <<<ctas, NW * 32, kSmemY, s>>>(*tm, *static_cast<const SweepArgs<T>*>(args));
    return cudaGetLastError();
}

}  // namespace

SweepKernels EU_NAME(sweep_kernels, EU_PREC, EU_SOLVER)() {
    SweepKernels k;
    k.x = LAUNCH_X;
    k.y = LAUNCH_Y;
    k.vec_x = VX;
    k.vec_y = VY;
    k.off_y = OFFY;
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
