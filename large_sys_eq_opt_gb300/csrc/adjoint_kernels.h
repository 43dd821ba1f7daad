// adjoint_kernels.h -- launch interface of the adjoint sweep kernels (not
// part of the public C ABI).
#pragma once
#include <cuda_runtime.h>

namespace eu {

// One adjoint sweep: P is the forward sweep's input state (with its ghost
// frame), A the adjoint of the sweep's interior outputs, G receives the
// adjoint of the sweep's interior inputs (ghost adjoints folded back by the
// boundary rule's transpose).  Each is a plane set of the handle's element
// type; interior cell (i, j) sits at column i + coff, row j + 2.
struct AdjSweepArgs {
    const void* P;
    long long p_pitch, p_plane;
    int p_coff;
    const void* A;
    long long a_pitch, a_plane;
    int a_coff;
    void* G;
    long long g_pitch, g_plane;
    int g_coff;
    int nx, ny;
    double lam_d;      // dt / dx (dir 0) or dt / dy (dir 1)
    int bc_lo, bc_hi;  // dir 0: left/right; dir 1: bottom/top
};

using AdjLaunch = cudaError_t (*)(int dir, const AdjSweepArgs& a, cudaStream_t s);

cudaError_t adjoint_sweep_32_0(int, const AdjSweepArgs&, cudaStream_t);
cudaError_t adjoint_sweep_32_1(int, const AdjSweepArgs&, cudaStream_t);
cudaError_t adjoint_sweep_32_2(int, const AdjSweepArgs&, cudaStream_t);
cudaError_t adjoint_sweep_32_3(int, const AdjSweepArgs&, cudaStream_t);
cudaError_t adjoint_sweep_64_0(int, const AdjSweepArgs&, cudaStream_t);
cudaError_t adjoint_sweep_64_1(int, const AdjSweepArgs&, cudaStream_t);
cudaError_t adjoint_sweep_64_2(int, const AdjSweepArgs&, cudaStream_t);
cudaError_t adjoint_sweep_64_3(int, const AdjSweepArgs&, cudaStream_t);

}  // namespace eu
