// grad_kernels.h -- launchers of the batched parameter-gradient kernels
// (grad_kernels.cu).
#pragma once
#include "euler_numerics.cuh"
#include "eu_internal.h"

namespace eu {

// One instance's scalar case parameters, as eu_case_params, plus the values
// the kernels derive from them on the host: h = min(dx, dy) (blast ramp
// width) and, for a shock-bubble, the post-shock state (rho2, u2, p2) and
// its derivatives with respect to the Mach number.
struct ParamState {
    int kind;        // 0 blast, 1 shock-bubble
    double v[8];
    double h;
    double ps[6];    // rho2, u2, p2, drho2/dM, du2/dM, dp2/dM
};

template <class T>
cudaError_t launch_init_param(Planes<T> P, int nx, int ny, double x0, double y0, double dx, double dy,
                              const ParamState& d, cudaStream_t s);
template <class T>
cudaError_t launch_objective(Planes<T> S, Planes<T> L, int nx, int ny, double x0, double y0, double dx, double dy,
                             const ParamState& d, double* part, int max_blocks, double* J, cudaStream_t s);
template <class T>
cudaError_t launch_tangent_dot(Planes<T> L, int nx, int ny, double x0, double y0, double dx, double dy,
                               const ParamState& d, double* part, int max_blocks, double* out, cudaStream_t s);

}  // namespace eu
