// aux_kernels.h -- launchers of the non-sweep kernels (aux_kernels.cu).
#pragma once
#include "eu_internal.h"

namespace eu {

struct GridGeom {
    int nx, ny;
    double x_min, x_max, y_min, y_max;
};
struct BlastDesc {
    double cx, cy, r, rho_in, p_in, rho_out, p_out;
};
struct ShockBubbleDesc {
    double rho0, p0, mach, shock_x, bub_cx, bub_cy, bub_r, rho_bubble;
};

template <class T> cudaError_t launch_pack_aos(const double* aos, Planes<T> P, int nx, int ny, cudaStream_t s);
template <class T>
cudaError_t launch_unpack_aos(Planes<T> P, int coff, int nx, int ny, const int bc[4], double* aos, cudaStream_t s);
template <class T> cudaError_t launch_fill_ghosts(Planes<T> P, int nx, int ny, const int bc[4], cudaStream_t s);
template <class T>
cudaError_t launch_unpack_snapshot(const T* snap, long long plane, int nx, int ny, const int bc[4], double* aos,
                                   cudaStream_t s);
template <class T> cudaError_t launch_init_blast(Planes<T> P, GridGeom g, BlastDesc b, cudaStream_t s);
template <class T>
cudaError_t launch_init_shock_bubble(Planes<T> P, GridGeom g, ShockBubbleDesc d, cudaStream_t s);
template <class T> cudaError_t launch_dt(Planes<T> P, int nx, int ny, Ctl* ctl, cudaStream_t s);
template <class T>
cudaError_t launch_totals(Planes<T> P, int coff, int nx, int ny, double* part, int max_blocks, double* out,
                          cudaStream_t s);

// Slab decomposition: the step size common to n sub-domains.  Every slab's
// step finalisation has proposed dt = cfl min(dx, dy) / (its own maximum
// signal speed), clipped to t_end; the grid's dt is the smallest proposal
// (x -> c / x is monotone and correctly rounded, so this equals the dt of
// the undivided grid bit for bit), and a status or stop of any slab stops all.
cudaError_t launch_domain_dt(Ctl* const* ctls, int n, cudaStream_t s);

// One entry per (precision, solver) translation unit of kern_sweeps.cu.
SweepKernels sweep_kernels_32_0();
SweepKernels sweep_kernels_32_1();
SweepKernels sweep_kernels_32_2();
SweepKernels sweep_kernels_32_3();
SweepKernels sweep_kernels_64_0();
SweepKernels sweep_kernels_64_1();
SweepKernels sweep_kernels_64_2();
SweepKernels sweep_kernels_64_3();

}  // namespace eu
