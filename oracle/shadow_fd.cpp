// shadow_fd.cpp -- branch-frozen central differences of the CPU restatement
// (TEST INFRASTRUCTURE: checks the discrete adjoint, never shipped).
//
// euler2d_oracle.c is compiled once more with every `double` replaced by
// Shadow, a scalar that carries the unperturbed ("nominal") value in lane 0
// and the values of 2*kDirs perturbed runs, U0 + eps d_k and U0 - eps d_k,
// in the other lanes.  Arithmetic, sqrt and pow act lane by lane; every
// comparison, min/max, fabs and finiteness test is decided on the nominal
// lane alone and that decision is applied to all lanes.  The perturbed
// lanes therefore run the reference algorithm's exact arithmetic
// (src/cpu/solver_cpu.cpp:22-185,400-499, head/physics.hpp:13-74,
// head/riemann.hpp:24-672) along the unperturbed run's branches: the limiter
// picks (minmod's zero branch and the smaller-magnitude argument), the
// physicality fallbacks, the Riemann solvers' upwind cases and fallbacks and
// the exact solver's Newton iteration count are those of the nominal run.
// That map is smooth in the initial state, so (J(+eps) - J(-eps)) / (2 eps)
// converges to the derivative of the discrete scheme along its branches --
// the quantity the hand-written adjoint computes -- with an O(eps^2) error
// instead of the O(1) error a limiter kink crossed inside +-eps adds.
//
// Each comparison also evaluates its outcome in the +eps and -eps lanes of
// every direction; the number of decisions on which they disagree (the
// branch flips an unfrozen pair of runs would take) is counted per
// direction.  Threads: the restatement's OpenMP loops, with per-thread flip
// counters.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace sfd {
constexpr int kDirs = 16;                 // directions per run
constexpr int kLanes = 1 + 2 * kDirs;     // nominal, then (+eps, -eps) per direction
constexpr int kMaxThreads = 512;
static unsigned long long g_flip[kMaxThreads][kDirs];
static inline int tid() {
#ifdef _OPENMP
    const int t = omp_get_thread_num();
    return t < kMaxThreads ? t : kMaxThreads - 1;
#else
    return 0;
#endif
}
}  // namespace sfd

struct Shadow {
    double v[sfd::kLanes];
    Shadow() = default;
    Shadow(double x) {
        for (int k = 0; k < sfd::kLanes; ++k) v[k] = x;
    }
    explicit operator double() const { return v[0]; }
};

#define SFD_LANEWISE(expr)                                       \
    Shadow r;                                                    \
    for (int k = 0; k < sfd::kLanes; ++k) r.v[k] = (expr);       \
    return r

inline Shadow operator+(const Shadow& a, const Shadow& b) { SFD_LANEWISE(a.v[k] + b.v[k]); }
inline Shadow operator-(const Shadow& a, const Shadow& b) { SFD_LANEWISE(a.v[k] - b.v[k]); }
inline Shadow operator*(const Shadow& a, const Shadow& b) { SFD_LANEWISE(a.v[k] * b.v[k]); }
inline Shadow operator/(const Shadow& a, const Shadow& b) { SFD_LANEWISE(a.v[k] / b.v[k]); }
inline Shadow operator-(const Shadow& a) { SFD_LANEWISE(-a.v[k]); }
inline Shadow& operator+=(Shadow& a, const Shadow& b) { return a = a + b; }
inline Shadow& operator-=(Shadow& a, const Shadow& b) { return a = a - b; }
inline Shadow& operator*=(Shadow& a, const Shadow& b) { return a = a * b; }
inline Shadow& operator/=(Shadow& a, const Shadow& b) { return a = a / b; }

// A decision taken on the nominal lane; counts, per direction, whether the
// +eps and -eps lanes would have decided differently.
template <class Cmp> inline bool decide(const Shadow& a, const Shadow& b, Cmp c) {
    unsigned long long* f = sfd::g_flip[sfd::tid()];
    for (int d = 0; d < sfd::kDirs; ++d)
        f[d] += c(a.v[1 + 2 * d], b.v[1 + 2 * d]) != c(a.v[2 + 2 * d], b.v[2 + 2 * d]);
    return c(a.v[0], b.v[0]);
}
inline bool operator<(const Shadow& a, const Shadow& b) { return decide(a, b, [](double x, double y) { return x < y; }); }
inline bool operator<=(const Shadow& a, const Shadow& b) { return decide(a, b, [](double x, double y) { return x <= y; }); }
inline bool operator>(const Shadow& a, const Shadow& b) { return decide(a, b, [](double x, double y) { return x > y; }); }
inline bool operator>=(const Shadow& a, const Shadow& b) { return decide(a, b, [](double x, double y) { return x >= y; }); }
inline bool operator==(const Shadow& a, const Shadow& b) { return decide(a, b, [](double x, double y) { return x == y; }); }
inline bool operator!=(const Shadow& a, const Shadow& b) { return decide(a, b, [](double x, double y) { return x != y; }); }

inline Shadow sqrt(const Shadow& a) { SFD_LANEWISE(std::sqrt(a.v[k])); }
inline Shadow pow(const Shadow& a, const Shadow& b) { SFD_LANEWISE(std::pow(a.v[k], b.v[k])); }
// |a| with the sign taken from the nominal lane (a kink: the branch is frozen)
inline Shadow fabs(const Shadow& a) { return (a < Shadow(0.0)) ? -a : a; }
// fmin / fmax select a whole operand, chosen on the nominal lane
inline Shadow fmin(const Shadow& a, const Shadow& b) { return (b < a) ? b : a; }
inline Shadow fmax(const Shadow& a, const Shadow& b) { return (a < b) ? b : a; }
inline bool isfinite(const Shadow& a) { return std::isfinite(a.v[0]); }

#ifdef _OPENMP
#pragma omp declare reduction(max : Shadow : omp_out = (omp_in > omp_out ? omp_in : omp_out)) \
    initializer(omp_priv = Shadow(0.0))
#endif

// The restatement, its entry points renamed so that this library and
// liboracle_euler2d.so can be loaded into one process side by side.
#define double Shadow
#define orc_grid_doubles sfd_grid_doubles_
#define orc_set_threads sfd_set_threads_
#define orc_get_threads sfd_get_threads_
#define orc_apply_boundary sfd_apply_boundary_
#define orc_compute_dt sfd_compute_dt_
#define orc_advance_second_order sfd_advance_second_order_
#define orc_advance_first_order sfd_advance_first_order_
#define orc_sweep_x sfd_sweep_x_
#define orc_sweep_y sfd_sweep_y_
#define orc_riemann_flux sfd_riemann_flux_
#define orc_run sfd_run_
#define orc_init_reference_case sfd_init_reference_case_
#define orc_init_blast sfd_init_blast_
#define orc_init_shock_bubble sfd_init_shock_bubble_
#include "euler2d_oracle.c"
#undef double

extern "C" {

int sfd_max_dirs(void) { return sfd::kDirs; }

// Frozen-dt forward of the restatement (scripts/cpu/main_cpu.cpp:221-241 with
// dt = dts[s]: ghost fill, then advance_second_order) from U0 and from
// U0 +- eps (d_k^rho, d_k^p) for ndir <= kDirs directions, all along the
// unperturbed run's branches.
//   U0       nominal grid, Grid2D AoS with ghosts (4*(nx+4)*(ny+4) doubles)
//   dirs     ndir directions, each 2*ny*nx doubles: the rho field, then the
//            p field (E moves by eps d^p / (gamma - 1), as u = v = 0 there)
//   mask     ny*nx bytes: J = sum of rho^2 over the interior cells with
//            mask != 0 at the end
//   J        out, 1 + 2*ndir values: nominal, then (+eps, -eps) per direction
//   flips    out, ndir counts of decisions the +eps and -eps lanes disagree on
//   U_out    out (may be NULL): the nominal lane's final grid, AoS
// Returns 0, 1 when ndir is out of range, 2 when memory runs out.
int sfd_frozen_fd(const double* U0, int nx, int ny, double x_min, double x_max, double y_min, double y_max,
                  const int* bc, const double* dts, long long nsteps, int solver, const double* dirs, int ndir,
                  double eps, const unsigned char* mask, double* J, unsigned long long* flips, double* U_out) {
    if (ndir < 1 || ndir > sfd::kDirs) return 1;
    orc_grid g;
    g.nx = nx;
    g.ny = ny;
    g.x_min = x_min;
    g.x_max = x_max;
    g.y_min = y_min;
    g.y_max = y_max;
    for (int s = 0; s < 4; ++s) g.bc[s] = bc ? bc[s] : 0;
    const long long tnx_ = nx + 4, n = 4 * tnx_ * (ny + 4);
    Shadow* U = static_cast<Shadow*>(calloc((size_t)n, sizeof(Shadow)));
    Shadow* Um = static_cast<Shadow*>(calloc((size_t)n, sizeof(Shadow)));
    Shadow* Un = static_cast<Shadow*>(calloc((size_t)n, sizeof(Shadow)));
    Shadow* fx = static_cast<Shadow*>(malloc(sizeof(Shadow) * 4 * (size_t)(nx + 1) * ny));
    Shadow* fy = static_cast<Shadow*>(malloc(sizeof(Shadow) * 4 * (size_t)nx * (ny + 1)));
    if (!U || !Um || !Un || !fx || !fy) {
        free(U); free(Um); free(Un); free(fx); free(fy);
        return 2;
    }
    const double gm1 = 0.3999999999999999;   // head/physics.hpp:11, GAMMA - 1
    for (long long q = 0; q < n; ++q) U[q] = Shadow(U0[q]);
    const long long plane = (long long)nx * ny;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const long long c = 4 * ((long long)(j + 2) * tnx_ + (i + 2));
            for (int d = 0; d < sfd::kDirs; ++d) {
                const double dr = d < ndir ? dirs[(long long)d * 2 * plane + (long long)j * nx + i] : 0.0;
                const double dp = d < ndir ? dirs[(long long)d * 2 * plane + plane + (long long)j * nx + i] : 0.0;
                U[c].v[1 + 2 * d] += eps * dr;
                U[c].v[2 + 2 * d] -= eps * dr;
                U[c + 3].v[1 + 2 * d] += eps * dp / gm1;
                U[c + 3].v[2 + 2 * d] -= eps * dp / gm1;
            }
        }
    memset(sfd::g_flip, 0, sizeof(sfd::g_flip));
    Shadow* cur = U;
    Shadow* nxt = Un;
    for (long long s = 0; s < nsteps; ++s) {
        sfd_apply_boundary_(cur, &g);
        sfd_advance_second_order_(cur, Um, nxt, &g, Shadow(dts[s]), solver, fx, fy);
        Shadow* t = cur; cur = nxt; nxt = t;
    }
    for (int k = 0; k < 1 + 2 * ndir; ++k) J[k] = 0.0;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            if (!mask[(long long)j * nx + i]) continue;
            const Shadow& r = cur[4 * ((long long)(j + 2) * tnx_ + (i + 2))];
            for (int k = 0; k < 1 + 2 * ndir; ++k) J[k] += r.v[k] * r.v[k];
        }
    if (U_out)
        for (long long q = 0; q < n; ++q) U_out[q] = cur[q].v[0];
    for (int d = 0; d < ndir; ++d) {
        unsigned long long t = 0;
        for (int th = 0; th < sfd::kMaxThreads; ++th) t += sfd::g_flip[th][d];
        flips[d] = t;
    }
    free(U); free(Um); free(Un); free(fx); free(fy);
    return 0;
}

}  // extern "C"
