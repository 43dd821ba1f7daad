// opcount.cpp -- floating-point operation counts of the CPU restatement
// (TEST INFRASTRUCTURE: measures the reference algorithm, never shipped).
//
// euler2d_oracle.c is compiled a second time with every `double` replaced by
// Counted, a scalar that holds one double and increments a per-category
// counter on every arithmetic operation, comparison, min/max, sqrt and pow.
// The algorithm, its branch structure and its operation order are therefore
// exactly the restatement's (src/cpu/solver_cpu.cpp:22-185,206-309,400-499,
// head/physics.hpp:13-74, head/riemann.hpp:24-672): the counts are the
// reference CPU path's floating-point work per cell-update, including the
// work it repeats (each cell reconstructed twice per sweep, primitives
// re-derived inside every flux and Riemann call).  Single-threaded (built
// without OpenMP) so the global counters need no atomics.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>

namespace opc {
enum { kAdd, kMul, kDiv, kSqrt, kPow, kCmp, kMinMax, kAbs, kN };
static unsigned long long g_count[kN];
}  // namespace opc

struct Counted {
    double v;
    Counted() = default;
    Counted(double x) : v(x) {}
    explicit operator double() const { return v; }
};
static_assert(sizeof(Counted) == sizeof(double), "Counted must overlay double arrays");

inline Counted operator+(Counted a, Counted b) { ++opc::g_count[opc::kAdd]; return Counted(a.v + b.v); }
inline Counted operator-(Counted a, Counted b) { ++opc::g_count[opc::kAdd]; return Counted(a.v - b.v); }
inline Counted operator*(Counted a, Counted b) { ++opc::g_count[opc::kMul]; return Counted(a.v * b.v); }
inline Counted operator/(Counted a, Counted b) { ++opc::g_count[opc::kDiv]; return Counted(a.v / b.v); }
inline Counted operator-(Counted a) { return Counted(-a.v); }   // a sign flip, not counted
inline Counted& operator+=(Counted& a, Counted b) { a = a + b; return a; }
inline Counted& operator-=(Counted& a, Counted b) { a = a - b; return a; }
inline Counted& operator*=(Counted& a, Counted b) { a = a * b; return a; }
inline Counted& operator/=(Counted& a, Counted b) { a = a / b; return a; }
inline bool operator<(Counted a, Counted b) { ++opc::g_count[opc::kCmp]; return a.v < b.v; }
inline bool operator<=(Counted a, Counted b) { ++opc::g_count[opc::kCmp]; return a.v <= b.v; }
inline bool operator>(Counted a, Counted b) { ++opc::g_count[opc::kCmp]; return a.v > b.v; }
inline bool operator>=(Counted a, Counted b) { ++opc::g_count[opc::kCmp]; return a.v >= b.v; }
inline bool operator==(Counted a, Counted b) { ++opc::g_count[opc::kCmp]; return a.v == b.v; }
inline bool operator!=(Counted a, Counted b) { ++opc::g_count[opc::kCmp]; return a.v != b.v; }
inline Counted sqrt(Counted a) { ++opc::g_count[opc::kSqrt]; return Counted(std::sqrt(a.v)); }
inline Counted pow(Counted a, Counted b) { ++opc::g_count[opc::kPow]; return Counted(std::pow(a.v, b.v)); }
inline Counted fabs(Counted a) { ++opc::g_count[opc::kAbs]; return Counted(std::fabs(a.v)); }
inline Counted fmin(Counted a, Counted b) { ++opc::g_count[opc::kMinMax]; return Counted(std::fmin(a.v, b.v)); }
inline Counted fmax(Counted a, Counted b) { ++opc::g_count[opc::kMinMax]; return Counted(std::fmax(a.v, b.v)); }
inline bool isfinite(Counted a) { ++opc::g_count[opc::kCmp]; return std::isfinite(a.v); }

// The restatement, with its entry points renamed so that this library and
// liboracle_euler2d.so can be loaded into one process side by side.
#define double Counted
#define orc_grid_doubles opc_grid_doubles_
#define orc_set_threads opc_set_threads_
#define orc_get_threads opc_get_threads_
#define orc_apply_boundary opc_apply_boundary_
#define orc_compute_dt opc_compute_dt_
#define orc_advance_second_order opc_advance_second_order_
#define orc_advance_first_order opc_advance_first_order_
#define orc_sweep_x opc_sweep_x_
#define orc_sweep_y opc_sweep_y_
#define orc_riemann_flux opc_riemann_flux_
#define orc_run opc_run_
#define orc_init_reference_case opc_init_reference_case_
#define orc_init_blast opc_init_blast_
#define orc_init_shock_bubble opc_init_shock_bubble_
#include "euler2d_oracle.c"
#undef double

extern "C" {

// Number of counter categories and their names, in output order.
int opc_ncat(void) { return opc::kN; }
const char* opc_cat_name(int k) {
    static const char* names[opc::kN] = {"add", "mul", "div", "sqrt", "pow", "cmp", "minmax", "abs"};
    return (k >= 0 && k < opc::kN) ? names[k] : "";
}

// The time loop of scripts/cpu/main_cpu.cpp:217-262 (ghost fill, compute_dt,
// advance_second_order) for at most max_steps steps on U (AoS with ghosts,
// 4*(nx+4)*(ny+4) doubles, advanced in place), counting every floating-point
// operation of the loop into counts[opc_ncat()].  The grid is given by its
// extents and boundary kinds as in orc_grid.  Returns the number of steps
// taken, or -1 on a non-positive wave speed.
long long opc_run_counted(double* U, int nx, int ny, double x_min, double x_max, double y_min, double y_max,
                          const int* bc, double cfl, double t_end, int solver, long long max_steps,
                          unsigned long long* counts) {
    orc_grid g;
    g.nx = nx;
    g.ny = ny;
    g.x_min = x_min;
    g.x_max = x_max;
    g.y_min = y_min;
    g.y_max = y_max;
    for (int s = 0; s < 4; ++s) g.bc[s] = bc ? bc[s] : 0;
    memset(opc::g_count, 0, sizeof(opc::g_count));
    Counted t = 0.0;
    long long steps = 0;
    const int rc = opc_run_(reinterpret_cast<Counted*>(U), &g, cfl, t_end, solver, max_steps, 0, &t, &steps,
                            nullptr, 0, nullptr, nullptr, nullptr);
    for (int k = 0; k < opc::kN; ++k) counts[k] = opc::g_count[k];
    return rc ? -1 : steps;
}

}  // extern "C"
