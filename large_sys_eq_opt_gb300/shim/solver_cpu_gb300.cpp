// solver_cpu_gb300.cpp -- drop-in replacement for the reference's
// src/cpu/solver_cpu.cpp: the functions declared in its
// head/cpu/solver_cpu.hpp, implemented on the GB300 through the C ABI of
// include/euler2d.h.  Compile it against the reference's own headers and
// link it in place of solver_cpu.o:
//
//   g++ -std=c++17 -O2 -I<reference>/head -I<this repo>/include -c solver_cpu_gb300.cpp
//   g++ main_cpu.o test_cases.o init.o solver_cpu_gb300.o -L<pkg> -leuler2d -Wl,-rpath,<pkg>
//
// Semantics follow the reference functions one for one:
//   compute_dt            src/cpu/solver_cpu.cpp:287-309 (throws on a non-positive speed)
//   advance_first_order   src/cpu/solver_cpu.cpp:315-383
//   advance_second_order  src/cpu/solver_cpu.cpp:400-517 (throws on an uninitialised workspace)
// Each call uploads its input Grid2D, runs on the device and downloads the
// outputs (Utmp included), so callers observe the same grids.  One device
// handle per geometry is created on first use and serves every call on that
// geometry: compute_dt needs no Riemann solver, and the advance calls set the
// handle's solver when it changes (the reference passes it per call), so a
// run holds one set of device grids.  The handles are destroyed at process
// exit.  EU_PRECISION=fp32 selects the FP32 form.
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "cpu/solver_cpu.hpp"
#include "euler2d.h"

namespace {

struct Entry {
    int nx, ny;
    double x0, x1, y0, y1;
    int solver;        // the handle's current Riemann solver
    eu_handle* h;
};

std::vector<Entry>& entries() {
    static std::vector<Entry> e;
    return e;
}

// Registered after the first eu_create, so it runs before the CUDA runtime's
// own exit-time teardown (exit handlers run in reverse order).
void destroy_all() {
    for (Entry& e : entries()) eu_destroy(e.h);
    entries().clear();
}

Entry& entry_for(const Grid2D& g) {
    for (Entry& e : entries())
        if (e.nx == g.nx() && e.ny == g.ny() && e.x0 == g.x_min() && e.x1 == g.x_max() && e.y0 == g.y_min() &&
            e.y1 == g.y_max())
            return e;
    if (g.ng() != 2) throw std::runtime_error("GB300 solver: ghost width must be 2");
    const eu_case c{g.nx(), g.ny(), g.ng(), g.x_min(), g.x_max(), g.y_min(), g.y_max(), 0.0, 0.0};
    const char* p = std::getenv("EU_PRECISION");
    const eu_precision prec = (p && std::string(p) == "fp32") ? EU_FP32 : EU_FP64;
    eu_handle* h = nullptr;
    if (eu_create(&c, prec, EU_HLL, EU_LIMITER_MINMOD, nullptr, &h) != EU_OK)
        throw std::runtime_error(std::string("GB300 solver: ") + eu_last_error(nullptr));
    static std::once_flag registered;
    std::call_once(registered, [] { std::atexit(destroy_all); });
    entries().push_back(Entry{g.nx(), g.ny(), g.x_min(), g.x_max(), g.y_min(), g.y_max(), EU_HLL, h});
    return entries().back();
}

const double* raw(const Grid2D& g) { return reinterpret_cast<const double*>(g.data().data()); }
double* raw(Grid2D& g) { return reinterpret_cast<double*>(g.data().data()); }

void check(eu_handle* h, int rc) {
    if (rc == EU_OK) return;
    if (rc == EU_ERR_NONPHYSICAL) throw std::runtime_error("compute_dt: non-positive maximum wave speed.");
    throw std::runtime_error(std::string("GB300 solver: ") + eu_last_error(h));
}

// The geometry's handle, switched to `solver`.
eu_handle* handle_for(const Grid2D& g, int solver) {
    Entry& e = entry_for(g);
    if (e.solver != solver) {
        check(e.h, eu_set_option(e.h, "solver", solver));
        e.solver = solver;
    }
    return e.h;
}

}  // namespace

double compute_dt(const Grid2D& grid, double cfl) {
    eu_handle* h = entry_for(grid).h;   // any solver: the CFL step needs none
    double dt = 0.0;
    check(h, eu_compute_dt_host(h, raw(grid), cfl, &dt));
    return dt;
}

void advance_first_order(const Grid2D& Uold, Grid2D& Unew, double dt, RiemannSolver solver) {
    eu_handle* h = handle_for(Uold, static_cast<int>(solver));
    check(h, eu_advance_first_order_host(h, raw(Uold), raw(Unew), dt));
}

void advance_first_order(const Grid2D& Uold, Grid2D& Unew, double dt) {
    advance_first_order(Uold, Unew, dt, RiemannSolver::HLL);
}

void advance_second_order(const Grid2D& Uold, Grid2D& Utmp, Grid2D& Unew, double dt, CpuWorkspace& ws,
                          RiemannSolver solver) {
    if (!ws.is_initialized()) {
        throw std::runtime_error(
            "advance_second_order: CpuWorkspace not initialised. "
            "Call ws.init(cfg.nx, cfg.ny) before the time loop.");
    }
    eu_handle* h = handle_for(Uold, static_cast<int>(solver));
    check(h, eu_advance_host(h, raw(Uold), raw(Utmp), raw(Unew), dt));
}

void advance_second_order(const Grid2D& Uold, Grid2D& Utmp, Grid2D& Unew, double dt, CpuWorkspace& ws) {
    advance_second_order(Uold, Utmp, Unew, dt, ws, RiemannSolver::HLL);
}
