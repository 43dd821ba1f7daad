// Stand-in for the reference's head/cpu/solver_cpu.hpp on a host where the
// reference tree is absent (TEST INFRASTRUCTURE).  It declares the types the
// GB300 shim (large_sys_eq_opt_gb300/shim/solver_cpu_gb300.cpp) compiles
// against with the reference's interface -- the same names, member functions
// and memory layout (head/types.hpp:13-23 Conserved, head/cpu/grid_cpu.hpp:10-89
// Grid2D, head/cpu/solver_cpu.hpp:16-40 CpuWorkspace, head/riemann.hpp:13-18
// RiemannSolver) and the solver entry points of head/cpu/solver_cpu.hpp:42-80
// -- so the shim can be built and run on the GPU host by tests/dropin/run_shim.cpp.
#pragma once
#include <cstddef>
#include <vector>

struct Conserved {
    double rho, rhou, rhov, E;
};

enum class RiemannSolver { HLL, HLLC, Exact, FORCE };

class Grid2D {
public:
    Grid2D() = default;
    Grid2D(int nx, int ny, int ng, double x_min, double x_max, double y_min, double y_max)
        : nx_(nx), ny_(ny), ng_(ng), x_min_(x_min), x_max_(x_max), y_min_(y_min), y_max_(y_max),
          U_(static_cast<std::size_t>(nx + 2 * ng) * (ny + 2 * ng), Conserved{0.0, 0.0, 0.0, 0.0}) {}
    int nx() const { return nx_; }
    int ny() const { return ny_; }
    int ng() const { return ng_; }
    int total_nx() const { return nx_ + 2 * ng_; }
    int total_ny() const { return ny_ + 2 * ng_; }
    double x_min() const { return x_min_; }
    double x_max() const { return x_max_; }
    double y_min() const { return y_min_; }
    double y_max() const { return y_max_; }
    Conserved& operator()(int i, int j) { return U_[static_cast<std::size_t>(j) * total_nx() + i]; }
    std::vector<Conserved>& data() { return U_; }
    const std::vector<Conserved>& data() const { return U_; }

private:
    int nx_ = 0, ny_ = 0, ng_ = 0;
    double x_min_ = 0.0, x_max_ = 1.0, y_min_ = 0.0, y_max_ = 1.0;
    std::vector<Conserved> U_;
};

struct CpuWorkspace {
    int nx = 0, ny = 0;
    void init(int nx_, int ny_) { nx = nx_; ny = ny_; }
    bool is_initialized() const { return nx > 0 && ny > 0; }
};

double compute_dt(const Grid2D& grid, double cfl);
void advance_first_order(const Grid2D& Uold, Grid2D& Unew, double dt, RiemannSolver solver);
void advance_first_order(const Grid2D& Uold, Grid2D& Unew, double dt);
void advance_second_order(const Grid2D& Uold, Grid2D& Utmp, Grid2D& Unew, double dt, CpuWorkspace& ws,
                          RiemannSolver solver);
void advance_second_order(const Grid2D& Uold, Grid2D& Utmp, Grid2D& Unew, double dt, CpuWorkspace& ws);
