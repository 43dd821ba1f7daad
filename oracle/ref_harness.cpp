// ref_harness.cpp -- extern "C" entry points over the UNMODIFIED reference CPU
// solver (TEST INFRASTRUCTURE).  Built by oracle/Makefile together with the
// reference's own src/cpu/solver_cpu.cpp, src/test_cases.cpp and src/init.cpp
// into oracle/_ref/libref_euler2d.so, only where the reference tree exists.
// It is used to pin the C restatement (euler2d_oracle.c) and to generate the
// golden fixtures under tests/golden/.
//
// Grids are passed as flat AoS arrays in the Grid2D::data() layout
// (head/cpu/grid_cpu.hpp:25,86-88): 4 doubles per cell, (nx+4)*(ny+4) cells.
#include <cstring>
#include <stdexcept>
#include <vector>

#include "cpu/boundary_cpu.hpp"
#include "cpu/grid_cpu.hpp"
#include "cpu/solver_cpu.hpp"
#include "init.hpp"
#include "riemann.hpp"
#include "test_cases.hpp"

namespace {

Grid2D make_grid(int nx, int ny, double x0, double x1, double y0, double y1,
                 const double* aos) {
    Grid2D g(nx, ny, 2, x0, x1, y0, y1);
    if (aos) std::memcpy(g.data().data(), aos, sizeof(double) * 4 * g.data().size());
    return g;
}

void copy_out(const Grid2D& g, double* aos) {
    std::memcpy(aos, g.data().data(), sizeof(double) * 4 * g.data().size());
}

RiemannSolver solver_of(int s) {
    switch (s) {
        case 1: return RiemannSolver::HLLC;
        case 2: return RiemannSolver::Exact;
        case 3: return RiemannSolver::FORCE;
        default: return RiemannSolver::HLL;
    }
}

}  // namespace

extern "C" {

void ref_apply_transmissive_boundary(double* aos, int nx, int ny, double x0, double x1,
                                     double y0, double y1) {
    Grid2D g = make_grid(nx, ny, x0, x1, y0, y1, aos);
    apply_transmissive_boundary(g);
    copy_out(g, aos);
}

// Returns 0 and writes *dt, or 1 when the reference throws.
int ref_compute_dt(const double* aos, int nx, int ny, double x0, double x1, double y0,
                   double y1, double cfl, double* dt) {
    Grid2D g = make_grid(nx, ny, x0, x1, y0, y1, aos);
    try {
        *dt = compute_dt(g, cfl);
    } catch (const std::exception&) {
        return 1;
    }
    return 0;
}

void ref_advance_second_order(const double* uold, double* utmp, double* unew, int nx, int ny,
                              double x0, double x1, double y0, double y1, double dt,
                              int solver) {
    Grid2D a = make_grid(nx, ny, x0, x1, y0, y1, uold);
    Grid2D b = make_grid(nx, ny, x0, x1, y0, y1, utmp);
    Grid2D c = make_grid(nx, ny, x0, x1, y0, y1, unew);
    CpuWorkspace ws;
    ws.init(nx, ny);
    advance_second_order(a, b, c, dt, ws, solver_of(solver));
    copy_out(b, utmp);
    copy_out(c, unew);
}

void ref_advance_first_order(const double* uold, double* unew, int nx, int ny, double x0,
                             double x1, double y0, double y1, double dt, int solver) {
    Grid2D a = make_grid(nx, ny, x0, x1, y0, y1, uold);
    Grid2D c = make_grid(nx, ny, x0, x1, y0, y1, unew);
    advance_first_order(a, c, dt, solver_of(solver));
    copy_out(c, unew);
}

void ref_riemann_flux(const double* ul, const double* ur, int dir, int solver, double* f) {
    const Conserved L(ul[0], ul[1], ul[2], ul[3]);
    const Conserved R(ur[0], ur[1], ur[2], ur[3]);
    const Conserved F = riemann_flux(L, R, dir == 0 ? Direction::X : Direction::Y,
                                     solver_of(solver));
    f[0] = F.rho; f[1] = F.rhou; f[2] = F.rhov; f[3] = F.E;
}

// Reference case geometry (src/test_cases.cpp:132-162,184-195):
// out[0..8] = nx, ny, ng, x_min, x_max, y_min, y_max, cfl, t_end.
void ref_case_config(int case_id, int n, double* out) {
    const CaseConfig c = get_n_case_config(case_id == 0 ? CaseId::ShockBubble : CaseId::BlastWave, n);
    out[0] = c.nx; out[1] = c.ny; out[2] = c.ng; out[3] = c.x_min; out[4] = c.x_max;
    out[5] = c.y_min; out[6] = c.y_max; out[7] = c.cfl; out[8] = c.t_end;
}

// make_n_grid (src/init.cpp:53-56) into a caller buffer sized from ref_case_config.
void ref_init_case(int case_id, int n, double* aos) {
    Grid2D g = make_n_grid(case_id == 0 ? CaseId::ShockBubble : CaseId::BlastWave, n);
    copy_out(g, aos);
}

// The time loop of scripts/cpu/main_cpu.cpp:206-262 on a caller grid.
int ref_run(double* aos, int nx, int ny, double x0, double x1, double y0, double y1,
            double cfl, double t_end, int solver, long long max_steps, int nsnap,
            double* t_out, long long* steps_out, double* dt_log, long long dt_cap,
            long long* snap_step, double* snap_t) {
    Grid2D U = make_grid(nx, ny, x0, x1, y0, y1, aos);
    Grid2D U_mid(nx, ny, 2, x0, x1, y0, y1);
    Grid2D U_next(nx, ny, 2, x0, x1, y0, y1);
    CpuWorkspace ws;
    ws.init(nx, ny);
    std::vector<double> snapshot_times;
    for (int k = 1; k <= nsnap; ++k)
        snapshot_times.push_back(t_end * static_cast<double>(k) / static_cast<double>(nsnap));
    double t = 0.0;
    long long step = 0;
    int next_snapshot = 0;
    int rc = 0;
    try {
        while (t < t_end && (max_steps <= 0 || step < max_steps)) {
            apply_transmissive_boundary(U);
            double dt = compute_dt(U, cfl);
            if (t + dt > t_end) dt = t_end - t;
            advance_second_order(U, U_mid, U_next, dt, ws, solver_of(solver));
            std::swap(U, U_next);
            if (dt_log && step < dt_cap) dt_log[step] = dt;
            t += dt;
            ++step;
            while (next_snapshot < nsnap && t >= snapshot_times[next_snapshot]) {
                if (snap_step) snap_step[next_snapshot] = step;
                if (snap_t) snap_t[next_snapshot] = t;
                ++next_snapshot;
            }
        }
    } catch (const std::exception&) {
        rc = 1;
    }
    copy_out(U, aos);
    if (t_out) *t_out = t;
    if (steps_out) *steps_out = step;
    return rc;
}

}  // extern "C"
