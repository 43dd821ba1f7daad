// run_shim.cpp -- the reference's CPU time loop (scripts/cpu/main_cpu.cpp:
// 217-262: ghost fill, compute_dt, t_end clip, advance_second_order, swap)
// driven through the GB300 shim, the way the unmodified reference driver
// calls it (TEST INFRASTRUCTURE; built against tests/dropin/cpu/solver_cpu.hpp
// where the reference headers are absent).
//
//   run_shim <in.bin> <out.bin> <solver> [<solver> ...]
// in.bin : int nx, ny; double x_min, x_max, y_min, y_max, cfl, t_end; then
//          the Grid2D AoS grid (4 doubles per cell, ghosts included)
// out.bin: per solver given: long long steps, double t, then the final grid.
// Every run starts from the same input, in one process, so the shim's
// geometry handle is reused across solvers.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "cpu/solver_cpu.hpp"

// head/cpu/boundary_cpu.hpp:5-37 (zero-gradient ghosts, corners included)
static void apply_transmissive_boundary(Grid2D& U) {
    const int ng = U.ng(), ib = ng, ie = ng + U.nx(), jb = ng, je = ng + U.ny();
    for (int j = jb; j < je; ++j)
        for (int g = 0; g < ng; ++g) {
            U(ib - 1 - g, j) = U(ib, j);
            U(ie + g, j) = U(ie - 1, j);
        }
    for (int i = 0; i < U.total_nx(); ++i)
        for (int g = 0; g < ng; ++g) {
            U(i, jb - 1 - g) = U(i, jb);
            U(i, je + g) = U(i, je - 1);
        }
}

static RiemannSolver parse(const std::string& s) {
    if (s == "hll") return RiemannSolver::HLL;
    if (s == "hllc") return RiemannSolver::HLLC;
    if (s == "exact") return RiemannSolver::Exact;
    if (s == "force") return RiemannSolver::FORCE;
    std::fprintf(stderr, "unknown solver %s\n", s.c_str());
    std::exit(2);
}

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: run_shim in.bin out.bin solver...\n");
        return 2;
    }
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int n[2];
    double geo[6];
    if (std::fread(n, sizeof(int), 2, f) != 2 || std::fread(geo, sizeof(double), 6, f) != 6) return 2;
    Grid2D init(n[0], n[1], 2, geo[0], geo[1], geo[2], geo[3]);
    const size_t cells = init.data().size();
    if (std::fread(init.data().data(), sizeof(Conserved), cells, f) != cells) return 2;
    std::fclose(f);
    const double cfl = geo[4], t_end = geo[5];
    FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 2;
    for (int a = 3; a < argc; ++a) {
        const RiemannSolver solver = parse(argv[a]);
        Grid2D U = init;
        Grid2D U_mid(n[0], n[1], 2, geo[0], geo[1], geo[2], geo[3]);
        Grid2D U_next(n[0], n[1], 2, geo[0], geo[1], geo[2], geo[3]);
        CpuWorkspace ws;
        ws.init(n[0], n[1]);
        double t = 0.0;
        long long step = 0;
        try {
            while (t < t_end) {
                apply_transmissive_boundary(U);
                double dt = compute_dt(U, cfl);
                if (t + dt > t_end) dt = t_end - t;
                advance_second_order(U, U_mid, U_next, dt, ws, solver);
                std::swap(U.data(), U_next.data());
                t += dt;
                ++step;
            }
        } catch (const std::exception& e) {
            std::fprintf(stderr, "exception: %s\n", e.what());
            return 1;
        }
        std::fwrite(&step, sizeof(step), 1, o);
        std::fwrite(&t, sizeof(t), 1, o);
        std::fwrite(U.data().data(), sizeof(Conserved), cells, o);
    }
    std::fclose(o);
    // the shim's error path: an uninitialised workspace throws as the reference does
    Grid2D a(4, 4, 2, 0, 1, 0, 1), b(4, 4, 2, 0, 1, 0, 1), c(4, 4, 2, 0, 1, 0, 1);
    CpuWorkspace none;
    try {
        advance_second_order(a, b, c, 1e-3, none, RiemannSolver::HLL);
        std::fprintf(stderr, "no exception for an uninitialised workspace\n");
        return 3;
    } catch (const std::runtime_error&) {
    }
    return 0;
}
