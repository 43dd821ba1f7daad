/*
 * euler2d_oracle.h -- CPU restatement of the reference's second-order
 * MUSCL-Hancock split step for the 2D Euler equations (TEST INFRASTRUCTURE).
 *
 * This library is the checker for the CUDA path.  Only the tests, the smoke
 * entry point and bench.py's CPU-baseline leg load it; the product library
 * never links or calls it.
 *
 * It restates, in plain C, the reference's CPU path:
 *   head/types.hpp:13-175        Conserved / Primitive arithmetic
 *   head/physics.hpp:13-74       cons_to_prim, prim_to_cons, sound_speed, flux_x/y
 *   head/riemann.hpp:24-672      HLL, HLLC, FORCE, exact Riemann solvers
 *   src/cpu/solver_cpu.cpp:19-99 limiter, physicality guards, reconstruction
 *   src/cpu/solver_cpu.cpp:106-309,315-499  face fluxes, compute_dt, advance_*
 *   head/cpu/boundary_cpu.hpp:5-37          transmissive boundary
 *   scripts/cpu/main_cpu.cpp:206-262        time loop and snapshot schedule
 * with one addition the reference lacks: a boundary hook (transmissive or
 * reflective per side).  On all-transmissive grids it is bit-identical to the
 * reference build (pinned by tests/golden fixtures produced from the
 * reference itself).
 *
 * Grid storage is the reference Grid2D layout (head/cpu/grid_cpu.hpp:10-89):
 * AoS, 4 doubles per cell (rho, rhou, rhov, E), (nx+4)*(ny+4) cells with a
 * 2-cell ghost frame, row-major index j*(nx+4)+i.
 */
#ifndef EULER2D_ORACLE_H
#define EULER2D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_HLL = 0, ORC_HLLC = 1, ORC_EXACT = 2, ORC_FORCE = 3 };
enum { ORC_BC_TRANSMISSIVE = 0, ORC_BC_REFLECTIVE = 1, ORC_BC_HALO = 2 };
enum { ORC_DIR_X = 0, ORC_DIR_Y = 1 };

typedef struct {
    int nx, ny;                     /* interior cells; ghost width fixed at 2 */
    double x_min, x_max, y_min, y_max;
    int bc[4];                      /* left, right, bottom, top */
} orc_grid;

/* Number of doubles in one AoS grid incl. ghosts: 4*(nx+4)*(ny+4). */
long long orc_grid_doubles(const orc_grid* g);

void orc_set_threads(int n);
int orc_get_threads(void);

/* Ghost fill (head/cpu/boundary_cpu.hpp:5-37 generalised per side;
 * ORC_BC_HALO sides are left to a halo exchange). */
void orc_apply_boundary(double* U, const orc_grid* g);

/* CFL step (src/cpu/solver_cpu.cpp:287-309).  Returns 0 and writes *dt,
 * or returns 1 when the maximum wave speed is not positive (the reference
 * throws std::runtime_error there). */
int orc_compute_dt(const double* U, const orc_grid* g, double cfl, double* dt);

/* One split step (src/cpu/solver_cpu.cpp:400-499): x-sweep Uold->Utmp, BC,
 * y-sweep Utmp->Unew, BC.  fx / fy are face-flux caches of 4*(nx+1)*ny and
 * 4*nx*(ny+1) doubles (CpuWorkspace, head/cpu/solver_cpu.hpp:16-40); pass
 * NULL to have them allocated per call. */
void orc_advance_second_order(const double* Uold, double* Utmp, double* Unew,
                              const orc_grid* g, double dt, int solver,
                              double* fx, double* fy);

/* The two halves of orc_advance_second_order without its ghost fills, for a
 * sub-domain stepper that exchanges halo rows between them: the x-sweep
 * Uold -> Utmp interior, and the y-sweep Utmp (ghost rows included) -> Unew
 * interior.  fx / fy as above, or NULL. */
void orc_sweep_x(const double* Uold, double* Utmp, const orc_grid* g, double dt, int solver, double* fx);
void orc_sweep_y(const double* Utmp, double* Unew, const orc_grid* g, double dt, int solver, double* fy);

/* First-order Godunov step (src/cpu/solver_cpu.cpp:315-369). */
void orc_advance_first_order(const double* Uold, double* Unew,
                             const orc_grid* g, double dt, int solver);

/* Single interface flux (head/riemann.hpp:650-672). UL, UR, F: 4 doubles. */
void orc_riemann_flux(const double* UL, const double* UR, int dir, int solver,
                      double* F);

/* Time loop of scripts/cpu/main_cpu.cpp:206-262 on grid U (in/out).
 * Runs while t < t_end and steps < max_steps (max_steps <= 0: unlimited).
 * dt_log (may be NULL) receives up to dt_cap step sizes.  Snapshot k
 * (1..nsnap) is taken at the first step with t >= t_end*k/nsnap; its step
 * index and time go to snap_step[k-1], snap_t[k-1] (may be NULL) and, when
 * snap_data is non-NULL, the full grid is copied to
 * snap_data + (k-1)*orc_grid_doubles(g).  Returns 0, or 1 on a
 * non-positive wave speed. */
int orc_run(double* U, const orc_grid* g, double cfl, double t_end, int solver,
            long long max_steps, int nsnap,
            double* t_out, long long* steps_out,
            double* dt_log, long long dt_cap,
            long long* snap_step, double* snap_t, double* snap_data);

/* Reference initial states (src/test_cases.cpp:24-101) and the parameterised
 * blast / shock-bubble states of the benchmark configurations.  Fills every
 * cell including ghosts at its cell centre, as src/init.cpp:29-38 does. */
void orc_init_reference_case(double* U, const orc_grid* g, int case_id);
void orc_init_blast(double* U, const orc_grid* g, double cx, double cy, double r,
                    double rho_in, double p_in, double rho_out, double p_out);
void orc_init_shock_bubble(double* U, const orc_grid* g, double rho0, double p0,
                           double mach, double shock_x, double bub_cx,
                           double bub_cy, double bub_r, double rho_bubble);

#ifdef __cplusplus
}
#endif
#endif
