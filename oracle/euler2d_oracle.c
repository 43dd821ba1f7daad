/*
 * euler2d_oracle.c -- CPU restatement of the reference MUSCL-Hancock split
 * step (TEST INFRASTRUCTURE: the checker for the CUDA path, never shipped).
 *
 * Every function below names the reference lines it restates.  The order of
 * floating-point operations follows the reference expression by expression
 * (C++ operators on Conserved/Primitive are component-wise and
 * left-associative, head/types.hpp:49-175), and the library is compiled with
 * -ffp-contract=off so no FMA contraction changes a rounding.  On grids whose
 * four sides are transmissive the results are bit-identical to the reference
 * CPU build (tests/golden fixtures pin this).
 */
#include "euler2d_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* head/physics.hpp:11 */
#define GAMMA 1.4
/* src/cpu/solver_cpu.cpp:19-20 */
#define RHO_FLOOR 1.0e-12
#define P_FLOOR 1.0e-12

typedef struct { double rho, rhou, rhov, E; } cons_t;   /* head/types.hpp:13-23 */
typedef struct { double rho, u, v, p; } prim_t;         /* head/types.hpp:25-35 */

/* ------------------------------------------------------------------------ */
/* head/types.hpp:49-111 component-wise arithmetic                          */
/* ------------------------------------------------------------------------ */
static inline cons_t c_make(double a, double b, double c, double d) {
    cons_t r; r.rho = a; r.rhou = b; r.rhov = c; r.E = d; return r;
}
static inline cons_t c_add(cons_t a, cons_t b) {
    return c_make(a.rho + b.rho, a.rhou + b.rhou, a.rhov + b.rhov, a.E + b.E);
}
static inline cons_t c_sub(cons_t a, cons_t b) {
    return c_make(a.rho - b.rho, a.rhou - b.rhou, a.rhov - b.rhov, a.E - b.E);
}
static inline cons_t c_scale(double s, cons_t a) {
    return c_make(s * a.rho, s * a.rhou, s * a.rhov, s * a.E);
}
static inline cons_t c_div(cons_t a, double s) {
    return c_make(a.rho / s, a.rhou / s, a.rhov / s, a.E / s);
}
static inline prim_t p_make(double a, double b, double c, double d) {
    prim_t r; r.rho = a; r.u = b; r.v = c; r.p = d; return r;
}
static inline prim_t p_sub(prim_t a, prim_t b) {
    return p_make(a.rho - b.rho, a.u - b.u, a.v - b.v, a.p - b.p);
}
static inline prim_t p_add(prim_t a, prim_t b) {
    return p_make(a.rho + b.rho, a.u + b.u, a.v + b.v, a.p + b.p);
}
static inline prim_t p_scale(double s, prim_t a) {
    return p_make(s * a.rho, s * a.u, s * a.v, s * a.p);
}

/* ------------------------------------------------------------------------ */
/* head/physics.hpp                                                         */
/* ------------------------------------------------------------------------ */
/* head/physics.hpp:13-20 */
static inline prim_t cons_to_prim(cons_t U) {
    const double inv_rho = 1.0 / U.rho;
    const double u = U.rhou * inv_rho;
    const double v = U.rhov * inv_rho;
    const double kinetic = 0.5 * U.rho * (u * u + v * v);
    const double p = (GAMMA - 1.0) * (U.E - kinetic);
    return p_make(U.rho, u, v, p);
}
/* head/physics.hpp:22-28 */
static inline cons_t prim_to_cons(prim_t V) {
    const double rhou = V.rho * V.u;
    const double rhov = V.rho * V.v;
    const double kinetic = 0.5 * V.rho * (V.u * V.u + V.v * V.v);
    const double E = V.p / (GAMMA - 1.0) + kinetic;
    return c_make(V.rho, rhou, rhov, E);
}
/* head/physics.hpp:39-41 */
static inline double sound_speed(prim_t V) { return sqrt(GAMMA * V.p / V.rho); }

/* head/physics.hpp:56-74 + head/riemann.hpp:24-30 */
static inline cons_t physical_flux(cons_t U, int dir) {
    const prim_t V = cons_to_prim(U);
    if (dir == ORC_DIR_X)
        return c_make(U.rhou, U.rhou * V.u + V.p, U.rhov * V.u, (U.E + V.p) * V.u);
    return c_make(U.rhov, U.rhou * V.v, U.rhov * V.v + V.p, (U.E + V.p) * V.v);
}

/* head/riemann.hpp:32-38 */
static inline double normal_velocity(prim_t V, int dir) { return dir == ORC_DIR_X ? V.u : V.v; }
static inline double tangential_velocity(prim_t V, int dir) { return dir == ORC_DIR_X ? V.v : V.u; }

/* head/riemann.hpp:40-64 */
static inline cons_t make_conserved_nt(double rho, double un, double ut, double p, int dir) {
    double u, v;
    if (dir == ORC_DIR_X) { u = un; v = ut; } else { u = ut; v = un; }
    return c_make(rho, rho * u, rho * v,
                  p / (GAMMA - 1.0) + 0.5 * rho * (u * u + v * v));
}

/* head/riemann.hpp:66-81 */
static inline int prim_physical_riemann(prim_t V) {
    return isfinite(V.rho) && isfinite(V.u) && isfinite(V.v) && isfinite(V.p) &&
           V.rho > 0.0 && V.p > 0.0;
}

/* ------------------------------------------------------------------------ */
/* Riemann solvers                                                          */
/* ------------------------------------------------------------------------ */
/* head/riemann.hpp:87-129 */
static cons_t hll_flux(cons_t UL, cons_t UR, int dir) {
    const prim_t VL = cons_to_prim(UL);
    const prim_t VR = cons_to_prim(UR);
    if (!prim_physical_riemann(VL) || !prim_physical_riemann(VR)) {
        const cons_t FL = physical_flux(UL, dir);
        const cons_t FR = physical_flux(UR, dir);
        return c_scale(0.5, c_add(FL, FR));
    }
    const double aL = sound_speed(VL), aR = sound_speed(VR);
    const double unL = normal_velocity(VL, dir), unR = normal_velocity(VR, dir);
    const double SL = fmin(unL - aL, unR - aR);
    const double SR = fmax(unL + aL, unR + aR);
    const cons_t FL = physical_flux(UL, dir);
    const cons_t FR = physical_flux(UR, dir);
    if (SL >= 0.0) return FL;
    if (SR <= 0.0) return FR;
    const double denom = SR - SL;
    if (fabs(denom) < 1.0e-14) return c_scale(0.5, c_add(FL, FR));
    /* (SR*FL - SL*FR + (SL*SR)*(UR-UL)) / denom */
    return c_div(c_add(c_sub(c_scale(SR, FL), c_scale(SL, FR)),
                       c_scale(SL * SR, c_sub(UR, UL))),
                 denom);
}

/* head/riemann.hpp:135-186 */
static cons_t hllc_star_state(cons_t U, prim_t V, double S, double Sstar, int dir) {
    const double rho = V.rho, p = V.p;
    const double un = normal_velocity(V, dir), ut = tangential_velocity(V, dir);
    const double denom = S - Sstar;
    if (fabs(denom) < 1.0e-14) return U;
    const double rho_star = rho * (S - un) / denom;
    if (!isfinite(rho_star) || rho_star <= 0.0) return U;
    const double E_per_rho = U.E / rho;
    const double E_star = rho_star * (E_per_rho + (Sstar - un) * (Sstar + p / (rho * (S - un))));
    if (!isfinite(E_star)) return U;
    if (dir == ORC_DIR_X) return c_make(rho_star, rho_star * Sstar, rho_star * ut, E_star);
    return c_make(rho_star, rho_star * ut, rho_star * Sstar, E_star);
}

/* head/riemann.hpp:192-271 */
static cons_t hllc_flux(cons_t UL, cons_t UR, int dir) {
    const prim_t VL = cons_to_prim(UL);
    const prim_t VR = cons_to_prim(UR);
    if (!prim_physical_riemann(VL) || !prim_physical_riemann(VR)) return hll_flux(UL, UR, dir);
    const double aL = sound_speed(VL), aR = sound_speed(VR);
    const double unL = normal_velocity(VL, dir), unR = normal_velocity(VR, dir);
    const double pL = VL.p, pR = VR.p, rhoL = VL.rho, rhoR = VR.rho;
    const double SL = fmin(unL - aL, unR - aR);
    const double SR = fmax(unL + aL, unR + aR);
    const cons_t FL = physical_flux(UL, dir);
    const cons_t FR = physical_flux(UR, dir);
    if (SL >= 0.0) return FL;
    if (SR <= 0.0) return FR;
    const double numerator = pR - pL + rhoL * unL * (SL - unL) - rhoR * unR * (SR - unR);
    const double denominator = rhoL * (SL - unL) - rhoR * (SR - unR);
    if (fabs(denominator) < 1.0e-14) return hll_flux(UL, UR, dir);
    const double Sstar = numerator / denominator;
    if (!isfinite(Sstar)) return hll_flux(UL, UR, dir);
    if (Sstar >= 0.0) {
        const cons_t Us = hllc_star_state(UL, VL, SL, Sstar, dir);
        return c_add(FL, c_scale(SL, c_sub(Us, UL)));
    } else {
        const cons_t Us = hllc_star_state(UR, VR, SR, Sstar, dir);
        return c_add(FR, c_scale(SR, c_sub(Us, UR)));
    }
}

/* head/riemann.hpp:284-325 (local-alpha FORCE) */
static cons_t force_flux(cons_t UL, cons_t UR, int dir) {
    const prim_t VL = cons_to_prim(UL);
    const prim_t VR = cons_to_prim(UR);
    if (!prim_physical_riemann(VL) || !prim_physical_riemann(VR)) return hll_flux(UL, UR, dir);
    const double aL = sound_speed(VL), aR = sound_speed(VR);
    const double unL = normal_velocity(VL, dir), unR = normal_velocity(VR, dir);
    const double alpha = fmax(fabs(unL) + aL, fabs(unR) + aR);
    const cons_t FL = physical_flux(UL, dir);
    const cons_t FR = physical_flux(UR, dir);
    if (!isfinite(alpha) || alpha <= 1.0e-14) return c_scale(0.5, c_add(FL, FR));
    const cons_t F_lf = c_sub(c_scale(0.5, c_add(FL, FR)), c_scale(0.5 * alpha, c_sub(UR, UL)));
    const cons_t U_ri = c_sub(c_scale(0.5, c_add(UL, UR)), c_scale(0.5 * (1.0 / alpha), c_sub(FR, FL)));
    const prim_t V_ri = cons_to_prim(U_ri);
    if (!prim_physical_riemann(V_ri)) return F_lf;
    const cons_t F_ri = physical_flux(U_ri, dir);
    return c_scale(0.5, c_add(F_lf, F_ri));
}

/* head/riemann.hpp:331-359 */
static void exact_pressure_function(double p, double rhoK, double pK, double aK,
                                    double* f, double* fd) {
    if (p > pK) {
        const double A = 2.0 / ((GAMMA + 1.0) * rhoK);
        const double B = (GAMMA - 1.0) / (GAMMA + 1.0) * pK;
        const double q = sqrt(A / (p + B));
        *f = (p - pK) * q;
        *fd = q * (1.0 - 0.5 * (p - pK) / (p + B));
    } else {
        const double pratio = p / pK;
        const double expo = (GAMMA - 1.0) / (2.0 * GAMMA);
        *f = 2.0 * aK / (GAMMA - 1.0) * (pow(pratio, expo) - 1.0);
        *fd = (1.0 / (rhoK * aK)) * pow(pratio, -(GAMMA + 1.0) / (2.0 * GAMMA));
    }
}

/* head/riemann.hpp:361-377 (PVRS guess) */
static double exact_guess_pressure(prim_t VL, prim_t VR, int dir) {
    const double aL = sound_speed(VL), aR = sound_speed(VR);
    const double unL = normal_velocity(VL, dir), unR = normal_velocity(VR, dir);
    const double p_pvrs = 0.5 * (VL.p + VR.p) - 0.125 * (unR - unL) * (VL.rho + VR.rho) * (aL + aR);
    return fmax(1.0e-12, p_pvrs);
}

/* head/riemann.hpp:379-443 (Newton for p*, u*) */
static int exact_star_pressure_velocity(prim_t VL, prim_t VR, int dir,
                                        double* p_star_out, double* u_star_out) {
    const double rhoL = VL.rho, rhoR = VR.rho, pL = VL.p, pR = VR.p;
    const double aL = sound_speed(VL), aR = sound_speed(VR);
    const double unL = normal_velocity(VL, dir), unR = normal_velocity(VR, dir);
    double p_star = exact_guess_pressure(VL, VR, dir);
    for (int iter = 0; iter < 20; ++iter) {
        double fL = 0.0, fR = 0.0, fdL = 0.0, fdR = 0.0;
        exact_pressure_function(p_star, rhoL, pL, aL, &fL, &fdL);
        exact_pressure_function(p_star, rhoR, pR, aR, &fR, &fdR);
        const double f = fL + fR + (unR - unL);
        const double fd = fdL + fdR;
        if (fabs(fd) < 1.0e-14) { *p_star_out = p_star; return 0; }
        const double p_old = p_star;
        p_star = p_old - f / fd;
        if (!isfinite(p_star) || p_star <= 0.0) p_star = 0.5 * p_old;
        if (fabs(p_star - p_old) / (0.5 * (p_star + p_old) + 1.0e-14) < 1.0e-8) break;
    }
    *p_star_out = p_star;
    if (!isfinite(p_star) || p_star <= 0.0) return 0;
    double fL = 0.0, fR = 0.0, dL = 0.0, dR = 0.0;
    exact_pressure_function(p_star, rhoL, pL, aL, &fL, &dL);
    exact_pressure_function(p_star, rhoR, pR, aR, &fR, &dR);
    const double u_star = 0.5 * (unL + unR + fR - fL);
    *u_star_out = u_star;
    return isfinite(u_star);
}

/* head/riemann.hpp:445-517 */
static cons_t exact_sample_left(prim_t VL, double p_star, double u_star, int dir) {
    const double rhoL = VL.rho, pL = VL.p;
    const double unL = normal_velocity(VL, dir), utL = tangential_velocity(VL, dir);
    const double aL = sound_speed(VL);
    const double xi = 0.0;
    double rho = rhoL, un = unL, p = pL;
    if (p_star > pL) {
        const double p_ratio = p_star / pL;
        const double SL = unL - aL * sqrt((GAMMA + 1.0) / (2.0 * GAMMA) * p_ratio +
                                          (GAMMA - 1.0) / (2.0 * GAMMA));
        if (xi <= SL) {
            rho = rhoL; un = unL; p = pL;
        } else {
            rho = rhoL * ((p_ratio + (GAMMA - 1.0) / (GAMMA + 1.0)) /
                          ((GAMMA - 1.0) / (GAMMA + 1.0) * p_ratio + 1.0));
            un = u_star; p = p_star;
        }
    } else {
        const double a_star = aL * pow(p_star / pL, (GAMMA - 1.0) / (2.0 * GAMMA));
        const double SHL = unL - aL;
        const double STL = u_star - a_star;
        if (xi <= SHL) {
            rho = rhoL; un = unL; p = pL;
        } else if (xi >= STL) {
            rho = rhoL * pow(p_star / pL, 1.0 / GAMMA);
            un = u_star; p = p_star;
        } else {
            const double a = 2.0 / (GAMMA + 1.0) * (aL + 0.5 * (GAMMA - 1.0) * (unL - xi));
            un = 2.0 / (GAMMA + 1.0) * (aL + 0.5 * (GAMMA - 1.0) * unL + xi);
            const double aratio = a / aL;
            rho = rhoL * pow(aratio, 2.0 / (GAMMA - 1.0));
            p = pL * pow(aratio, 2.0 * GAMMA / (GAMMA - 1.0));
        }
    }
    return make_conserved_nt(rho, un, utL, p, dir);
}

/* head/riemann.hpp:519-591 */
static cons_t exact_sample_right(prim_t VR, double p_star, double u_star, int dir) {
    const double rhoR = VR.rho, pR = VR.p;
    const double unR = normal_velocity(VR, dir), utR = tangential_velocity(VR, dir);
    const double aR = sound_speed(VR);
    const double xi = 0.0;
    double rho = rhoR, un = unR, p = pR;
    if (p_star > pR) {
        const double p_ratio = p_star / pR;
        const double SR = unR + aR * sqrt((GAMMA + 1.0) / (2.0 * GAMMA) * p_ratio +
                                          (GAMMA - 1.0) / (2.0 * GAMMA));
        if (xi >= SR) {
            rho = rhoR; un = unR; p = pR;
        } else {
            rho = rhoR * ((p_ratio + (GAMMA - 1.0) / (GAMMA + 1.0)) /
                          ((GAMMA - 1.0) / (GAMMA + 1.0) * p_ratio + 1.0));
            un = u_star; p = p_star;
        }
    } else {
        const double a_star = aR * pow(p_star / pR, (GAMMA - 1.0) / (2.0 * GAMMA));
        const double SHR = unR + aR;
        const double STR = u_star + a_star;
        if (xi >= SHR) {
            rho = rhoR; un = unR; p = pR;
        } else if (xi <= STR) {
            rho = rhoR * pow(p_star / pR, 1.0 / GAMMA);
            un = u_star; p = p_star;
        } else {
            const double a = 2.0 / (GAMMA + 1.0) * (aR - 0.5 * (GAMMA - 1.0) * (unR - xi));
            un = 2.0 / (GAMMA + 1.0) * (-aR + 0.5 * (GAMMA - 1.0) * unR + xi);
            const double aratio = a / aR;
            rho = rhoR * pow(aratio, 2.0 / (GAMMA - 1.0));
            p = pR * pow(aratio, 2.0 * GAMMA / (GAMMA - 1.0));
        }
    }
    return make_conserved_nt(rho, un, utR, p, dir);
}

/* head/riemann.hpp:601-644 */
static cons_t exact_flux(cons_t UL, cons_t UR, int dir) {
    const prim_t VL = cons_to_prim(UL);
    const prim_t VR = cons_to_prim(UR);
    if (!prim_physical_riemann(VL) || !prim_physical_riemann(VR)) return hll_flux(UL, UR, dir);
    double p_star = 0.0, u_star = 0.0;
    const int ok = exact_star_pressure_velocity(VL, VR, dir, &p_star, &u_star);
    if (!ok || !isfinite(p_star) || !isfinite(u_star) || p_star <= 0.0) return hll_flux(UL, UR, dir);
    const cons_t Us = (u_star >= 0.0) ? exact_sample_left(VL, p_star, u_star, dir)
                                      : exact_sample_right(VR, p_star, u_star, dir);
    const prim_t Vs = cons_to_prim(Us);
    if (!prim_physical_riemann(Vs)) return hll_flux(UL, UR, dir);
    return physical_flux(Us, dir);
}

/* head/riemann.hpp:650-672 */
static inline cons_t riemann_flux(cons_t UL, cons_t UR, int dir, int solver) {
    switch (solver) {
        case ORC_HLLC: return hllc_flux(UL, UR, dir);
        case ORC_EXACT: return exact_flux(UL, UR, dir);
        case ORC_FORCE: return force_flux(UL, UR, dir);
        default: return hll_flux(UL, UR, dir);
    }
}

/* ------------------------------------------------------------------------ */
/* src/cpu/solver_cpu.cpp:22-99 limiter and MUSCL-Hancock reconstruction    */
/* ------------------------------------------------------------------------ */
static inline double minmod_scalar(double a, double b) {
    if (a * b <= 0.0) return 0.0;
    /* std::min(a,b) = (b < a) ? b : a ; std::max(a,b) = (a < b) ? b : a */
    return (a > 0.0) ? ((b < a) ? b : a) : ((a < b) ? b : a);
}
static inline int is_physical(prim_t V) {
    return isfinite(V.rho) && isfinite(V.u) && isfinite(V.v) && isfinite(V.p) &&
           (V.rho > RHO_FLOOR) && (V.p > P_FLOOR);
}
static inline void reconstruct(cons_t Um, cons_t Uc, cons_t Up, double dt_over_d, int dir,
                               cons_t* UL_star, cons_t* UR_star) {
    const prim_t Wm = cons_to_prim(Um);
    const prim_t Wc = cons_to_prim(Uc);
    const prim_t Wp = cons_to_prim(Up);
    const prim_t a = p_sub(Wc, Wm), b = p_sub(Wp, Wc);
    const prim_t slope = p_make(minmod_scalar(a.rho, b.rho), minmod_scalar(a.u, b.u),
                                minmod_scalar(a.v, b.v), minmod_scalar(a.p, b.p));
    prim_t WL = p_sub(Wc, p_scale(0.5, slope));
    prim_t WR = p_add(Wc, p_scale(0.5, slope));
    if (!is_physical(WL)) WL = Wc;
    if (!is_physical(WR)) WR = Wc;
    const cons_t UL = prim_to_cons(WL);
    const cons_t UR = prim_to_cons(WR);
    const cons_t FL = physical_flux(UL, dir);
    const cons_t FR = physical_flux(UR, dir);
    const cons_t half = c_scale(0.5 * dt_over_d, c_sub(FR, FL));
    const cons_t cl = c_sub(UL, half);
    const cons_t cr = c_sub(UR, half);
    *UL_star = is_physical(cons_to_prim(cl)) ? cl : UL;
    *UR_star = is_physical(cons_to_prim(cr)) ? cr : UR;
}

/* ------------------------------------------------------------------------ */
/* Grid helpers (head/cpu/grid_cpu.hpp:10-89)                               */
/* ------------------------------------------------------------------------ */
#define NG 2
static inline long long tnx(const orc_grid* g) { return (long long)g->nx + 2 * NG; }
static inline long long tny(const orc_grid* g) { return (long long)g->ny + 2 * NG; }
static inline cons_t ld(const double* U, const orc_grid* g, int i, int j) {
    const double* p = U + 4 * ((long long)j * tnx(g) + i);
    return c_make(p[0], p[1], p[2], p[3]);
}
static inline void st(double* U, const orc_grid* g, int i, int j, cons_t v) {
    double* p = U + 4 * ((long long)j * tnx(g) + i);
    p[0] = v.rho; p[1] = v.rhou; p[2] = v.rhov; p[3] = v.E;
}
static inline double gdx(const orc_grid* g) { return (g->x_max - g->x_min) / (double)g->nx; }
static inline double gdy(const orc_grid* g) { return (g->y_max - g->y_min) / (double)g->ny; }

long long orc_grid_doubles(const orc_grid* g) { return 4 * tnx(g) * tny(g); }

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* head/cpu/boundary_cpu.hpp:5-37, generalised: each ghost layer g copies the
 * nearest interior cell (transmissive) or mirrors cell g with the normal
 * momentum negated (reflective).  x pass over interior rows, then y pass
 * over every column so corners take the y rule of the x ghosts.  A side of
 * kind ORC_BC_HALO (an internal side of a sub-domain) is left untouched: its
 * ghosts are a neighbour's cells, filled by a halo exchange. */
void orc_apply_boundary(double* U, const orc_grid* g) {
    const int ib = NG, ie = NG + g->nx, jb = NG, je = NG + g->ny;
    const int total_nx = (int)tnx(g);
    for (int j = jb; j < je; ++j) {
        for (int k = 0; k < NG && g->bc[0] != ORC_BC_HALO; ++k) {
            if (g->bc[0] == ORC_BC_REFLECTIVE) {
                cons_t s = ld(U, g, ib + k, j); s.rhou = -s.rhou; st(U, g, ib - 1 - k, j, s);
            } else {
                st(U, g, ib - 1 - k, j, ld(U, g, ib, j));
            }
        }
        for (int k = 0; k < NG && g->bc[1] != ORC_BC_HALO; ++k) {
            if (g->bc[1] == ORC_BC_REFLECTIVE) {
                cons_t s = ld(U, g, ie - 1 - k, j); s.rhou = -s.rhou; st(U, g, ie + k, j, s);
            } else {
                st(U, g, ie + k, j, ld(U, g, ie - 1, j));
            }
        }
    }
    for (int i = 0; i < total_nx; ++i) {
        for (int k = 0; k < NG && g->bc[2] != ORC_BC_HALO; ++k) {
            if (g->bc[2] == ORC_BC_REFLECTIVE) {
                cons_t s = ld(U, g, i, jb + k); s.rhov = -s.rhov; st(U, g, i, jb - 1 - k, s);
            } else {
                st(U, g, i, jb - 1 - k, ld(U, g, i, jb));
            }
        }
        for (int k = 0; k < NG && g->bc[3] != ORC_BC_HALO; ++k) {
            if (g->bc[3] == ORC_BC_REFLECTIVE) {
                cons_t s = ld(U, g, i, je - 1 - k); s.rhov = -s.rhov; st(U, g, i, je + k, s);
            } else {
                st(U, g, i, je + k, ld(U, g, i, je - 1));
            }
        }
    }
}

/* src/cpu/solver_cpu.cpp:287-309 */
int orc_compute_dt(const double* U, const orc_grid* g, double cfl, double* dt) {
    double max_speed = 0.0;
    const int jb = NG, je = NG + g->ny, ib = NG, ie = NG + g->nx;
#ifdef _OPENMP
#pragma omp parallel for collapse(2) reduction(max : max_speed) schedule(static)
#endif
    for (int j = jb; j < je; ++j) {
        for (int i = ib; i < ie; ++i) {
            const prim_t V = cons_to_prim(ld(U, g, i, j));
            const double a = sound_speed(V);
            const double sx = fabs(V.u) + a;
            const double sy = fabs(V.v) + a;
            const double m = (sx < sy) ? sy : sx;
            max_speed = (max_speed < m) ? m : max_speed;
        }
    }
    if (max_speed <= 0.0) return 1;
    const double dx = gdx(g), dy = gdy(g);
    *dt = cfl * ((dy < dx) ? dy : dx) / max_speed;
    return 0;
}

/* src/cpu/solver_cpu.cpp:106-144 */
static inline cons_t muscl_flux_x(const double* U, const orc_grid* g, int i, int j,
                                  double lam, int solver) {
    cons_t a_l, a_r, b_l, b_r;
    reconstruct(ld(U, g, i - 1, j), ld(U, g, i, j), ld(U, g, i + 1, j), lam, ORC_DIR_X, &a_l, &a_r);
    reconstruct(ld(U, g, i, j), ld(U, g, i + 1, j), ld(U, g, i + 2, j), lam, ORC_DIR_X, &b_l, &b_r);
    return riemann_flux(a_r, b_l, ORC_DIR_X, solver);
}
/* src/cpu/solver_cpu.cpp:147-185 */
static inline cons_t muscl_flux_y(const double* U, const orc_grid* g, int i, int j,
                                  double lam, int solver) {
    cons_t a_l, a_r, b_l, b_r;
    reconstruct(ld(U, g, i, j - 1), ld(U, g, i, j), ld(U, g, i, j + 1), lam, ORC_DIR_Y, &a_l, &a_r);
    reconstruct(ld(U, g, i, j), ld(U, g, i, j + 1), ld(U, g, i, j + 2), lam, ORC_DIR_Y, &b_l, &b_r);
    return riemann_flux(a_r, b_l, ORC_DIR_Y, solver);
}

/* The x half of src/cpu/solver_cpu.cpp:400-499: fill_x_face_cache
 * (:206-238) and the x update (:437-457) of Utmp's interior from Uold; no
 * ghost fill.  fx: 4*(nx+1)*ny doubles or NULL. */
void orc_sweep_x(const double* Uold, double* Utmp, const orc_grid* g, double dt, int solver, double* fx) {
    const int ib = NG, ie = NG + g->nx, jb = NG, je = NG + g->ny;
    const int nx = g->nx, ny = g->ny;
    const int nx_faces = nx + 1;
    double* fx_own = NULL;
    if (!fx) fx = fx_own = (double*)malloc(sizeof(double) * 4 * (size_t)(nx + 1) * ny);
    const double dt_over_dx = dt / gdx(g);
    {
        const double lam = dt / gdx(g);   /* recomputed in fill_x_face_cache */
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
        for (int j = jb; j < je; ++j)
            for (int i = ib - 1; i < ie; ++i) {
                const cons_t F = muscl_flux_x(Uold, g, i, j, lam, solver);
                double* p = fx + 4 * ((size_t)(j - jb) * nx_faces + (size_t)(i - (ib - 1)));
                p[0] = F.rho; p[1] = F.rhou; p[2] = F.rhov; p[3] = F.E;
            }
    }
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
    for (int j = jb; j < je; ++j)
        for (int i = ib; i < ie; ++i) {
            const double* pm = fx + 4 * ((size_t)(j - jb) * nx_faces + (size_t)((i - 1) - (ib - 1)));
            const double* pp = fx + 4 * ((size_t)(j - jb) * nx_faces + (size_t)(i - (ib - 1)));
            const cons_t Fm = c_make(pm[0], pm[1], pm[2], pm[3]);
            const cons_t Fp = c_make(pp[0], pp[1], pp[2], pp[3]);
            st(Utmp, g, i, j, c_sub(ld(Uold, g, i, j), c_scale(dt_over_dx, c_sub(Fp, Fm))));
        }
    free(fx_own);
}

/* The y half: fill_y_face_cache (src/cpu/solver_cpu.cpp:247-279) and the y
 * update (:474-494) of Unew's interior from Utmp (ghost rows included in
 * its stencil); no ghost fill.  fy: 4*nx*(ny+1) doubles or NULL. */
void orc_sweep_y(const double* Utmp, double* Unew, const orc_grid* g, double dt, int solver, double* fy) {
    const int ib = NG, ie = NG + g->nx, jb = NG, je = NG + g->ny;
    const int nx = g->nx, ny = g->ny;
    double* fy_own = NULL;
    if (!fy) fy = fy_own = (double*)malloc(sizeof(double) * 4 * (size_t)nx * (ny + 1));
    const double dt_over_dy = dt / gdy(g);
    {
        const double lam = dt / gdy(g);
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
        for (int j = jb - 1; j < je; ++j)
            for (int i = ib; i < ie; ++i) {
                const cons_t F = muscl_flux_y(Utmp, g, i, j, lam, solver);
                double* p = fy + 4 * ((size_t)(j - (jb - 1)) * nx + (size_t)(i - ib));
                p[0] = F.rho; p[1] = F.rhou; p[2] = F.rhov; p[3] = F.E;
            }
    }
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
    for (int j = jb; j < je; ++j)
        for (int i = ib; i < ie; ++i) {
            const double* pm = fy + 4 * ((size_t)((j - 1) - (jb - 1)) * nx + (size_t)(i - ib));
            const double* pp = fy + 4 * ((size_t)(j - (jb - 1)) * nx + (size_t)(i - ib));
            const cons_t Fm = c_make(pm[0], pm[1], pm[2], pm[3]);
            const cons_t Fp = c_make(pp[0], pp[1], pp[2], pp[3]);
            st(Unew, g, i, j, c_sub(ld(Utmp, g, i, j), c_scale(dt_over_dy, c_sub(Fp, Fm))));
        }
    free(fy_own);
}

/* src/cpu/solver_cpu.cpp:400-499 (plus the BC hook at :461 and :498) */
void orc_advance_second_order(const double* Uold, double* Utmp, double* Unew,
                              const orc_grid* g, double dt, int solver,
                              double* fx, double* fy) {
    orc_sweep_x(Uold, Utmp, g, dt, solver, fx);
    orc_apply_boundary(Utmp, g);
    orc_sweep_y(Utmp, Unew, g, dt, solver, fy);
    orc_apply_boundary(Unew, g);
}

/* src/cpu/solver_cpu.cpp:315-369 */
void orc_advance_first_order(const double* Uold, double* Unew, const orc_grid* g,
                             double dt, int solver) {
    const int ib = NG, ie = NG + g->nx, jb = NG, je = NG + g->ny;
    const double dt_over_dx = dt / gdx(g);
    const double dt_over_dy = dt / gdy(g);
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
    for (int j = jb; j < je; ++j)
        for (int i = ib; i < ie; ++i) {
            const cons_t Fxp = riemann_flux(ld(Uold, g, i, j), ld(Uold, g, i + 1, j), ORC_DIR_X, solver);
            const cons_t Fxm = riemann_flux(ld(Uold, g, i - 1, j), ld(Uold, g, i, j), ORC_DIR_X, solver);
            const cons_t Fyp = riemann_flux(ld(Uold, g, i, j), ld(Uold, g, i, j + 1), ORC_DIR_Y, solver);
            const cons_t Fym = riemann_flux(ld(Uold, g, i, j - 1), ld(Uold, g, i, j), ORC_DIR_Y, solver);
            st(Unew, g, i, j,
               c_sub(c_sub(ld(Uold, g, i, j), c_scale(dt_over_dx, c_sub(Fxp, Fxm))),
                     c_scale(dt_over_dy, c_sub(Fyp, Fym))));
        }
    orc_apply_boundary(Unew, g);
}

void orc_riemann_flux(const double* UL, const double* UR, int dir, int solver, double* F) {
    const cons_t r = riemann_flux(c_make(UL[0], UL[1], UL[2], UL[3]),
                                  c_make(UR[0], UR[1], UR[2], UR[3]), dir, solver);
    F[0] = r.rho; F[1] = r.rhou; F[2] = r.rhov; F[3] = r.E;
}

/* scripts/cpu/main_cpu.cpp:206-262 */
int orc_run(double* U, const orc_grid* g, double cfl, double t_end, int solver,
            long long max_steps, int nsnap,
            double* t_out, long long* steps_out,
            double* dt_log, long long dt_cap,
            long long* snap_step, double* snap_t, double* snap_data) {
    const long long n = orc_grid_doubles(g);
    double* Umid = (double*)calloc((size_t)n, sizeof(double));
    double* Unext = (double*)calloc((size_t)n, sizeof(double));
    double* fx = (double*)malloc(sizeof(double) * 4 * (size_t)(g->nx + 1) * g->ny);
    double* fy = (double*)malloc(sizeof(double) * 4 * (size_t)g->nx * (g->ny + 1));
    double* cur = U;
    double* nxt = Unext;
    double t = 0.0;
    long long step = 0;
    int next_snapshot = 0;
    int rc = 0;
    while (t < t_end && (max_steps <= 0 || step < max_steps)) {
        orc_apply_boundary(cur, g);
        double dt = 0.0;
        if (orc_compute_dt(cur, g, cfl, &dt)) { rc = 1; break; }
        if (t + dt > t_end) dt = t_end - t;
        orc_advance_second_order(cur, Umid, nxt, g, dt, solver, fx, fy);
        double* tmp = cur; cur = nxt; nxt = tmp;
        if (dt_log && step < dt_cap) dt_log[step] = dt;
        t += dt;
        ++step;
        while (next_snapshot < nsnap &&
               t >= t_end * (double)(next_snapshot + 1) / (double)nsnap) {
            if (snap_step) snap_step[next_snapshot] = step;
            if (snap_t) snap_t[next_snapshot] = t;
            if (snap_data) memcpy(snap_data + (size_t)next_snapshot * (size_t)n, cur, sizeof(double) * (size_t)n);
            ++next_snapshot;
        }
    }
    if (cur != U) memcpy(U, cur, sizeof(double) * (size_t)n);
    if (t_out) *t_out = t;
    if (steps_out) *steps_out = step;
    free(Umid); free(Unext); free(fx); free(fy);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Initial states                                                           */
/* ------------------------------------------------------------------------ */
/* src/test_cases.cpp:11-18 */
static cons_t make_conserved(double rho, double u, double v, double p) {
    return c_make(rho, rho * u, rho * v, p / (GAMMA - 1.0) + 0.5 * rho * (u * u + v * v));
}

/* src/test_cases.cpp:24-69 with the state constants as parameters */
static cons_t shock_bubble_state(double x, double y, double rho0, double p0, double mach,
                                 double shock_x, double bcx, double bcy, double br, double rho_b) {
    const double a0 = sqrt(GAMMA * p0 / rho0);
    const double M2 = mach * mach;
    const double rho2 = rho0 * ((GAMMA + 1.0) * M2) / ((GAMMA - 1.0) * M2 + 2.0);
    const double p2 = p0 * (1.0 + 2.0 * GAMMA / (GAMMA + 1.0) * (M2 - 1.0));
    const double u2 = 2.0 * a0 / (GAMMA + 1.0) * (mach - 1.0 / mach);
    double rho = rho0, u = 0.0, v = 0.0, p = p0;
    if (x < shock_x) { rho = rho2; u = u2; v = 0.0; p = p2; }
    const double dx = x - bcx, dy = y - bcy;
    if (dx * dx + dy * dy <= br * br) rho = rho_b;
    return make_conserved(rho, u, v, p);
}

/* src/test_cases.cpp:78-101 with the state constants as parameters */
static cons_t blast_state(double x, double y, double cx, double cy, double r,
                          double rho_in, double p_in, double rho_out, double p_out) {
    const double dx = x - cx, dy = y - cy;
    const double r2 = dx * dx + dy * dy;
    if (r2 <= r * r) return make_conserved(rho_in, 0.0, 0.0, p_in);
    return make_conserved(rho_out, 0.0, 0.0, p_out);
}

/* src/init.cpp:29-38: state at every cell centre, ghosts included */
#define FOR_ALL_CELLS(g, body)                                                   \
    do {                                                                         \
        const double dx_ = gdx(g), dy_ = gdy(g);                                 \
        for (int j = 0; j < (int)tny(g); ++j)                                    \
            for (int i = 0; i < (int)tnx(g); ++i) {                              \
                const double x = (g)->x_min + ((double)(i - NG) + 0.5) * dx_;    \
                const double y = (g)->y_min + ((double)(j - NG) + 0.5) * dy_;    \
                body;                                                            \
            }                                                                    \
    } while (0)

void orc_init_blast(double* U, const orc_grid* g, double cx, double cy, double r,
                    double rho_in, double p_in, double rho_out, double p_out) {
    FOR_ALL_CELLS(g, st(U, g, i, j, blast_state(x, y, cx, cy, r, rho_in, p_in, rho_out, p_out)));
}

void orc_init_shock_bubble(double* U, const orc_grid* g, double rho0, double p0,
                           double mach, double shock_x, double bub_cx,
                           double bub_cy, double bub_r, double rho_bubble) {
    FOR_ALL_CELLS(g, st(U, g, i, j, shock_bubble_state(x, y, rho0, p0, mach, shock_x,
                                                       bub_cx, bub_cy, bub_r, rho_bubble)));
}

/* src/test_cases.cpp:24-33,78-89: case 0 = shock_bubble, 1 = blast_wave
 * (CaseId order, head/test_cases.hpp:20-23) with the reference constants. */
void orc_init_reference_case(double* U, const orc_grid* g, int case_id) {
    if (case_id == 0)
        orc_init_shock_bubble(U, g, 1.29, 1.01325e5, 1.22, 0.005, 0.035, 0.0445, 0.025, 0.214);
    else
        orc_init_blast(U, g, 0.5, 0.5, 0.1, 1.0, 100.0, 1.0, 1.0);
}
