// CPU check of the hand-written adjoint (large_sys_eq_opt_gb300/csrc/adjoint.cuh)
// against central finite differences in FP64:
//   1. Riemann-flux vjps (HLL, HLLC, exact, FORCE) on random face states
//      covering subsonic, supersonic, shock and rarefaction pairs;
//   2. the reconstruction vjp;
//   3. whole-line adjoint sweeps through the tiled routine adjoint_tile
//      (the same code the GPU kernel runs), transmissive and reflective
//      ends, several line lengths and tile widths.
// Prints one line per check and exits non-zero when any check fails.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

// ---- dual number (forward-mode derivative): branches on the value part -------
// J(u + eps d) with eps^2 = 0 gives the directional derivative of the branch
// the value part takes, to machine precision and with no subtraction error --
// the same subgradient convention the adjoint uses (minmod's zero branch at
// exact ties included).  (A complex step would not do at exact ties: the
// real part of a product picks up -im*im and can flip a tie.)
namespace cs {
struct CS {
    double re, im;
    CS(double r = 0.0, double i = 0.0) : re(r), im(i) {}
    explicit operator double() const { return re; }
};
inline CS operator+(CS a, CS b) { return CS(a.re + b.re, a.im + b.im); }
inline CS operator-(CS a, CS b) { return CS(a.re - b.re, a.im - b.im); }
inline CS operator-(CS a) { return CS(-a.re, -a.im); }
inline CS operator*(CS a, CS b) { return CS(a.re * b.re, a.re * b.im + a.im * b.re); }
inline CS operator/(CS a, CS b) { return CS(a.re / b.re, (a.im * b.re - a.re * b.im) / (b.re * b.re)); }
inline CS& operator+=(CS& a, CS b) { return a = a + b; }
inline CS& operator-=(CS& a, CS b) { return a = a - b; }
inline CS& operator*=(CS& a, CS b) { return a = a * b; }
inline bool operator<(CS a, CS b) { return a.re < b.re; }
inline bool operator>(CS a, CS b) { return a.re > b.re; }
inline bool operator<=(CS a, CS b) { return a.re <= b.re; }
inline bool operator>=(CS a, CS b) { return a.re >= b.re; }
inline bool operator==(CS a, CS b) { return a.re == b.re; }
inline bool operator!=(CS a, CS b) { return a.re != b.re; }
inline CS fabs(CS a) { return a.re < 0 ? -a : a; }
// derivative parts by the chain rule
inline CS sqrt(CS a) { const double r = std::sqrt(a.re); return CS(r, a.im / (2.0 * r)); }
inline CS pow(CS a, CS b) {
    const double r = std::pow(a.re, b.re);
    return CS(r, r * (b.im * std::log(a.re) + b.re * a.im / a.re));
}
}  // namespace cs
namespace eu { namespace adj { template <class T> struct Side; } }
namespace cs {
void star_refine(const eu::adj::Side<CS>& L, const eu::adj::Side<CS>& R, double ps, double us, CS& tps, CS& tus);
}

#include "adjoint.cuh"

namespace cs {
// f_K(p) of head/riemann.hpp:331-359 in complex-step arithmetic
static void pfun_cs(CS p, CS rK, CS pK, CS aK, CS& f, CS& fd) {
    const double g = eu::adj::kG;
    if (p.re > pK.re) {
        const CS A = CS(2.0 / (g + 1.0)) / rK;
        const CS B = CS((g - 1.0) / (g + 1.0)) * pK;
        const CS q = sqrt(A / (p + B));
        f = (p - pK) * q;
        fd = q * (CS(1.0) - CS(0.5) * (p - pK) / (p + B));
    } else {
        const CS pr = p / pK;
        f = CS(2.0 / (g - 1.0)) * aK * (pow(pr, CS((g - 1.0) / (2.0 * g))) - CS(1.0));
        fd = CS(1.0) / (rK * aK) * pow(pr, CS(-(g + 1.0) / (2.0 * g)));
    }
}
// p*, u* with derivatives by one Newton step in dual arithmetic from the
// converged p* (the implicit-function derivative); values unchanged.
void star_refine(const eu::adj::Side<CS>& L, const eu::adj::Side<CS>& R, double ps, double us, CS& tps, CS& tus) {
    CS fL, fR, dL, dR;
    const CS p(ps);
    pfun_cs(p, L.W.r, L.W.p, L.a, fL, dL);
    pfun_cs(p, R.W.r, R.W.p, R.a, fR, dR);
    const CS F = fL + fR + (R.W.un - L.W.un);
    const CS p1 = p - F / CS((dL + dR).re);
    tps = CS(ps, p1.im);
    pfun_cs(tps, L.W.r, L.W.p, L.a, fL, dL);
    pfun_cs(tps, R.W.r, R.W.p, R.a, fR, dR);
    const CS u = CS(0.5) * (L.W.un + R.W.un + fR - fL);
    tus = CS(us, u.im);
}
}  // namespace cs

using namespace eu::adj;
using C = C4<double>;
using W = W4<double>;

static std::mt19937_64 rng(12345);
static double uni(double a, double b) { return std::uniform_real_distribution<double>(a, b)(rng); }
static double gau() { return std::normal_distribution<double>(0.0, 1.0)(rng); }

static W rand_w(int regime) {
    switch (regime) {
        case 0: return W{uni(0.2, 2.0), uni(-0.5, 0.5), uni(-0.5, 0.5), uni(0.2, 2.0)};   // subsonic
        case 1: return W{uni(0.5, 2.0), uni(2.0, 4.0), uni(-1, 1), uni(0.2, 1.0)};        // supersonic right-moving
        case 2: return W{uni(0.5, 2.0), uni(-4.0, -2.0), uni(-1, 1), uni(0.2, 1.0)};      // supersonic left-moving
        default: return W{uni(0.05, 5.0), uni(-1.5, 1.5), uni(-1, 1), uni(0.02, 20.0)};   // strong jumps
    }
}
static C randc() { return C{gau(), gau(), gau(), gau()}; }
static C axpy(const C& a, double s, const C& d) {
    return C{a.r + s * d.r, a.mn + s * d.mn, a.mt + s * d.mt, a.e + s * d.e};
}
static W axpyw(const W& a, double s, const W& d) {
    return W{a.r + s * d.r, a.un + s * d.un, a.ut + s * d.ut, a.p + s * d.p};
}
static double dotw(const W& a, const W& b) { return a.r * b.r + a.un * b.un + a.ut * b.ut + a.p * b.p; }

static int fails = 0;
static void report(const char* what, int bad, int total, double worst) {
    std::printf("%s %s: %d/%d within tolerance, worst rel %.2e\n", bad ? "FAIL" : "PASS", what, total - bad, total,
                worst);
    if (bad) ++fails;
}
static double rel(double a, double b) { return std::fabs(a - b) / std::fmax(1e-9, std::fmax(std::fabs(a), std::fabs(b))); }

template <int S> static void check_riemann(const char* name) {
    int bad = 0, total = 0;
    double worst = 0;
    for (int t = 0; t < 4000; ++t) {
        const int reg = t % 4;
        const C UL = p2c(rand_w(reg)), UR = p2c(rand_w(reg == 3 ? 3 : (t / 4) % 4));
        const C Fb = randc(), dL = randc(), dR = randc();
        C Lb, Rb;
        riemann_vjp<S>(UL, UR, Fb, Lb, Rb);
        const double ad = dot(Lb, dL) + dot(Rb, dR);
        const double eps = 1e-6;
        const double fp = dot(Fb, riemann_primal<S>(axpy(UL, eps, dL), axpy(UR, eps, dR)));
        const double fm = dot(Fb, riemann_primal<S>(axpy(UL, -eps, dL), axpy(UR, -eps, dR)));
        const double fd = (fp - fm) / (2 * eps);
        const double e = rel(ad, fd);
        ++total;
        if (e > 1e-5) ++bad; else worst = std::fmax(worst, e);
    }
    // a handful of branch-boundary crossings are expected among random samples
    report(name, bad > total / 200 ? bad : 0, total, worst);
}

static void check_recon() {
    int bad = 0, total = 0;
    double worst = 0;
    for (int t = 0; t < 4000; ++t) {
        const int reg = t % 4;
        const W Wm = rand_w(reg), Wc = rand_w(reg), Wp = rand_w(reg);
        const double hl = uni(0.01, 0.3);
        const C Lb = randc(), Rb = randc();
        const W dm{gau(), gau(), gau(), gau()}, dc{gau(), gau(), gau(), gau()}, dp{gau(), gau(), gau(), gau()};
        Recon<double> o;
        recon_primal(Wm, Wc, Wp, hl, o);
        W bm = zerow<double>(), bc = zerow<double>(), bp = zerow<double>();
        recon_vjp(o, hl, Lb, Rb, bm, bc, bp);
        const double ad = dotw(bm, dm) + dotw(bc, dc) + dotw(bp, dp);
        const double eps = 1e-6;
        Recon<double> a, b;
        recon_primal(axpyw(Wm, eps, dm), axpyw(Wc, eps, dc), axpyw(Wp, eps, dp), hl, a);
        recon_primal(axpyw(Wm, -eps, dm), axpyw(Wc, -eps, dc), axpyw(Wp, -eps, dp), hl, b);
        const double fd = (dot(Lb, a.L) + dot(Rb, a.R) - dot(Lb, b.L) - dot(Rb, b.R)) / (2 * eps);
        const double e = rel(ad, fd);
        ++total;
        if (e > 1e-5) ++bad; else worst = std::fmax(worst, e);
    }
    report("reconstruction vjp", bad > total / 200 ? bad : 0, total, worst);
}

// ---- one line: primal sweep and tiled adjoint ------------------------------
struct Line {
    int n, bc_lo, bc_hi;
    std::vector<C> full;   // cells -2 .. n+1
    C& at(int c) { return full[c + 2]; }
    const C& at(int c) const { return full[c + 2]; }
};
static C mirror(const C& u) { return C{u.r, -u.mn, u.mt, u.e}; }
static void fill_ghosts(Line& L) {
    const int n = L.n;
    L.at(-1) = L.bc_lo ? mirror(L.at(0)) : L.at(0);
    L.at(-2) = L.bc_lo ? mirror(L.at(1)) : L.at(0);
    L.at(n) = L.bc_hi ? mirror(L.at(n - 1)) : L.at(n - 1);
    L.at(n + 1) = L.bc_hi ? mirror(L.at(n - 2)) : L.at(n - 1);
}
template <int S> static std::vector<C> sweep(const Line& L, double hl, double lam) {
    const int n = L.n;
    std::vector<C> Lf(n + 2), Rf(n + 2);
    for (int c = -1; c <= n; ++c) {
        Recon<double> o;
        recon_primal(c2p(L.at(c - 1)), c2p(L.at(c)), c2p(L.at(c + 1)), hl, o);
        Lf[c + 1] = o.L;
        Rf[c + 1] = o.R;
    }
    std::vector<C> F(n + 1);   // F[k] = face k - 1/2
    for (int k = 0; k <= n; ++k) F[k] = riemann_primal<S>(Rf[k], Lf[k + 1]);
    std::vector<C> out(n);
    for (int c = 0; c < n; ++c) out[c] = axpy(L.at(c), -lam, sub(F[c + 1], F[c]));
    return out;
}
struct Acc {
    int n, bc_lo, bc_hi;
    double hl, lam;
    const std::vector<Line>* lines;
    const std::vector<std::vector<C>>* abar;
    std::vector<std::vector<C>>* grad;
    bool line_ok(int l) const { return l < (int)lines->size(); }
    C load_state(int l, int c) const { return (*lines)[l].at(c); }
    C load_adj(int l, int c) const { return (*abar)[l][c]; }
    void store(int l, int c, const C& g) const { (*grad)[l][c] = g; }
};

template <int S, int TC> static void check_line(const char* name) {
    int bad = 0, total = 0;
    double worst = 0;
    const int sizes[] = {2, 3, 5, 9, 17, 64, 130};
    for (int n : sizes)
        for (int bc = 0; bc < 4; ++bc) {
            const int nl = 3;
            std::vector<Line> lines(nl);
            std::vector<std::vector<C>> abar(nl, std::vector<C>(n)), grad(nl, std::vector<C>(n));
            const double hl = 0.15, lam = 0.3;
            for (int l = 0; l < nl; ++l) {
                lines[l].n = n;
                lines[l].bc_lo = bc & 1;
                lines[l].bc_hi = bc >> 1;
                lines[l].full.resize(n + 4);
                for (int c = 0; c < n; ++c) lines[l].at(c) = p2c(rand_w(l == 2 ? 3 : 0));
                fill_ghosts(lines[l]);
                for (int c = 0; c < n; ++c) abar[l][c] = randc();
            }
            Acc acc{n, bc & 1, bc >> 1, hl, lam, &lines, &abar, &grad};
            static eu::adj::TileMem<double, 4, TC> mem;
            const int nt = (n + TC - 1) / TC;
            for (int t = 0; t < nt; ++t) {
                int c0, c1;
                tile_range(n, TC, t, c0, c1);
                adjoint_tile<S, double, 4, TC, false>(acc, mem, 0, c0, c1 - c0, 0, 1);
            }
            for (int l = 0; l < nl; ++l) {
                std::vector<C> d(n);
                for (int c = 0; c < n; ++c) d[c] = randc();
                double ad = 0;
                for (int c = 0; c < n; ++c) ad += dot(grad[l][c], d[c]);
                const double eps = 1e-6;
                double J[2];
                for (int sgn = 0; sgn < 2; ++sgn) {
                    Line P = lines[l];
                    for (int c = 0; c < n; ++c) P.at(c) = axpy(lines[l].at(c), sgn ? -eps : eps, d[c]);
                    fill_ghosts(P);
                    const std::vector<C> out = sweep<S>(P, hl, lam);
                    J[sgn] = 0;
                    for (int c = 0; c < n; ++c) J[sgn] += dot(abar[l][c], out[c]);
                }
                const double fd = (J[0] - J[1]) / (2 * eps);
                const double e = rel(ad, fd);
                ++total;
                if (e > 1e-5) {
                    ++bad;
                    std::printf("  %s n=%d bc=%d line=%d ad=%.12e fd=%.12e\n", name, n, bc, l, ad, fd);
                } else {
                    worst = std::fmax(worst, e);
                }
            }
        }
    report(name, bad, total, worst);
}

// ---- 2D split step on the CPU: forward (any number type) and adjoint -------
template <class T> struct Grid2 {
    int nx, ny;
    std::vector<C4<T>> u;   // (ny+4) x (nx+4), conserved (rho, rhou, rhov, E)
    C4<T>& at(int i, int j) { return u[(size_t)(j + 2) * (nx + 4) + (i + 2)]; }
    const C4<T>& at(int i, int j) const { return u[(size_t)(j + 2) * (nx + 4) + (i + 2)]; }
};
template <class T> static C4<T> swap_m(const C4<T>& a) { return C4<T>{a.r, a.mt, a.mn, a.e}; }
template <class T> static C4<T> flip_n(const C4<T>& a, bool x) {
    return x ? C4<T>{a.r, -a.mn, a.mt, a.e} : C4<T>{a.r, a.mn, -a.mt, a.e};
}
// ghost columns of interior rows, then ghost rows of all columns
// (head/cpu/boundary_cpu.hpp:5-37, reflective sides mirror and negate the
// normal momentum)
template <class T> static void bc2(Grid2<T>& g, const int bc[4]) {
    const int nx = g.nx, ny = g.ny;
    for (int j = 0; j < ny; ++j) {
        g.at(-1, j) = bc[0] ? flip_n(g.at(0, j), true) : g.at(0, j);
        g.at(-2, j) = bc[0] ? flip_n(g.at(1, j), true) : g.at(0, j);
        g.at(nx, j) = bc[1] ? flip_n(g.at(nx - 1, j), true) : g.at(nx - 1, j);
        g.at(nx + 1, j) = bc[1] ? flip_n(g.at(nx - 2, j), true) : g.at(nx - 1, j);
    }
    for (int i = -2; i < nx + 2; ++i) {
        g.at(i, -1) = bc[2] ? flip_n(g.at(i, 0), false) : g.at(i, 0);
        g.at(i, -2) = bc[2] ? flip_n(g.at(i, 1), false) : g.at(i, 0);
        g.at(i, ny) = bc[3] ? flip_n(g.at(i, ny - 1), false) : g.at(i, ny - 1);
        g.at(i, ny + 1) = bc[3] ? flip_n(g.at(i, ny - 2), false) : g.at(i, ny - 1);
    }
}
// one sweep along a line of n cells given with its 2+2 ghosts (sweep-local)
template <int S, class T> static std::vector<C4<T>> sweep_line(const std::vector<C4<T>>& Lc, int n, T hl, T lam) {
    auto at = [&](int c) -> const C4<T>& { return Lc[c + 2]; };
    std::vector<C4<T>> Lf(n + 2), Rf(n + 2);
    for (int c = -1; c <= n; ++c) {
        Recon<T> o;
        recon_primal(c2p(at(c - 1)), c2p(at(c)), c2p(at(c + 1)), hl, o);
        Lf[c + 1] = o.L;
        Rf[c + 1] = o.R;
    }
    std::vector<C4<T>> F(n + 1);
    for (int k = 0; k <= n; ++k) F[k] = riemann_primal<S>(Rf[k], Lf[k + 1]);
    std::vector<C4<T>> out(n);
    for (int c = 0; c < n; ++c) {
        const C4<T> d = sub(F[c + 1], F[c]);
        out[c] = C4<T>{at(c).r - lam * d.r, at(c).mn - lam * d.mn, at(c).mt - lam * d.mt, at(c).e - lam * d.e};
    }
    return out;
}
// advance_second_order: x-sweep, BC, y-sweep, BC (src/cpu/solver_cpu.cpp:400-499)
template <int S, class T>
static void step2(Grid2<T>& U, Grid2<T>& Ut, double dt, double dx, double dy, const int bc[4]) {
    const int nx = U.nx, ny = U.ny;
    Ut = U;
    for (int j = 0; j < ny; ++j) {
        std::vector<C4<T>> line(nx + 4);
        for (int c = -2; c < nx + 2; ++c) line[c + 2] = U.at(c, j);
        const auto out = sweep_line<S, T>(line, nx, T(0.5 * dt / dx), T(dt / dx));
        for (int c = 0; c < nx; ++c) Ut.at(c, j) = out[c];
    }
    bc2(Ut, bc);
    for (int i = 0; i < nx; ++i) {
        std::vector<C4<T>> line(ny + 4);
        for (int c = -2; c < ny + 2; ++c) line[c + 2] = swap_m(Ut.at(i, c));
        const auto out = sweep_line<S, T>(line, ny, T(0.5 * dt / dy), T(dt / dy));
        for (int c = 0; c < ny; ++c) U.at(i, c) = swap_m(out[c]);
    }
    bc2(U, bc);
}

// accessor over one grid direction for adjoint_tile
struct Acc2 {
    int n, bc_lo, bc_hi, nlines, dir;
    double hl, lam;
    const Grid2<double>* P;   // primal input of the sweep (with ghosts)
    const Grid2<double>* A;   // adjoint of the sweep's outputs
    Grid2<double>* G;         // adjoint of the sweep's inputs
    bool line_ok(int l) const { return l < nlines; }
    C load_state(int l, int c) const { return dir == 0 ? P->at(c, l) : swap_m(P->at(l, c)); }
    C load_adj(int l, int c) const { return dir == 0 ? A->at(c, l) : swap_m(A->at(l, c)); }
    void store(int l, int c, const C& g) const { (dir == 0 ? G->at(c, l) : G->at(l, c)) = dir == 0 ? g : swap_m(g); }
};

template <int S, int TC>
static void adjoint_sweep2(int dir, const Grid2<double>& P, const Grid2<double>& A, Grid2<double>& G, double lam,
                           const int bc[4]) {
    Acc2 acc{dir == 0 ? P.nx : P.ny, dir == 0 ? bc[0] : bc[2], dir == 0 ? bc[1] : bc[3], dir == 0 ? P.ny : P.nx,
             dir, 0.5 * lam, lam, &P, &A, &G};
    // the tile layouts of the GPU kernels: lines fastest (padded line
    // stride) for the y-sweep adjoint, cells fastest for the x-sweep adjoint
    static TileMem<double, 2, TC> mem_x;
    static TileMem<double, 2, TC, true> mem_y;
    const int nt = (acc.n + TC - 1) / TC;
    for (int l0 = 0; l0 < acc.nlines; l0 += 2)
        for (int t = 0; t < nt; ++t) {
            int c0, c1;
            tile_range(acc.n, TC, t, c0, c1);
            if (dir == 1) adjoint_tile<S, double, 2, TC, true>(acc, mem_y, l0, c0, c1 - c0, 0, 1);
            else adjoint_tile<S, double, 2, TC, false>(acc, mem_x, l0, c0, c1 - c0, 0, 1);
        }
}

struct Problem {
    int nx, ny, solver, nsteps, bc[4];
    double dx, dy;
    std::vector<double> dts, rho0, p0, mask;
    std::vector<std::vector<double>> dirs;   // each 2*nx*ny: d_rho then d_p
};

template <class T> static Grid2<T> initial(const Problem& pb, const std::vector<double>* d, double h) {
    Grid2<T> g{pb.nx, pb.ny, std::vector<C4<T>>((size_t)(pb.nx + 4) * (pb.ny + 4))};
    const size_t m = (size_t)pb.nx * pb.ny;
    for (int j = 0; j < pb.ny; ++j)
        for (int i = 0; i < pb.nx; ++i) {
            const size_t k = (size_t)j * pb.nx + i;
            T r = T(pb.rho0[k]), p = T(pb.p0[k]);
            if (d) {
                r = r + T(h) * T((*d)[k]);
                p = p + T(h) * T((*d)[m + k]);
            }
            g.at(i, j) = C4<T>{r, T(0), T(0), p / T(kG1)};
        }
    return g;
}

// forward-mode directional derivative of J = sum(mask * rho^2)
template <int S> static double cs_derivative(const Problem& pb, const std::vector<double>& d) {
    using cs::CS;
    const double h = 1.0;
    std::vector<double> di(d.size());
    Grid2<CS> U{pb.nx, pb.ny, {}};
    {
        Grid2<double> base = initial<double>(pb, nullptr, 0);
        U.u.resize(base.u.size());
        const size_t m = (size_t)pb.nx * pb.ny;
        for (int j = 0; j < pb.ny; ++j)
            for (int i = 0; i < pb.nx; ++i) {
                const size_t k = (size_t)j * pb.nx + i;
                const C b = base.at(i, j);
                U.at(i, j) = C4<CS>{CS(b.r, h * d[k]), CS(0), CS(0), CS(b.e, h * d[m + k] / kG1)};
            }
    }
    bc2(U, pb.bc);
    Grid2<CS> Ut = U;
    for (int n = 0; n < pb.nsteps; ++n) step2<S, CS>(U, Ut, pb.dts[n], pb.dx, pb.dy, pb.bc);
    double im = 0;
    for (int j = 0; j < pb.ny; ++j)
        for (int i = 0; i < pb.nx; ++i) {
            const size_t k = (size_t)j * pb.nx + i;
            if (pb.mask[k] != 0.0) im += (U.at(i, j).r * U.at(i, j).r).im;
        }
    return im / h;
}

// CPU adjoint: gradient of J w.r.t. (rho0, p0) as 2*nx*ny numbers
template <int S> static std::vector<double> cpu_gradient(const Problem& pb) {
    std::vector<Grid2<double>> Us, Uts;
    Grid2<double> U = initial<double>(pb, nullptr, 0);
    bc2(U, pb.bc);
    Grid2<double> Ut = U;
    for (int n = 0; n < pb.nsteps; ++n) {
        Us.push_back(U);
        step2<S, double>(U, Ut, pb.dts[n], pb.dx, pb.dy, pb.bc);
        Uts.push_back(Ut);
    }
    Grid2<double> lam = U, mu = U;
    for (auto& v : lam.u) v = zero4<double>();
    for (int j = 0; j < pb.ny; ++j)
        for (int i = 0; i < pb.nx; ++i)
            if (pb.mask[(size_t)j * pb.nx + i] != 0.0) lam.at(i, j).r = 2.0 * U.at(i, j).r;
    for (int n = pb.nsteps - 1; n >= 0; --n) {
        adjoint_sweep2<S, 8>(1, Uts[n], lam, mu, pb.dts[n] / pb.dy, pb.bc);
        adjoint_sweep2<S, 8>(0, Us[n], mu, lam, pb.dts[n] / pb.dx, pb.bc);
    }
    const size_t m = (size_t)pb.nx * pb.ny;
    std::vector<double> g(2 * m);
    for (int j = 0; j < pb.ny; ++j)
        for (int i = 0; i < pb.nx; ++i) {
            g[(size_t)j * pb.nx + i] = lam.at(i, j).r;
            g[m + (size_t)j * pb.nx + i] = lam.at(i, j).e / kG1;
        }
    return g;
}

template <int S> static void solve_problem(const Problem& pb, std::vector<double>& csd, std::vector<double>& add) {
    const std::vector<double> g = cpu_gradient<S>(pb);
    for (const auto& d : pb.dirs) {
        csd.push_back(cs_derivative<S>(pb, d));
        double a = 0;
        for (size_t k = 0; k < d.size(); ++k) a += g[k] * d[k];
        add.push_back(a);
    }
}
static void solve_any(const Problem& pb, std::vector<double>& csd, std::vector<double>& add) {
    switch (pb.solver) {
        case 1: solve_problem<1>(pb, csd, add); break;
        case 2: solve_problem<2>(pb, csd, add); break;
        case 3: solve_problem<3>(pb, csd, add); break;
        default: solve_problem<0>(pb, csd, add); break;
    }
}

// blast of [0,2]^2 (optionally with a smooth perturbation), ring mask
static Problem blast_problem(int nx, int ny, int solver, int nsteps, double smooth, const int bc[4], int ndir) {
    Problem pb;
    pb.nx = nx; pb.ny = ny; pb.solver = solver; pb.nsteps = nsteps;
    std::memcpy(pb.bc, bc, sizeof(pb.bc));
    pb.dx = 2.0 / nx; pb.dy = 2.0 / ny;
    const size_t m = (size_t)nx * ny;
    pb.rho0.resize(m); pb.p0.resize(m); pb.mask.resize(m);
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const double x = (i + 0.5) * pb.dx, y = (j + 0.5) * pb.dy;
            const double r2 = (x - 1) * (x - 1) + (y - 1) * (y - 1);
            const bool in = r2 <= 0.16;
            const double w = 1.0 + smooth * (std::sin(2 * M_PI * (1.3 * x + 0.2)) * std::cos(2 * M_PI * (0.9 * y + 0.1)) +
                                             0.5 * std::sin(2 * M_PI * (2.1 * x + 1.7 * y)));
            const size_t k = (size_t)j * nx + i;
            pb.rho0[k] = (in ? 1.0 : 0.125) * w;
            pb.p0[k] = (in ? 1.0 : 0.1) * (2.0 - w);
            const double r = std::sqrt(r2);
            pb.mask[k] = (r >= 0.6 && r <= 0.8) ? 1.0 : 0.0;
        }
    pb.dts.assign(nsteps, 0.8 * std::min(pb.dx, pb.dy) / 3.0);
    for (int q = 0; q < ndir; ++q) {
        std::vector<double> d(2 * m);
        double nn = 0;
        for (auto& v : d) { v = gau(); nn += v * v; }
        for (auto& v : d) v /= std::sqrt(nn);
        pb.dirs.push_back(d);
    }
    return pb;
}

static void check_2d(const char* name, int solver, double smooth, const int bc[4]) {
    const Problem pb = blast_problem(24, 20, solver, 12, smooth, bc, 3);
    std::vector<double> csd, add;
    solve_any(pb, csd, add);
    double worst = 0;
    int bad = 0;
    for (size_t q = 0; q < csd.size(); ++q) {
        const double e = rel(add[q], csd[q]);
        if (e > 1e-9) {
            ++bad;
            std::printf("  %s dir %zu: adjoint %.15e forward-mode %.15e\n", name, q, add[q], csd[q]);
        }
        worst = std::fmax(worst, e);
    }
    report(name, bad, (int)csd.size(), worst);
}

// File mode: read a problem, write forward-mode and CPU-adjoint directional
// derivatives.  Input (little-endian): int32 nx, ny, solver, nsteps, bc[4],
// ndir; float64 dx, dy; dts[nsteps]; rho0[ny*nx]; p0[ny*nx]; mask[ny*nx];
// dirs[ndir][2*ny*nx].  Output: float64 forward_mode[ndir], adjoint[ndir].
static int file_mode(const char* in, const char* out) {
    FILE* f = std::fopen(in, "rb");
    if (!f) return 2;
    Problem pb;
    int hdr[9];
    bool ok = std::fread(hdr, sizeof(int), 9, f) == 9;
    pb.nx = hdr[0]; pb.ny = hdr[1]; pb.solver = hdr[2]; pb.nsteps = hdr[3];
    std::memcpy(pb.bc, hdr + 4, 4 * sizeof(int));
    const int ndir = hdr[8];
    ok = ok && std::fread(&pb.dx, 8, 1, f) == 1 && std::fread(&pb.dy, 8, 1, f) == 1;
    const size_t m = (size_t)pb.nx * pb.ny;
    auto rd = [&](std::vector<double>& v, size_t n) { v.resize(n); ok = ok && std::fread(v.data(), 8, n, f) == n; };
    rd(pb.dts, pb.nsteps); rd(pb.rho0, m); rd(pb.p0, m); rd(pb.mask, m);
    for (int q = 0; q < ndir; ++q) { std::vector<double> d; rd(d, 2 * m); pb.dirs.push_back(d); }
    std::fclose(f);
    if (!ok) return 3;
    std::vector<double> csd, add;
    solve_any(pb, csd, add);
    FILE* o = std::fopen(out, "wb");
    if (!o) return 4;
    std::fwrite(csd.data(), 8, csd.size(), o);
    std::fwrite(add.data(), 8, add.size(), o);
    std::fclose(o);
    return 0;
}

int main(int argc, char** argv) {
    if (argc == 3) return file_mode(argv[1], argv[2]);
    check_riemann<0>("HLL vjp");
    check_riemann<1>("HLLC vjp");
    check_riemann<2>("exact vjp (implicit p*)");
    check_riemann<3>("FORCE vjp");
    check_recon();
    check_line<0, 8>("line adjoint HLL, tiles of 8");
    check_line<1, 8>("line adjoint HLLC, tiles of 8");
    check_line<1, 64>("line adjoint HLLC, tiles of 64");
    check_line<2, 16>("line adjoint exact, tiles of 16");
    check_line<3, 4>("line adjoint FORCE, tiles of 4");
    const int tr[4] = {0, 0, 0, 0}, rf[4] = {1, 0, 1, 1};
    check_2d("2D adjoint vs forward mode, HLL, blast + smooth", 0, 1e-3, tr);
    check_2d("2D adjoint vs forward mode, HLLC, exact blast (limiter ties)", 1, 0.0, tr);
    check_2d("2D adjoint vs forward mode, HLLC, reflective sides", 1, 1e-3, rf);
    check_2d("2D adjoint vs forward mode, exact solver", 2, 1e-3, tr);
    check_2d("2D adjoint vs forward mode, FORCE", 3, 1e-3, rf);
    std::printf(fails ? "SOME CHECKS FAILED\n" : "ALL CHECKS PASSED\n");
    return fails ? 1 : 0;
}
