// adjoint.cuh -- discrete adjoint of one MUSCL-Hancock sweep, host/device.
//
// The forward sweep along a line of cells (sweep-local conserved states
// U = (rho, m_n, m_t, E)) is
//   W_c = cons_to_prim(U_c)                                   head/physics.hpp:13-20
//   (L*_c, R*_c) = reconstruct(W_{c-1}, W_c, W_{c+1})         src/cpu/solver_cpu.cpp:68-99
//   F_{c+1/2} = riemann(R*_c, L*_{c+1})                       head/riemann.hpp:87-672
//   U'_c = U_c - (dt/d) (F_{c+1/2} - F_{c-1/2})               src/cpu/solver_cpu.cpp:440-455
// Its adjoint, for output adjoints a_c (zero outside the interior):
//   Fbar_{c+1/2} = (dt/d) (a_{c+1} - a_c)
//   (Rbar*_c, Lbar*_{c+1}) = J_riemann^T Fbar_{c+1/2}
//   (Wbar_{c-1}, Wbar_c, Wbar_{c+1}) += J_reconstruct^T (Lbar*_c, Rbar*_c)
//   Ubar_c = a_c + J_cons_to_prim^T Wbar_c
// with the boundary rule's transpose folding ghost-cell adjoints back onto
// the interior cells they were copied from.
//
// Every vector-Jacobian product (vjp) below recomputes its primal
// intermediates with the branch structure of the forward solver (the
// physicality fallbacks of src/cpu/solver_cpu.cpp:39-99, the upwind cases and
// HLL/central fallbacks of head/riemann.hpp), so each branch decision is
// recomputed identically and differentiated as taken.  Derivatives:
//   minmod      subgradient: 1 for the selected argument, 0 when the
//               arguments' product is not positive
//   min / max   the selected argument (fmin/fmax ties: the first)
//   |x|         sign(x)
//   exact p*    implicit differentiation of f(p*) = f_L + f_R + du = 0 at the
//               converged p*: dp* = -(df/dtheta)/(df/dp*) dtheta
//               (head/riemann.hpp:331-359,379-443)
// The time step is a frozen constant (no derivative through the CFL rule).
//
// The header is plain C++ when not compiled by nvcc, so the vjps can be
// checked against finite differences on a CPU.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define EUA_HD __host__ __device__ __forceinline__
#define EUA_HD_NOINLINE static __host__ __device__ __noinline__
#else
#define EUA_HD inline
#define EUA_HD_NOINLINE static inline
#endif

namespace eu {
namespace adj {

constexpr double kG = 1.4;
constexpr double kG1 = kG - 1.0;
constexpr double kFloor = 1.0e-12;

template <class T> struct C4 { T r, mn, mt, e; };   // conserved, sweep-local
template <class T> struct W4 { T r, un, ut, p; };   // primitive, sweep-local

template <class T> EUA_HD T sq(T x) { return x * x; }
// On the device the FP64 tests below run on the integer pipes (bit
// patterns; the FP64 pipe is this part's narrowest), with the results of the
// comparisons they replace.
template <class T> EUA_HD bool fin(T x) {
#if defined(__CUDA_ARCH__)
    if constexpr (sizeof(T) == 8) return (__double2hiint(x) & 0x7ff00000) != 0x7ff00000;
#endif
    return fabs(x) < T(INFINITY);
}
// floor < x < inf for a finite floor >= 0
template <class T> EUA_HD bool in_range(T x, T floor) {
#if defined(__CUDA_ARCH__)
    if constexpr (sizeof(T) == 8) {
        const long long i = __double_as_longlong(x);
        return i > __double_as_longlong(floor) && i < 0x7ff0000000000000ll;
    }
#endif
    return x > floor && x < T(INFINITY);
}
template <class T> EUA_HD T tsqrt(T x) { return sqrt(x); }
template <class T> EUA_HD T tpow(T a, T b) { return pow(a, b); }

template <class T> EUA_HD C4<T> zero4() { return C4<T>{T(0), T(0), T(0), T(0)}; }
template <class T> EUA_HD W4<T> zerow() { return W4<T>{T(0), T(0), T(0), T(0)}; }
template <class T> EUA_HD void add(C4<T>& a, const C4<T>& b) { a.r += b.r; a.mn += b.mn; a.mt += b.mt; a.e += b.e; }
template <class T> EUA_HD void add(W4<T>& a, const W4<T>& b) { a.r += b.r; a.un += b.un; a.ut += b.ut; a.p += b.p; }
template <class T> EUA_HD C4<T> scale(const C4<T>& a, T s) { return C4<T>{a.r * s, a.mn * s, a.mt * s, a.e * s}; }
template <class T> EUA_HD T dot(const C4<T>& a, const C4<T>& b) { return a.r * b.r + a.mn * b.mn + a.mt * b.mt + a.e * b.e; }
template <class T> EUA_HD C4<T> sub(const C4<T>& a, const C4<T>& b) { return C4<T>{a.r - b.r, a.mn - b.mn, a.mt - b.mt, a.e - b.e}; }

// ---------------------------------------------------------------------------
// primal building blocks
// ---------------------------------------------------------------------------
template <class T> EUA_HD W4<T> c2p(const C4<T>& U) {
    W4<T> W;
    const T ir = T(1) / U.r;
    W.r = U.r;
    W.un = U.mn * ir;
    W.ut = U.mt * ir;
    W.p = T(kG1) * (U.e - T(0.5) * U.r * (W.un * W.un + W.ut * W.ut));
    return W;
}
template <class T> EUA_HD C4<T> p2c(const W4<T>& W) {
    return C4<T>{W.r, W.r * W.un, W.r * W.ut, W.p / T(kG1) + T(0.5) * W.r * (W.un * W.un + W.ut * W.ut)};
}
// normal flux of a state given by its conserved and primitive forms
template <class T> EUA_HD C4<T> flux(const C4<T>& U, const W4<T>& W) {
    return C4<T>{U.mn, U.mn * W.un + W.p, U.mt * W.un, (U.e + W.p) * W.un};
}
template <class T> EUA_HD T sound(const W4<T>& W) { return tsqrt(T(kG) * W.p / W.r); }
// head/riemann.hpp:74-81
template <class T> EUA_HD bool phys_riemann(const W4<T>& W) {
    return fin(W.un) && fin(W.ut) && in_range(W.r, T(0)) && in_range(W.p, T(0));
}
// src/cpu/solver_cpu.cpp:39-43
template <class T> EUA_HD bool phys_recon(const W4<T>& W) {
    return fin(W.un) && fin(W.ut) && in_range(W.r, T(kFloor)) && in_range(W.p, T(kFloor));
}
template <class T> EUA_HD C4<T> avg(const C4<T>& a, const C4<T>& b) {
    return C4<T>{T(0.5) * (a.r + b.r), T(0.5) * (a.mn + b.mn), T(0.5) * (a.mt + b.mt), T(0.5) * (a.e + b.e)};
}

// ---------------------------------------------------------------------------
// reverse building blocks (all accumulate into the bar arguments)
// ---------------------------------------------------------------------------
// W = c2p(U): Ubar += J^T Wbar (J depends on W only)
template <class T> EUA_HD void c2p_vjp(const W4<T>& W, const W4<T>& Wb, C4<T>& Ub) {
    const T ir = T(1) / W.r;
    Ub.e += T(kG1) * Wb.p;
    Ub.mn += Wb.un * ir - T(kG1) * W.un * Wb.p;
    Ub.mt += Wb.ut * ir - T(kG1) * W.ut * Wb.p;
    Ub.r += Wb.r - (Wb.un * W.un + Wb.ut * W.ut) * ir + T(0.5 * kG1) * (W.un * W.un + W.ut * W.ut) * Wb.p;
}
// U = p2c(W): Wbar += J^T Ubar
template <class T> EUA_HD void p2c_vjp(const W4<T>& W, const C4<T>& Ub, W4<T>& Wb) {
    Wb.r += Ub.r + W.un * Ub.mn + W.ut * Ub.mt + T(0.5) * (W.un * W.un + W.ut * W.ut) * Ub.e;
    Wb.un += W.r * Ub.mn + W.r * W.un * Ub.e;
    Wb.ut += W.r * Ub.mt + W.r * W.ut * Ub.e;
    Wb.p += Ub.e / T(kG1);
}
// F = flux(U, W) with U and W independent inputs
template <class T>
EUA_HD void flux_vjp(const C4<T>& U, const W4<T>& W, const C4<T>& Fb, C4<T>& Ub, W4<T>& Wb) {
    Ub.mn += Fb.r + Fb.mn * W.un;
    Ub.mt += Fb.mt * W.un;
    Ub.e += Fb.e * W.un;
    Wb.un += Fb.mn * U.mn + Fb.mt * U.mt + Fb.e * (U.e + W.p);
    Wb.p += Fb.mn + Fb.e * W.un;
}
// a = sqrt(gamma p / rho)
template <class T> EUA_HD void sound_vjp(const W4<T>& W, T a, T ab, W4<T>& Wb) {
    Wb.p += ab * a / (T(2) * W.p);
    Wb.r -= ab * a / (T(2) * W.r);
}

// ---------------------------------------------------------------------------
// reconstruction (src/cpu/solver_cpu.cpp:22-99)
// ---------------------------------------------------------------------------
// minmod with the index of the selected argument: 0 none, 1 a, 2 b
// (On the device in FP64: equal signs, both non-zero and neither NaN, in
// place of a * b > 0 -- the same except for same-sign pairs whose product
// underflows, below 1e-308, where it agrees with the forward sweeps.)
template <class T> EUA_HD T minmod_sel(T a, T b, int& sel) {
#if defined(__CUDA_ARCH__)
    if constexpr (sizeof(T) == 8) {
        const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
        const long long ma = ia & 0x7fffffffffffffffll, mb = ib & 0x7fffffffffffffffll;
        const long long inf = 0x7ff0000000000000ll;
        if (!((ia ^ ib) >= 0 && ma != 0 && mb != 0 && ma <= inf && mb <= inf)) { sel = 0; return T(0); }
        if (ma <= mb) { sel = 1; return a; }
        sel = 2;
        return b;
    }
#endif
    if (!(a * b > T(0))) { sel = 0; return T(0); }
    if (fabs(a) <= fabs(b)) { sel = 1; return a; }
    sel = 2;
    return b;
}

template <class T> struct Recon {
    W4<T> WL, WR;           // face primitives before the half step (after the guard)
    C4<T> UL, UR, FL, FR;   // their conserved states and fluxes
    C4<T> L, R;             // evolved face states (outputs)
    int sel[4];
    bool physL, physR, okL, okR;
};

template <class T>
EUA_HD void recon_primal(const W4<T>& Wm, const W4<T>& Wc, const W4<T>& Wp, T hl, Recon<T>& o) {
    W4<T> s;
    s.r = minmod_sel(Wc.r - Wm.r, Wp.r - Wc.r, o.sel[0]);
    s.un = minmod_sel(Wc.un - Wm.un, Wp.un - Wc.un, o.sel[1]);
    s.ut = minmod_sel(Wc.ut - Wm.ut, Wp.ut - Wc.ut, o.sel[2]);
    s.p = minmod_sel(Wc.p - Wm.p, Wp.p - Wc.p, o.sel[3]);
    o.WL = W4<T>{Wc.r - T(0.5) * s.r, Wc.un - T(0.5) * s.un, Wc.ut - T(0.5) * s.ut, Wc.p - T(0.5) * s.p};
    o.WR = W4<T>{Wc.r + T(0.5) * s.r, Wc.un + T(0.5) * s.un, Wc.ut + T(0.5) * s.ut, Wc.p + T(0.5) * s.p};
    o.physL = phys_recon(o.WL);
    o.physR = phys_recon(o.WR);
    if (!o.physL) o.WL = Wc;
    if (!o.physR) o.WR = Wc;
    o.UL = p2c(o.WL);
    o.UR = p2c(o.WR);
    o.FL = flux(o.UL, o.WL);
    o.FR = flux(o.UR, o.WR);
    const C4<T> h = scale(sub(o.FR, o.FL), hl);
    const C4<T> cl = sub(o.UL, h), cr = sub(o.UR, h);
    o.okL = phys_recon(c2p(cl));
    o.okR = phys_recon(c2p(cr));
    o.L = o.okL ? cl : o.UL;
    o.R = o.okR ? cr : o.UR;
}

// flux of a face state given by its primitives: F(W) = flux(p2c(W), W)
template <class T> EUA_HD void fluxw_vjp(const W4<T>& W, const C4<T>& U, const C4<T>& Fb, W4<T>& Wb) {
    C4<T> Ub = zero4<T>();
    flux_vjp(U, W, Fb, Ub, Wb);
    p2c_vjp(W, Ub, Wb);
}

// Given Lbar, Rbar (adjoints of the evolved face states), accumulate the
// adjoints of the three primitive inputs.
template <class T>
EUA_HD void recon_vjp(const Recon<T>& o, T hl, const C4<T>& Lb, const C4<T>& Rb, W4<T>& Wmb, W4<T>& Wcb,
                      W4<T>& Wpb) {
    C4<T> ULb = Lb, URb = Rb, FLb = zero4<T>(), FRb = zero4<T>();
    if (o.okL) { add(FLb, scale(Lb, hl)); add(FRb, scale(Lb, -hl)); }
    if (o.okR) { add(FLb, scale(Rb, hl)); add(FRb, scale(Rb, -hl)); }
    W4<T> WLb = zerow<T>(), WRb = zerow<T>();
    p2c_vjp(o.WL, ULb, WLb);
    p2c_vjp(o.WR, URb, WRb);
    fluxw_vjp(o.WL, o.UL, FLb, WLb);
    fluxw_vjp(o.WR, o.UR, FRb, WRb);
    // WL = Wc - s/2 (or Wc), WR = Wc + s/2 (or Wc)
    add(Wcb, WLb);
    add(Wcb, WRb);
    W4<T> sb = zerow<T>();
    if (o.physL) { sb.r -= T(0.5) * WLb.r; sb.un -= T(0.5) * WLb.un; sb.ut -= T(0.5) * WLb.ut; sb.p -= T(0.5) * WLb.p; }
    if (o.physR) { sb.r += T(0.5) * WRb.r; sb.un += T(0.5) * WRb.un; sb.ut += T(0.5) * WRb.ut; sb.p += T(0.5) * WRb.p; }
    const T s[4] = {sb.r, sb.un, sb.ut, sb.p};
    T* m[4] = {&Wmb.r, &Wmb.un, &Wmb.ut, &Wmb.p};
    T* c[4] = {&Wcb.r, &Wcb.un, &Wcb.ut, &Wcb.p};
    T* p[4] = {&Wpb.r, &Wpb.un, &Wpb.ut, &Wpb.p};
    for (int q = 0; q < 4; ++q) {
        if (o.sel[q] == 1) { *c[q] += s[q]; *m[q] -= s[q]; }
        else if (o.sel[q] == 2) { *p[q] += s[q]; *c[q] -= s[q]; }
    }
}

// ---------------------------------------------------------------------------
// Riemann solvers: primal flux and its vjp w.r.t. the two conserved inputs
// ---------------------------------------------------------------------------
// Side data shared by the solvers.
template <class T> struct Side {
    C4<T> U;
    W4<T> W;
    C4<T> F;
    T a;
    bool phys;
};
template <class T> EUA_HD Side<T> side_of(const C4<T>& U) {
    Side<T> s;
    s.U = U;
    s.W = c2p(U);
    s.F = flux(U, s.W);
    s.phys = phys_riemann(s.W);
    s.a = s.phys ? sound(s.W) : T(0);
    return s;
}
// Adjoint accumulators of one side: direct conserved part + primitive part.
template <class T> struct SideBar {
    C4<T> U;
    W4<T> W;
    T a;
};
template <class T> EUA_HD SideBar<T> zero_side() { return SideBar<T>{zero4<T>(), zerow<T>(), T(0)}; }
// Fbar of the side's physical flux
template <class T> EUA_HD void side_flux_vjp(const Side<T>& s, const C4<T>& Fb, SideBar<T>& b) {
    flux_vjp(s.U, s.W, Fb, b.U, b.W);
}
// Collapse a side's accumulators into the conserved input adjoint.
template <class T> EUA_HD C4<T> side_close(const Side<T>& s, SideBar<T> b) {
    if (b.a != T(0)) sound_vjp(s.W, s.a, b.a, b.W);
    C4<T> Ub = b.U;
    c2p_vjp(s.W, b.W, Ub);
    return Ub;
}

// Davis wave speeds with the selected arguments (head/riemann.hpp:97-98)
template <class T> struct Speeds {
    T SL, SR;
    bool selLleft, selRleft;
};
template <class T> EUA_HD Speeds<T> speeds(const Side<T>& L, const Side<T>& R) {
    Speeds<T> s;
    const T l1 = L.W.un - L.a, l2 = R.W.un - R.a;
    const T r1 = L.W.un + L.a, r2 = R.W.un + R.a;
    s.selLleft = !(l2 < l1);   // fmin(l1, l2): l1 unless l2 is smaller
    s.SL = s.selLleft ? l1 : l2;
    s.selRleft = !(r2 > r1);   // fmax(r1, r2): r1 unless r2 is larger
    s.SR = s.selRleft ? r1 : r2;
    return s;
}
template <class T>
EUA_HD void speeds_vjp(const Speeds<T>& s, T SLb, T SRb, SideBar<T>& Lb, SideBar<T>& Rb) {
    if (s.selLleft) { Lb.W.un += SLb; Lb.a -= SLb; } else { Rb.W.un += SLb; Rb.a -= SLb; }
    if (s.selRleft) { Lb.W.un += SRb; Lb.a += SRb; } else { Rb.W.un += SRb; Rb.a += SRb; }
}

// ---- HLL (head/riemann.hpp:87-129) ---------------------------------------
// kind: 0 central average, 1 FL, 2 FR, 3 HLL average
template <class T>
EUA_HD int hll_kind(const Side<T>& L, const Side<T>& R, const Speeds<T>& s) {
    if (!L.phys || !R.phys) return 0;
    if (s.SL >= T(0)) return 1;
    if (s.SR <= T(0)) return 2;
    if (fabs(s.SR - s.SL) < T(1.0e-14)) return 0;
    return 3;
}
template <class T>
EUA_HD C4<T> hll_primal(const Side<T>& L, const Side<T>& R, const Speeds<T>& s, int kind) {
    if (kind == 0) return avg(L.F, R.F);
    if (kind == 1) return L.F;
    if (kind == 2) return R.F;
    const T D = s.SR - s.SL, ss = s.SL * s.SR;
    return C4<T>{(s.SR * L.F.r - s.SL * R.F.r + ss * (R.U.r - L.U.r)) / D,
                 (s.SR * L.F.mn - s.SL * R.F.mn + ss * (R.U.mn - L.U.mn)) / D,
                 (s.SR * L.F.mt - s.SL * R.F.mt + ss * (R.U.mt - L.U.mt)) / D,
                 (s.SR * L.F.e - s.SL * R.F.e + ss * (R.U.e - L.U.e)) / D};
}
template <class T>
EUA_HD void hll_vjp(const Side<T>& L, const Side<T>& R, const Speeds<T>& s, int kind, const C4<T>& Fb,
                    SideBar<T>& Lb, SideBar<T>& Rb) {
    if (kind == 0) {
        side_flux_vjp(L, scale(Fb, T(0.5)), Lb);
        side_flux_vjp(R, scale(Fb, T(0.5)), Rb);
        return;
    }
    if (kind == 1) { side_flux_vjp(L, Fb, Lb); return; }
    if (kind == 2) { side_flux_vjp(R, Fb, Rb); return; }
    const T D = s.SR - s.SL, iD = T(1) / D, ss = s.SL * s.SR;
    const C4<T> F = hll_primal(L, R, s, 3);
    const C4<T> dU = sub(R.U, L.U);
    side_flux_vjp(L, scale(Fb, s.SR * iD), Lb);
    side_flux_vjp(R, scale(Fb, -s.SL * iD), Rb);
    add(Rb.U, scale(Fb, ss * iD));
    add(Lb.U, scale(Fb, -ss * iD));
    // dF/dSR = (FL + SL dU - F)/D, dF/dSL = (-FR + SR dU + F)/D
    const T SRb = (dot(Fb, L.F) + s.SL * dot(Fb, dU) - dot(Fb, F)) * iD;
    const T SLb = (-dot(Fb, R.F) + s.SR * dot(Fb, dU) + dot(Fb, F)) * iD;
    speeds_vjp(s, SLb, SRb, Lb, Rb);
}

// ---- HLLC (head/riemann.hpp:135-271) -------------------------------------
template <class T> struct Hllc {
    int mode;      // 0..3 as hll_kind (0 central, 1 FL, 2 FR, 3 HLL average), 4 star flux
    bool left, ok;
    T qL, qR, N, Dn, Sstar, dS, rs, G, A, B;
};
template <class T>
EUA_HD Hllc<T> hllc_plan(const Side<T>& L, const Side<T>& R, const Speeds<T>& s) {
    Hllc<T> h{};
    if (!L.phys || !R.phys) { h.mode = 0; return h; }
    if (s.SL >= T(0)) { h.mode = 1; return h; }
    if (s.SR <= T(0)) { h.mode = 2; return h; }
    h.qL = L.W.r * (s.SL - L.W.un);
    h.qR = R.W.r * (s.SR - R.W.un);
    h.N = R.W.p - L.W.p + h.qL * L.W.un - h.qR * R.W.un;
    h.Dn = h.qL - h.qR;
    if (fabs(h.Dn) < T(1.0e-14)) { h.mode = hll_kind(L, R, s); return h; }
    h.Sstar = h.N / h.Dn;
    if (!fin(h.Sstar)) { h.mode = hll_kind(L, R, s); return h; }
    h.mode = 4;
    h.left = h.Sstar >= T(0);
    const Side<T>& K = h.left ? L : R;
    const T S = h.left ? s.SL : s.SR;
    const T q = h.left ? h.qL : h.qR;
    h.dS = S - h.Sstar;
    h.ok = !(fabs(h.dS) < T(1.0e-14));
    if (h.ok) {
        h.rs = q / h.dS;
        h.ok = fin(h.rs) && h.rs > T(0);
    }
    if (h.ok) {
        h.A = h.Sstar - K.W.un;
        h.B = h.Sstar + K.W.p / q;
        h.G = K.U.e / K.W.r + h.A * h.B;
        h.ok = fin(h.rs * h.G);
    }
    return h;
}
template <class T>
EUA_HD C4<T> hllc_primal(const Side<T>& L, const Side<T>& R, const Speeds<T>& s, const Hllc<T>& h) {
    if (h.mode != 4) return hll_primal(L, R, s, h.mode);
    const Side<T>& K = h.left ? L : R;
    if (!h.ok) return K.F;
    const T S = h.left ? s.SL : s.SR;
    const C4<T> Us{h.rs, h.rs * h.Sstar, h.rs * K.W.ut, h.rs * h.G};
    C4<T> F = K.F;
    add(F, scale(sub(Us, K.U), S));
    return F;
}
template <class T>
EUA_HD void hllc_vjp(const Side<T>& L, const Side<T>& R, const Speeds<T>& s, const Hllc<T>& h, const C4<T>& Fb,
                     SideBar<T>& Lb, SideBar<T>& Rb) {
    if (h.mode != 4) { hll_vjp(L, R, s, h.mode, Fb, Lb, Rb); return; }
    const Side<T>& K = h.left ? L : R;
    SideBar<T>& Kb = h.left ? Lb : Rb;
    side_flux_vjp(K, Fb, Kb);
    if (!h.ok) return;
    const T S = h.left ? s.SL : s.SR;
    const T q = h.left ? h.qL : h.qR;
    const C4<T> Us{h.rs, h.rs * h.Sstar, h.rs * K.W.ut, h.rs * h.G};
    // F = F_K + S (U* - U_K)
    T Sb = dot(Fb, sub(Us, K.U));
    add(Kb.U, scale(Fb, -S));
    const C4<T> Usb = scale(Fb, S);
    T rsb = Usb.r + h.Sstar * Usb.mn + K.W.ut * Usb.mt + h.G * Usb.e;
    T Ssb = h.rs * Usb.mn;
    Kb.W.ut += h.rs * Usb.mt;
    // E* = rs G, G = E_K / rho_K + A B, A = S* - un_K, B = S* + p_K / q
    const T Gb = h.rs * Usb.e;
    Kb.U.e += Gb / K.W.r;
    Kb.U.r -= Gb * K.U.e / (K.W.r * K.W.r);
    const T Ab = Gb * h.B, Bb = Gb * h.A;
    Ssb += Ab + Bb;
    Kb.W.un -= Ab;
    Kb.W.p += Bb / q;
    T qb = -Bb * K.W.p / (q * q);
    // rs = q / dS, dS = S - S*
    qb += rsb / h.dS;
    const T dSb = -rsb * h.rs / h.dS;
    Sb += dSb;
    Ssb -= dSb;
    T qLb = h.left ? qb : T(0), qRb = h.left ? T(0) : qb;
    T SLb = h.left ? Sb : T(0), SRb = h.left ? T(0) : Sb;
    // S* = N / Dn, N = pR - pL + qL unL - qR unR, Dn = qL - qR
    const T Nb = Ssb / h.Dn, Dnb = -Ssb * h.Sstar / h.Dn;
    Rb.W.p += Nb;
    Lb.W.p -= Nb;
    qLb += Nb * L.W.un + Dnb;
    Lb.W.un += Nb * h.qL;
    qRb += -Nb * R.W.un - Dnb;
    Rb.W.un -= Nb * h.qR;
    // qL = rL (SL - unL), qR = rR (SR - unR)
    Lb.W.r += qLb * (s.SL - L.W.un);
    SLb += qLb * L.W.r;
    Lb.W.un -= qLb * L.W.r;
    Rb.W.r += qRb * (s.SR - R.W.un);
    SRb += qRb * R.W.r;
    Rb.W.un -= qRb * R.W.r;
    speeds_vjp(s, SLb, SRb, Lb, Rb);
}

// ---- FORCE (head/riemann.hpp:284-325, local alpha) -----------------------
template <class T> struct Force {
    int mode;      // 0 central average, 1 Lax-Friedrichs part only, 2 full
    bool selL;     // alpha from the left state
    T alpha;
    C4<T> Uri;
    W4<T> Wri;
};
template <class T> EUA_HD Force<T> force_plan(const Side<T>& L, const Side<T>& R) {
    Force<T> f{};
    if (!L.phys || !R.phys) { f.mode = 0; return f; }
    const T xl = fabs(L.W.un) + L.a, xr = fabs(R.W.un) + R.a;
    f.selL = !(xr > xl);
    f.alpha = f.selL ? xl : xr;
    if (!fin(f.alpha) || f.alpha <= T(1.0e-14)) { f.mode = 0; return f; }
    const T hia = T(0.5) / f.alpha;
    const C4<T> Ua = avg(L.U, R.U);
    f.Uri = sub(Ua, scale(sub(R.F, L.F), hia));
    f.Wri = c2p(f.Uri);
    f.mode = phys_riemann(f.Wri) ? 2 : 1;
    return f;
}
template <class T> EUA_HD C4<T> force_primal(const Side<T>& L, const Side<T>& R, const Force<T>& f) {
    const C4<T> Fc = avg(L.F, R.F);
    if (f.mode == 0) return Fc;
    const C4<T> Flf = sub(Fc, scale(sub(R.U, L.U), T(0.5) * f.alpha));
    if (f.mode == 1) return Flf;
    return avg(Flf, flux(f.Uri, f.Wri));
}
template <class T>
EUA_HD void force_vjp(const Side<T>& L, const Side<T>& R, const Force<T>& f, const C4<T>& Fb, SideBar<T>& Lb,
                      SideBar<T>& Rb) {
    if (f.mode == 0) {
        side_flux_vjp(L, scale(Fb, T(0.5)), Lb);
        side_flux_vjp(R, scale(Fb, T(0.5)), Rb);
        return;
    }
    C4<T> Flfb = Fb, Urib = zero4<T>();
    if (f.mode == 2) {
        Flfb = scale(Fb, T(0.5));
        W4<T> Wrib = zerow<T>();
        flux_vjp(f.Uri, f.Wri, scale(Fb, T(0.5)), Urib, Wrib);
        c2p_vjp(f.Wri, Wrib, Urib);
    }
    // Flf = Fc - alpha/2 (UR - UL)
    T ab = -T(0.5) * dot(Flfb, sub(R.U, L.U));
    add(Rb.U, scale(Flfb, -T(0.5) * f.alpha));
    add(Lb.U, scale(Flfb, T(0.5) * f.alpha));
    C4<T> FLb = scale(Flfb, T(0.5)), FRb = scale(Flfb, T(0.5));
    if (f.mode == 2) {
        // Uri = (UL + UR)/2 - (FR - FL)/(2 alpha)
        add(Lb.U, scale(Urib, T(0.5)));
        add(Rb.U, scale(Urib, T(0.5)));
        const T hia = T(0.5) / f.alpha;
        ab += dot(Urib, sub(R.F, L.F)) * hia / f.alpha;
        add(FRb, scale(Urib, -hia));
        add(FLb, scale(Urib, hia));
    }
    side_flux_vjp(L, FLb, Lb);
    side_flux_vjp(R, FRb, Rb);
    // alpha = max(|unL| + aL, |unR| + aR)
    if (f.selL) { Lb.W.un += (L.W.un >= T(0) ? ab : -ab); Lb.a += ab; }
    else { Rb.W.un += (R.W.un >= T(0) ? ab : -ab); Rb.a += ab; }
}

// ---- exact solver (head/riemann.hpp:331-644) -----------------------------
// f_K(p) and its partial derivatives w.r.t. p, rho_K, p_K, a_K
struct PFun { double f, fp, fr, fpk, fa; };
EUA_HD PFun pfun(double p, double rK, double pK, double aK) {
    PFun o;
    if (p > pK) {
        const double A = 2.0 / ((kG + 1.0) * rK);
        const double B = (kG - 1.0) / (kG + 1.0) * pK;
        const double Q = sqrt(A / (p + B));
        o.f = (p - pK) * Q;
        o.fp = Q * (1.0 - 0.5 * (p - pK) / (p + B));
        o.fr = -0.5 * o.f / rK;
        o.fpk = -Q - 0.5 * (p - pK) * Q / (p + B) * ((kG - 1.0) / (kG + 1.0));
        o.fa = 0.0;
    } else {
        const double pr = p / pK, z = (kG - 1.0) / (2.0 * kG);
        const double prz = pow(pr, z);
        o.f = 2.0 * aK / (kG - 1.0) * (prz - 1.0);
        o.fp = (1.0 / (rK * aK)) * pow(pr, -(kG + 1.0) / (2.0 * kG));
        o.fpk = -o.fp * p / pK;
        o.fa = 2.0 / (kG - 1.0) * (prz - 1.0);
        o.fr = 0.0;
    }
    return o;
}
// PVRS guess, <= 20 Newton steps with halving (head/riemann.hpp:361-443), in FP64
EUA_HD_NOINLINE bool exact_star_d(double rL, double uL, double pL, double aL, double rR, double uR, double pR,
                                  double aR, double& ps, double& us) {
    const double pv = 0.5 * (pL + pR) - 0.125 * (uR - uL) * (rL + rR) * (aL + aR);
    ps = fmax(1.0e-12, pv);
    for (int it = 0; it < 20; ++it) {
        const PFun l = pfun(ps, rL, pL, aL), r = pfun(ps, rR, pR, aR);
        const double f = l.f + r.f + (uR - uL);
        const double fd = l.fp + r.fp;
        if (fabs(fd) < 1.0e-14) return false;
        const double po = ps;
        ps = po - f / fd;
        if (!(fabs(ps) < INFINITY) || ps <= 0.0) ps = 0.5 * po;
        if (fabs(ps - po) / (0.5 * (ps + po) + 1.0e-14) < 1.0e-8) break;
    }
    if (!(fabs(ps) < INFINITY) || ps <= 0.0) return false;
    const PFun l = pfun(ps, rL, pL, aL), r = pfun(ps, rR, pR, aR);
    us = 0.5 * (uL + uR + r.f - l.f);
    return fabs(us) < INFINITY;
}
// p*, u* in the working type.  (A number type that carries derivatives can
// overload this to attach dp*/dtheta by implicit differentiation.)
template <class T>
EUA_HD void star_refine(const Side<T>&, const Side<T>&, double ps, double us, T& tps, T& tus) {
    tps = T(ps);
    tus = T(us);
}
template <class T> struct Exact {
    int mode;     // 0..3 HLL kinds (fallbacks), 4 sampled state
    bool left;
    int branch;   // 0 side state, 1 shock star, 2 rarefaction star, 3 fan
    T ps, us;     // p*, u*
    W4<T> Ws;     // sampled primitive state
    C4<T> Us;
    Speeds<T> sp;
};
template <class T> EUA_HD Exact<T> exact_plan(const Side<T>& L, const Side<T>& R) {
    Exact<T> x{};
    x.sp = speeds(L, R);
    if (!L.phys || !R.phys) { x.mode = 0; return x; }
    double ps, us;
    if (!exact_star_d((double)L.W.r, (double)L.W.un, (double)L.W.p, (double)L.a, (double)R.W.r,
                      (double)R.W.un, (double)R.W.p, (double)R.a, ps, us)) {
        x.mode = hll_kind(L, R, x.sp);
        return x;
    }
    star_refine(L, R, ps, us, x.ps, x.us);
    x.left = us >= 0.0;
    const Side<T>& K = x.left ? L : R;
    const T sg = x.left ? T(1) : T(-1);
    const T g = T(kG);
    const T unK = sg * K.W.un, uss = sg * x.us;
    T rho = K.W.r, un = unK, p = K.W.p;
    x.branch = 0;
    if (x.ps > K.W.p) {
        const T pr = x.ps / K.W.p;
        const T S = unK - K.a * tsqrt((g + T(1)) / (T(2) * g) * pr + (g - T(1)) / (T(2) * g));
        if (!(T(0) <= S)) {
            const T k = (g - T(1)) / (g + T(1));
            rho = K.W.r * ((pr + k) / (k * pr + T(1)));
            un = uss;
            p = x.ps;
            x.branch = 1;
        }
    } else {
        const T a_star = K.a * tpow(x.ps / K.W.p, (g - T(1)) / (T(2) * g));
        const T SH = unK - K.a, ST = uss - a_star;
        if (T(0) <= SH) {
        } else if (T(0) >= ST) {
            rho = K.W.r * tpow(x.ps / K.W.p, T(1) / g);
            un = uss;
            p = x.ps;
            x.branch = 2;
        } else {
            un = T(2) / (g + T(1)) * (K.a + T(0.5) * (g - T(1)) * unK);
            const T ar = un / K.a;
            rho = K.W.r * tpow(ar, T(2) / (g - T(1)));
            p = K.W.p * tpow(ar, T(2) * g / (g - T(1)));
            x.branch = 3;
        }
    }
    x.Ws = W4<T>{rho, sg * un, K.W.ut, p};
    x.Us = p2c(x.Ws);
    if (!phys_riemann(c2p(x.Us))) { x.mode = hll_kind(L, R, x.sp); return x; }
    x.mode = 4;
    return x;
}
template <class T> EUA_HD C4<T> exact_primal(const Side<T>& L, const Side<T>& R, const Exact<T>& x) {
    if (x.mode != 4) return hll_primal(L, R, x.sp, x.mode);
    return flux(x.Us, x.Ws);
}
template <class T>
EUA_HD void exact_vjp(const Side<T>& L, const Side<T>& R, const Exact<T>& x, const C4<T>& Fb, SideBar<T>& Lb,
                      SideBar<T>& Rb) {
    if (x.mode != 4) { hll_vjp(L, R, x.sp, x.mode, Fb, Lb, Rb); return; }
    W4<T> Wsb = zerow<T>();
    fluxw_vjp(x.Ws, x.Us, Fb, Wsb);
    const Side<T>& K = x.left ? L : R;
    SideBar<T>& Kb = x.left ? Lb : Rb;
    const T sg = x.left ? T(1) : T(-1);
    const T g = T(kG);
    Kb.W.ut += Wsb.ut;
    T psb = 0, usb = 0;
    const T unb_loc = sg * Wsb.un;   // un_final = sg * un_local
    if (x.branch == 0) {
        Kb.W.r += Wsb.r;
        Kb.W.un += Wsb.un;
        Kb.W.p += Wsb.p;
    } else if (x.branch == 1 || x.branch == 2) {
        const T pr = x.ps / K.W.p;
        T prb;
        if (x.branch == 1) {
            const T k = (g - T(1)) / (g + T(1));
            const T den = k * pr + T(1);
            Kb.W.r += Wsb.r * (pr + k) / den;
            prb = Wsb.r * K.W.r * (T(1) - k * k) / (den * den);
        } else {
            const T e = T(1) / g;
            Kb.W.r += Wsb.r * tpow(pr, e);
            prb = Wsb.r * K.W.r * e * tpow(pr, e - T(1));
        }
        psb += prb / K.W.p + Wsb.p;
        Kb.W.p -= prb * pr / K.W.p;
        usb += sg * unb_loc;   // un_local = sg * u*
    } else {
        const T unK = sg * K.W.un;
        const T unl = T(2) / (g + T(1)) * (K.a + T(0.5) * (g - T(1)) * unK);
        const T ar = unl / K.a;
        const T er = T(2) / (g - T(1)), ep = T(2) * g / (g - T(1));
        const T rho = x.Ws.r, p = x.Ws.p;
        const T arb = Wsb.r * rho * er / ar + Wsb.p * p * ep / ar;
        Kb.W.r += Wsb.r * tpow(ar, er);
        Kb.W.p += Wsb.p * tpow(ar, ep);
        const T unlb = unb_loc + arb / K.a;
        Kb.a += -arb * ar / K.a + unlb * T(2) / (g + T(1));
        Kb.W.un += sg * unlb * (g - T(1)) / (g + T(1));
    }
    // u* = (unL + unR + fR(p*) - fL(p*)) / 2, f(p*) = fL + fR + unR - unL = 0
    const PFun l = pfun((double)x.ps, (double)L.W.r, (double)L.W.p, (double)L.a);
    const PFun r = pfun((double)x.ps, (double)R.W.r, (double)R.W.p, (double)R.a);
    Lb.W.un += T(0.5) * usb;
    Rb.W.un += T(0.5) * usb;
    const T fRb = T(0.5) * usb, fLb = -T(0.5) * usb;
    psb += fRb * T(r.fp) + fLb * T(l.fp);
    Lb.W.r += fLb * T(l.fr); Lb.W.p += fLb * T(l.fpk); Lb.a += fLb * T(l.fa);
    Rb.W.r += fRb * T(r.fr); Rb.W.p += fRb * T(r.fpk); Rb.a += fRb * T(r.fa);
    // implicit: dp* = -(df/dtheta) / (df/dp*)
    const T w = -psb / T(l.fp + r.fp);
    Lb.W.r += w * T(l.fr); Lb.W.p += w * T(l.fpk); Lb.a += w * T(l.fa);
    Rb.W.r += w * T(r.fr); Rb.W.p += w * T(r.fpk); Rb.a += w * T(r.fa);
    Rb.W.un += w;
    Lb.W.un -= w;
}

// ---- dispatch ---------------------------------------------------------------
// Flux of the face between states UL (left) and UR (right).
template <int S, class T> EUA_HD C4<T> riemann_primal(const C4<T>& UL, const C4<T>& UR) {
    const Side<T> L = side_of(UL), R = side_of(UR);
    if constexpr (S == 1) {
        const Speeds<T> s = speeds(L, R);
        return hllc_primal(L, R, s, hllc_plan(L, R, s));
    } else if constexpr (S == 2) {
        return exact_primal(L, R, exact_plan(L, R));
    } else if constexpr (S == 3) {
        return force_primal(L, R, force_plan(L, R));
    } else {
        const Speeds<T> s = speeds(L, R);
        return hll_primal(L, R, s, hll_kind(L, R, s));
    }
}
// (ULbar, URbar) = J^T Fbar
template <int S, class T>
EUA_HD void riemann_vjp(const C4<T>& UL, const C4<T>& UR, const C4<T>& Fb, C4<T>& ULb, C4<T>& URb) {
    const Side<T> L = side_of(UL), R = side_of(UR);
    SideBar<T> Lb = zero_side<T>(), Rb = zero_side<T>();
    if constexpr (S == 1) {
        const Speeds<T> s = speeds(L, R);
        hllc_vjp(L, R, s, hllc_plan(L, R, s), Fb, Lb, Rb);
    } else if constexpr (S == 2) {
        exact_vjp(L, R, exact_plan(L, R), Fb, Lb, Rb);
    } else if constexpr (S == 3) {
        force_vjp(L, R, force_plan(L, R), Fb, Lb, Rb);
    } else {
        const Speeds<T> s = speeds(L, R);
        hll_vjp(L, R, s, hll_kind(L, R, s), Fb, Lb, Rb);
    }
    ULb = side_close(L, Lb);
    URb = side_close(R, Rb);
}

// ---------------------------------------------------------------------------
// One tile of an adjoint sweep: NL lines x up to TC consecutive cells
// [c0, c0+tl) of each line.  Five phases over the tile, each parallel over
// its cells (tid/nthr: the calling thread and the thread count; a CPU caller
// passes 0/1 and runs the phases in order):
//   P0  load W = cons_to_prim(U) and the output adjoints a for cells
//       c0-3 .. c0+tl+2 (indices clamped to the ghost frame; a = 0 off the
//       interior)
//   P1  reconstruct cells c0-2 .. c0+tl+1 -> evolved face states L*, R*
//   P2  faces c0-3/2 .. c0+tl+1/2: Fbar = (dt/d)(a_right - a_left), then the
//       Riemann vjp -> Rbar* of the left cell, Lbar* of the right cell (in
//       place of L*, R*: every slot is read and written by one face only)
//   P3  reconstruction vjp of cells c0-1 .. c0+tl -> primitive adjoints of
//       each cell's three inputs
//   P4  gather: Ubar_c = a_c + J_c2p^T (sum of the three contributions), and
//       at a domain edge the boundary rule's transpose (transmissive: both
//       ghost adjoints onto the edge cell; reflective: mirror images with
//       the normal momentum negated onto the two edge cells)
// The accessor supplies load_state(l, c), load_adj(l, c), store(l, c, U),
// line_ok(l) and the scalars n, hl = dt/(2d), lam = dt/d, bc_lo, bc_hi.
// ---------------------------------------------------------------------------
#if defined(__CUDA_ARCH__)
#define EUA_SYNC() __syncthreads()
#else
#define EUA_SYNC() ((void)0)
#endif

// Shared tile of NL lines x (TC + 6) cells, one array per quantity.  With
// lines fastest (LF: consecutive threads on consecutive lines, same cell)
// the line stride is padded to one element past a multiple of 128 bytes, so
// that a quarter-warp's 16-byte accesses fall on distinct banks (FP32; FP64
// elements of 32 bytes: two per 128 bytes at most).  Cells fastest needs no
// padding: consecutive threads read consecutive elements.
template <class T, int NL, int TC, bool LF = false> struct TileMem {
    static constexpr int kQ = 128 / (int)sizeof(C4<T>);
    static constexpr int W_ = LF ? (TC + 6 - 1 + kQ - 1) / kQ * kQ + 1 : TC + 6;
    W4<T> W[NL][W_];
    C4<T> A[NL][W_];
    C4<T> L[NL][W_];       // L* (P1) -> adjoint of L* (P2) -> contribution to the left neighbour (P3)
    C4<T> R[NL][W_];       // R* (P1) -> adjoint of R* (P2) -> contribution to the cell itself (P3)
    W4<T> Xp[NL][W_];      // contribution to the right neighbour (P3)
};

// idx -> (line, cell) with lines fastest (LF) or cells fastest
template <bool LF, int NL> EUA_HD void tile_split(int idx, int width, int& l, int& cc) {
    if (LF) { l = idx % NL; cc = idx / NL; }
    else { l = idx / width; cc = idx % width; }
}

template <int S, class T, int NL, int TC, bool LF, class Acc>
EUA_HD void adjoint_tile(const Acc& acc, TileMem<T, NL, TC, LF>& m, int line0, int c0, int tl, int tid, int nthr) {
    const int n = acc.n;
    const T hl = acc.hl, lam = acc.lam;
    // P0
    {
        const int w = tl + 6;
        for (int idx = tid; idx < NL * w; idx += nthr) {
            int l, cc;
            tile_split<LF, NL>(idx, w, l, cc);
            const int line = line0 + l;
            const int c = c0 - 3 + cc;
            const int cl = c < -2 ? -2 : (c > n + 1 ? n + 1 : c);
            const bool ok = acc.line_ok(line);
            const C4<T> U = acc.load_state(ok ? line : line0, cl);
            m.W[l][cc] = c2p(U);
            m.A[l][cc] = (ok && c >= 0 && c < n) ? acc.load_adj(line, c) : zero4<T>();
        }
    }
    EUA_SYNC();
    // P1: cells cc in [1, tl+5)
    {
        const int w = tl + 4;
        for (int idx = tid; idx < NL * w; idx += nthr) {
            int l, k;
            tile_split<LF, NL>(idx, w, l, k);
            const int cc = k + 1;
            Recon<T> o;
            recon_primal(m.W[l][cc - 1], m.W[l][cc], m.W[l][cc + 1], hl, o);
            m.L[l][cc] = o.L;
            m.R[l][cc] = o.R;
        }
    }
    EUA_SYNC();
    // P2: faces with left cell cc in [1, tl+4)
    {
        const int w = tl + 3;
        for (int idx = tid; idx < NL * w; idx += nthr) {
            int l, k;
            tile_split<LF, NL>(idx, w, l, k);
            const int cc = k + 1;
            const C4<T> Fb = scale(sub(m.A[l][cc + 1], m.A[l][cc]), lam);
            C4<T> Lb, Rb;
            riemann_vjp<S>(m.R[l][cc], m.L[l][cc + 1], Fb, Lb, Rb);
            m.R[l][cc] = Lb;       // adjoint of R* of the left cell
            m.L[l][cc + 1] = Rb;   // adjoint of L* of the right cell
        }
    }
    EUA_SYNC();
    // P3: cells cc in [2, tl+4)
    {
        const int w = tl + 2;
        for (int idx = tid; idx < NL * w; idx += nthr) {
            int l, k;
            tile_split<LF, NL>(idx, w, l, k);
            const int cc = k + 2;
            Recon<T> o;
            recon_primal(m.W[l][cc - 1], m.W[l][cc], m.W[l][cc + 1], hl, o);
            W4<T> bm = zerow<T>(), bc = zerow<T>(), bp = zerow<T>();
            recon_vjp(o, hl, m.L[l][cc], m.R[l][cc], bm, bc, bp);
            m.L[l][cc] = C4<T>{bm.r, bm.un, bm.ut, bm.p};
            m.R[l][cc] = C4<T>{bc.r, bc.un, bc.ut, bc.p};
            m.Xp[l][cc] = bp;
        }
    }
    EUA_SYNC();
    // P4: cells cc in [3, tl+3)
    {
        const int w = tl;
        for (int idx = tid; idx < NL * w; idx += nthr) {
            int l, k;
            tile_split<LF, NL>(idx, w, l, k);
            const int line = line0 + l;
            if (!acc.line_ok(line)) continue;
            const int cc = k + 3;
            const int c = c0 + k;
            // primitive adjoint gathered from the reconstructions of c-1, c, c+1
            auto wbar = [&](int q, bool left_ok, bool right_ok) {
                W4<T> b = W4<T>{m.R[l][q].r, m.R[l][q].mn, m.R[l][q].mt, m.R[l][q].e};
                if (left_ok) add(b, m.Xp[l][q - 1]);
                if (right_ok) {
                    const C4<T>& x = m.L[l][q + 1];
                    add(b, W4<T>{x.r, x.mn, x.mt, x.e});
                }
                return b;
            };
            auto ubar = [&](int q, const W4<T>& b) {
                C4<T> u = zero4<T>();
                c2p_vjp(m.W[l][q], b, u);
                return u;
            };
            C4<T> G = m.A[l][cc];
            c2p_vjp(m.W[l][cc], wbar(cc, true, true), G);
            // boundary transpose: ghost cells hold copies of edge cells
            const bool refl_lo = acc.bc_lo == 1, refl_hi = acc.bc_hi == 1;
            if (c == 0 || (c == 1 && refl_lo)) {
                // ghost -1 (cc-1 of cell 0): reconstructions of -1 and 0; ghost -2: of -1 only
                const int q1 = cc - c - 1, q2 = cc - c - 2;   // tile slots of ghosts -1, -2
                const C4<T> g1 = ubar(q1, wbar(q1, false, true));
                W4<T> b2 = zerow<T>();
                { const C4<T>& x = m.L[l][q2 + 1]; add(b2, W4<T>{x.r, x.mn, x.mt, x.e}); }
                const C4<T> g2 = ubar(q2, b2);
                if (!refl_lo) { add(G, g1); add(G, g2); }
                else if (c == 0) add(G, C4<T>{g1.r, -g1.mn, g1.mt, g1.e});
                else add(G, C4<T>{g2.r, -g2.mn, g2.mt, g2.e});
            }
            if (c == n - 1 || (c == n - 2 && refl_hi)) {
                const int q1 = cc + (n - c), q2 = q1 + 1;      // tile slots of ghosts n, n+1
                const C4<T> g1 = ubar(q1, wbar(q1, true, false));
                const C4<T> g2 = ubar(q2, m.Xp[l][q2 - 1]);
                if (!refl_hi) { add(G, g1); add(G, g2); }
                else if (c == n - 1) add(G, C4<T>{g1.r, -g1.mn, g1.mt, g1.e});
                else add(G, C4<T>{g2.r, -g2.mn, g2.mt, g2.e});
            }
            acc.store(line, c, G);
        }
    }
}

// Balanced split of n cells into ceil(n / TC) tiles of at least TC/2 cells
// (n >= TC) so the two cells at each end of a line share their edge tile.
EUA_HD void tile_range(int n, int TC, int t, int& c0, int& c1) {
    const int nt = (n + TC - 1) / TC;
    c0 = (int)((long long)t * n / nt);
    c1 = (int)((long long)(t + 1) * n / nt);
}

}  // namespace adj
}  // namespace eu
