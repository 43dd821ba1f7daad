// euler_numerics.cuh -- device numerics of the MUSCL-Hancock split step.
//
// States are held in sweep-local (normal, tangential) coordinates: for the
// x-sweep (mn, mt) = (rho*u, rho*v), for the y-sweep (mn, mt) = (rho*v, rho*u).
// The reference writes flux_x/flux_y and every Riemann solver with an explicit
// Direction argument (head/physics.hpp:56-74, head/riemann.hpp:24-64); in
// (n, t) coordinates the two directions are the same formulas, so one code
// path serves both sweeps and the y-sweep only swaps the two momentum planes
// when it loads and stores.
//
// The branch structure (physicality guards, upwind cases, HLLC->HLL
// fallbacks, exact-solver Newton with halving, FORCE fallbacks) follows the
// reference line by line; the arithmetic is reorganised for the GPU:
//   * every primitive state is computed once per cell and reused (the
//     reference reconstructs each cell twice per sweep, src/cpu/solver_cpu.cpp:118-136,
//     and re-derives primitives inside every flux and Riemann call);
//   * divisions by constants and repeated divisions by the same value become
//     multiplications by a reciprocal;
//   * the FP32 form (T = float) runs in single precision with approximate
//     reciprocal / square root, and keeps FP64 in two places, each of them
//     conditional (a deviation from an unconditional FP64 island, stated
//     with the FP32 error figures):
//       - pressure recovery p = (gamma-1)(E - rho|u|^2/2) is redone in FP64
//         only when the kinetic energy exceeds half the total energy (there
//         the FP32 subtraction would lose more than one bit to
//         cancellation; below it loses at most one);
//       - the exact solver's p*: Newton's iteration runs in FP32 to a
//         relative step of 1e-5 and is finished by one FP64 Newton step
//         (exact_star_mixed); irregular cases (non-positive iterate, no
//         convergence in 12 steps, tiny f', a large FP64 step) run the full
//         FP64 iteration.  The FP64 form keeps the reference's iteration.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#include "lanes.cuh"


namespace eu {

enum SolverId { kHLL = 0, kHLLC = 1, kExact = 2, kFORCE = 3 };

constexpr double kGammaD = 1.4;                 // head/physics.hpp:11
constexpr double kGm1D = kGammaD - 1.0;         // 0.3999999999999999 as in the reference
constexpr double kRhoFloorD = 1.0e-12;          // src/cpu/solver_cpu.cpp:19-20
constexpr double kPFloorD = 1.0e-12;

template <class T> struct Cons { T r, mn, mt, e; };
template <class T> struct Prim { T r, un, ut, p, ir; };   // ir = 1/rho when known

// ---------------------------------------------------------------------------
// Scalar arithmetic per precision
// ---------------------------------------------------------------------------
template <class T> struct Ar;

// FP64 comparisons run on the integer pipes, off the FP64 pipe (this part's
// narrowest): non-negative doubles order like their bit patterns as
// integers, negative ones in reverse, and the patterns whose magnitude lies
// above +inf's are the NaNs.  Each helper has the IEEE comparison's result
// for every input, NaN included; fmin_/fmax_ return the other argument for
// one NaN, as fmin/fmax do, and differ from them at most in the sign of a
// zero result.
template <> struct Ar<double> {
    static constexpr long long kInf = 0x7ff0000000000000ll;
    static constexpr long long kMag = 0x7fffffffffffffffll;
    static __device__ __forceinline__ long long bits(double x) { return __double_as_longlong(x); }
    static __device__ __forceinline__ bool nan_(long long i) { return (i & kMag) > kInf; }
    // total-order key: increasing with the value (-0 below +0)
    static __device__ __forceinline__ long long key(long long i) { return i ^ ((i >> 63) & kMag); }
    static __device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
    static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
    static __device__ __forceinline__ double fabs_(double x) { return fabs(x); }
    static __device__ __forceinline__ double fmin_(double a, double b) {
        const long long ia = bits(a), ib = bits(b);
        return (nan_(ib) || (!nan_(ia) && key(ia) <= key(ib))) ? a : b;
    }
    static __device__ __forceinline__ double fmax_(double a, double b) {
        const long long ia = bits(a), ib = bits(b);
        return (nan_(ib) || (!nan_(ia) && key(ia) >= key(ib))) ? a : b;
    }
    // x > c for a finite c >= 0
    static __device__ __forceinline__ bool gt(double x, double c) {
        const long long i = bits(x);
        return i > bits(c) && i <= kInf;
    }

    // exponent field not all ones (on the integer pipes)
    static __device__ __forceinline__ bool finite(double x) {
        return (__double2hiint(x) & 0x7ff00000) != 0x7ff00000;
    }
    static __device__ __forceinline__ double pow_(double a, double b) { return pow(a, b); }
    static __device__ __forceinline__ double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }
};

template <> struct Ar<float> {
    // Hardware approximate reciprocal and square root (PTX rcp.approx /
    // sqrt.approx, about 1 ulp); the FP32 form is judged against FP64 by its
    // L1/Linf error, not bit for bit.
    static __device__ __forceinline__ float rcp(float x) {
        float y;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
        return y;
    }
    static __device__ __forceinline__ float sqrt_(float x) {
        float y;
        asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
        return y;
    }
    static __device__ __forceinline__ float fabs_(float x) { return fabsf(x); }
    static __device__ __forceinline__ float fmin_(float a, float b) { return fminf(a, b); }
    static __device__ __forceinline__ float fmax_(float a, float b) { return fmaxf(a, b); }
    static __device__ __forceinline__ bool finite(float x) { return fabsf(x) < INFINITY; }
    static __device__ __forceinline__ float pow_(float a, float b) { return powf(a, b); }
    static __device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
};

template <class T> __device__ __forceinline__ T gm1() { return T(kGm1D); }
template <class T> __device__ __forceinline__ T inv_gm1() { return T(1.0 / kGm1D); }
template <class T> __device__ __forceinline__ T gam() { return T(kGammaD); }

// Arithmetic of the full-logic path (cell_full and the functions it calls).
// FP64 keeps plain operators (fused by the compiler, within the tolerance of
// the FP64 parity tests).  FP32 fixes every rounding (lanes.cuh), so that a
// flagged cell's bits do not depend on the kernel the call is compiled into:
// the same cell may be recomputed in full by the x-sweep, by either y-sweep
// pass or by an ensemble task, and must come out the same from each.
template <class T> __device__ __forceinline__ T xadd(T a, T b) { return a + b; }
template <class T> __device__ __forceinline__ T xsub(T a, T b) { return a - b; }
template <class T> __device__ __forceinline__ T xmul(T a, T b) { return a * b; }
template <class T> __device__ __forceinline__ T xfma(T a, T b, T c) { return a * b + c; }   // a b + c
template <class T> __device__ __forceinline__ T xfms(T a, T b, T c) { return c - a * b; }   // c - a b
template <> __device__ __forceinline__ float xadd<float>(float a, float b) { return vadd(a, b); }
template <> __device__ __forceinline__ float xsub<float>(float a, float b) { return vsub(a, b); }
template <> __device__ __forceinline__ float xmul<float>(float a, float b) { return vmul(a, b); }
template <> __device__ __forceinline__ float xfma<float>(float a, float b, float c) { return vfma(a, b, c); }
template <> __device__ __forceinline__ float xfms<float>(float a, float b, float c) { return vfma(-a, b, c); }

// ---------------------------------------------------------------------------
// head/physics.hpp:13-20  cons_to_prim (pressure recovery)
// ---------------------------------------------------------------------------
template <class T> __device__ __forceinline__ Prim<T> cons_to_prim(const Cons<T>& U);

template <> __device__ __forceinline__ Prim<double> cons_to_prim<double>(const Cons<double>& U) {
    Prim<double> V;
    V.ir = 1.0 / U.r;
    V.r = U.r;
    V.un = U.mn * V.ir;
    V.ut = U.mt * V.ir;
    const double kinetic = 0.5 * U.r * (V.un * V.un + V.ut * V.ut);
    V.p = kGm1D * (U.e - kinetic);
    return V;
}

// FP64 recovery of p from the FP32 conserved state: exact squares of the
// 24-bit momenta, one IEEE division.  Taken only where the FP32 form would
// cancel (kinetic > E/2), i.e. strong rarefactions and high-Mach flow.
static __device__ __noinline__ float pressure_fp64(float r, float mn, float mt, float e) {
    const double kin = __ddiv_rn(__dmul_rn(0.5, __fma_rn((double)mn, (double)mn, __dmul_rn((double)mt, (double)mt))),
                                 (double)r);
    return __double2float_rn(__dmul_rn(kGm1D, __dsub_rn((double)e, kin)));
}

template <> __device__ __forceinline__ Prim<float> cons_to_prim<float>(const Cons<float>& U) {
    Prim<float> V;
    V.ir = vrcp(U.r);
    V.r = U.r;
    V.un = vmul(U.mn, V.ir);
    V.ut = vmul(U.mt, V.ir);
    const float kinetic = vmul(vmul(0.5f, U.r), vfma(V.un, V.un, vmul(V.ut, V.ut)));
    V.p = vmul(gm1<float>(), vsub(U.e, kinetic));
    if (__builtin_expect(vmul(2.0f, kinetic) > U.e, 0)) V.p = pressure_fp64(U.r, U.mn, U.mt, U.e);
    return V;
}

// head/physics.hpp:22-28
template <class T> __device__ __forceinline__ Cons<T> prim_to_cons(const Prim<T>& V) {
    Cons<T> U;
    U.r = V.r;
    U.mn = xmul(V.r, V.un);
    U.mt = xmul(V.r, V.ut);
    const T kinetic = xmul(xmul(T(0.5), V.r), xfma(V.un, V.un, xmul(V.ut, V.ut)));
    U.e = xfma(V.p, inv_gm1<T>(), kinetic);
    return U;
}

// head/physics.hpp:39-41 with 1/rho reused
template <class T> __device__ __forceinline__ T sound_speed(const Prim<T>& V) {
    return Ar<T>::sqrt_(gam<T>() * V.p * V.ir);
}

// head/physics.hpp:56-74 normal flux, given the state's primitives
template <class T> __device__ __forceinline__ Cons<T> flux(const Cons<T>& U, const Prim<T>& V) {
    Cons<T> F;
    F.r = U.mn;
    F.mn = xfma(U.mn, V.un, V.p);
    F.mt = xmul(U.mt, V.un);
    F.e = xmul(xadd(U.e, V.p), V.un);
    return F;
}

template <class T> __device__ __forceinline__ Cons<T> c_avg(const Cons<T>& a, const Cons<T>& b) {
    return Cons<T>{T(0.5) * (a.r + b.r), T(0.5) * (a.mn + b.mn), T(0.5) * (a.mt + b.mt),
                   T(0.5) * (a.e + b.e)};
}

// head/riemann.hpp:74-81
template <class T> __device__ __forceinline__ bool physical_riemann(const Prim<T>& V) {
    return Ar<T>::finite(V.un) && Ar<T>::finite(V.ut) && V.r > T(0) && V.p > T(0) &&
           V.r < T(INFINITY) && V.p < T(INFINITY);
}

// src/cpu/solver_cpu.cpp:39-43
template <class T> __device__ __forceinline__ bool physical_recon(const Prim<T>& V) {
    return Ar<T>::finite(V.un) && Ar<T>::finite(V.ut) && V.r > T(kRhoFloorD) &&
           V.p > T(kPFloorD) && V.r < T(INFINITY) && V.p < T(INFINITY);
}

// FP64: the same tests on the integer pipes (non-negative doubles order like
// their bit patterns as signed integers; negative ones and -0 have negative
// patterns; +inf and the NaNs lie at and above 0x7ff0...).
__device__ __forceinline__ bool finite_above(double x, double floor) {
    const long long ix = __double_as_longlong(x);
    return ix > __double_as_longlong(floor) && ix < Ar<double>::kInf;
}
template <> __device__ __forceinline__ bool physical_riemann<double>(const Prim<double>& V) {
    return Ar<double>::finite(V.un) && Ar<double>::finite(V.ut) && finite_above(V.r, 0.0) &&
           finite_above(V.p, 0.0);
}
template <> __device__ __forceinline__ bool physical_recon<double>(const Prim<double>& V) {
    static_assert(kRhoFloorD == kPFloorD, "one floor for rho and p");
    return Ar<double>::finite(V.un) && Ar<double>::finite(V.ut) && finite_above(V.r, kRhoFloorD) &&
           finite_above(V.p, kPFloorD);
}

// ---------------------------------------------------------------------------
// Riemann solvers.  Inputs carry their primitives (V = cons_to_prim(U)).
// ---------------------------------------------------------------------------
// HLL flux given the wave-speed estimates and the physical fluxes
// (head/riemann.hpp:114-128).
template <class T>
__device__ __forceinline__ Cons<T> hll_from(const Cons<T>& UL, const Cons<T>& UR, const Cons<T>& FL,
                                            const Cons<T>& FR, T SL, T SR) {
    if (SL >= T(0)) return FL;
    if (SR <= T(0)) return FR;
    const T den = xsub(SR, SL);
    if (Ar<T>::fabs_(den) < T(1.0e-14)) return c_avg(FL, FR);
    const T id = Ar<T>::rcp(den), ss = xmul(SL, SR);
    // (SR F_L - SL F_R + SL SR (U_R - U_L)) / (SR - SL)
    auto h = [&](T fl, T fr, T ul, T ur) { return xmul(xfma(ss, xsub(ur, ul), xfms(SL, fr, xmul(SR, fl))), id); };
    return Cons<T>{h(FL.r, FR.r, UL.r, UR.r), h(FL.mn, FR.mn, UL.mn, UR.mn), h(FL.mt, FR.mt, UL.mt, UR.mt),
                   h(FL.e, FR.e, UL.e, UR.e)};
}

// head/riemann.hpp:87-129 (Davis wave speeds; central average for
// non-physical input)
template <class T>
__device__ __forceinline__ Cons<T> hll_flux(const Cons<T>& UL, const Prim<T>& VL, const Cons<T>& UR,
                                            const Prim<T>& VR) {
    const Cons<T> FL = flux(UL, VL), FR = flux(UR, VR);
    if (!physical_riemann(VL) || !physical_riemann(VR)) return c_avg(FL, FR);
    const T aL = sound_speed(VL), aR = sound_speed(VR);
    const T SL = Ar<T>::fmin_(xsub(VL.un, aL), xsub(VR.un, aR));
    const T SR = Ar<T>::fmax_(xadd(VL.un, aL), xadd(VR.un, aR));
    return hll_from(UL, UR, FL, FR, SL, SR);
}

// head/riemann.hpp:135-271
template <class T>
__device__ __forceinline__ Cons<T> hllc_flux(const Cons<T>& UL, const Prim<T>& VL,
                                             const Cons<T>& UR, const Prim<T>& VR) {
    const Cons<T> FL = flux(UL, VL), FR = flux(UR, VR);
    // non-physical input: hll_flux, which returns the central average
    if (!physical_riemann(VL) || !physical_riemann(VR)) return c_avg(FL, FR);
    const T aL = sound_speed(VL), aR = sound_speed(VR);
    const T unL = VL.un, unR = VR.un;
    const T SL = Ar<T>::fmin_(xsub(unL, aL), xsub(unR, aR));
    const T SR = Ar<T>::fmax_(xadd(unL, aL), xadd(unR, aR));
    if (SL >= T(0)) return FL;
    if (SR <= T(0)) return FR;
    const T qL = xmul(VL.r, xsub(SL, unL)), qR = xmul(VR.r, xsub(SR, unR));
    const T numerator = xfms(qR, unR, xfma(qL, unL, xsub(VR.p, VL.p)));
    const T denominator = xsub(qL, qR);
    const T Sstar = xmul(numerator, Ar<T>::rcp(denominator));
    if (Ar<T>::fabs_(denominator) < T(1.0e-14) || !Ar<T>::finite(Sstar))
        return hll_from(UL, UR, FL, FR, SL, SR);
    // Upwind side of the contact: one star state, selected without branching.
    const bool left = Sstar >= T(0);
    const Cons<T> U = left ? UL : UR;
    const Cons<T> F = left ? FL : FR;
    const T rho = left ? VL.r : VR.r;
    const T p = left ? VL.p : VR.p;
    const T un = left ? unL : unR;
    const T ut = left ? VL.ut : VR.ut;
    const T irho = left ? VL.ir : VR.ir;
    const T S = left ? SL : SR;
    // hllc_star_state (head/riemann.hpp:135-186): falls back to U itself
    const T dS = xsub(S, Sstar);
    const T q = xmul(rho, xsub(S, un));
    const T rho_star = xmul(q, Ar<T>::rcp(dS));
    // E* = rho* (E/rho + (S* - u)(S* + p/q))
    const T E_star = xmul(rho_star, xfma(U.e, irho, xmul(xsub(Sstar, un), xfma(p, Ar<T>::rcp(q), Sstar))));
    const bool ok = !(Ar<T>::fabs_(dS) < T(1.0e-14)) && Ar<T>::finite(rho_star) && rho_star > T(0) &&
                    Ar<T>::finite(E_star);
    const Cons<T> Us = ok ? Cons<T>{rho_star, xmul(rho_star, Sstar), xmul(rho_star, ut), E_star} : U;
    return Cons<T>{xfma(S, xsub(Us.r, U.r), F.r), xfma(S, xsub(Us.mn, U.mn), F.mn), xfma(S, xsub(Us.mt, U.mt), F.mt),
                   xfma(S, xsub(Us.e, U.e), F.e)};
}

// head/riemann.hpp:284-325 (local-alpha FORCE)
template <class T>
__device__ __forceinline__ Cons<T> force_flux(const Cons<T>& UL, const Prim<T>& VL,
                                              const Cons<T>& UR, const Prim<T>& VR) {
    const Cons<T> FL = flux(UL, VL), FR = flux(UR, VR);
    const Cons<T> Fc = c_avg(FL, FR);
    if (!physical_riemann(VL) || !physical_riemann(VR)) return Fc;   // hll_flux -> central average
    const T aL = sound_speed(VL), aR = sound_speed(VR);
    const T alpha = Ar<T>::fmax_(xadd(Ar<T>::fabs_(VL.un), aL), xadd(Ar<T>::fabs_(VR.un), aR));
    if (!Ar<T>::finite(alpha) || alpha <= T(1.0e-14)) return Fc;
    const T ha = xmul(T(0.5), alpha);
    const T hia = xmul(T(0.5), Ar<T>::rcp(alpha));
    const Cons<T> Flf{xfms(ha, xsub(UR.r, UL.r), Fc.r), xfms(ha, xsub(UR.mn, UL.mn), Fc.mn),
                      xfms(ha, xsub(UR.mt, UL.mt), Fc.mt), xfms(ha, xsub(UR.e, UL.e), Fc.e)};
    const Cons<T> Ua = c_avg(UL, UR);
    const Cons<T> Uri{xfms(hia, xsub(FR.r, FL.r), Ua.r), xfms(hia, xsub(FR.mn, FL.mn), Ua.mn),
                      xfms(hia, xsub(FR.mt, FL.mt), Ua.mt), xfms(hia, xsub(FR.e, FL.e), Ua.e)};
    const Prim<T> Vri = cons_to_prim(Uri);
    if (!physical_riemann(Vri)) return Flf;
    return c_avg(Flf, flux(Uri, Vri));
}

// ---- exact solver (head/riemann.hpp:331-644), Newton always in FP64 ------
struct PrimD { double r, un, ut, p, a; };

// With gamma = 1.4 every power the exact solver takes of a pressure ratio is
// a multiple of 1/7: (g-1)/(2g) = 1/7, -(g+1)/(2g) = -6/7, 1/g = 5/7,
// 2/(g-1) = 5 and 2g/(g-1) = 7.  So one reciprocal seventh root w = r^(-1/7)
// and integer powers replace every pow(): r^(1/7) = r w^6, r^(-6/7) = w^6,
// r^(5/7) = (r^(1/7))^5.  (The reference's FP64 exponents differ from these
// by 1-2 ulp, which moves a power by under 1e-15 relative.)
static_assert(kGammaD == 1.4, "the seventh-root forms of the exact solver assume gamma = 1.4");
template <class T> __device__ __forceinline__ T rroot7(T r);
template <> __device__ __forceinline__ float rroot7<float>(float r) { return powf(r, -1.0f / 7.0f); }
// FP64: Newton's iteration for w^-7 = r in its division-free form
// w <- w (8 - r w^7) / 7 (relative error e -> -4 e^2), seeded with the FP32
// power (e ~ 3e-7): two steps reach full FP64 precision (a few ulp).
// Outside the FP32 normal range of the seed, pow().
template <> __device__ __forceinline__ double rroot7<double>(double r) {
    if (r == 1.0) return 1.0;                 // uniform states: p* equals the side's pressure
    if (!(r >= 1.0e-30 && r <= 1.0e30)) return pow(r, -1.0 / 7.0);
    double w = (double)powf((float)r, -1.0f / 7.0f);
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const double w2 = w * w, w3 = w2 * w, w7 = w3 * w3 * w;
        w = w * (8.0 - r * w7) * (1.0 / 7.0);
    }
    return w;
}
template <class T> __device__ __forceinline__ T pow5(T x) {
    const T x2 = x * x;
    return x2 * x2 * x;
}

// head/riemann.hpp:331-359.  The shock branch divides by p + B once; at
// p = pK the rarefaction branch is f = 0, fd = 1/(rho_K a_K) exactly (the
// reference's pow(1, e) is 1), taken without the root.
__device__ __forceinline__ void exact_pressure_function(double p, double rK, double pK, double aK,
                                                        double& f, double& fd) {
    if (p > pK) {
        const double A = 2.0 / ((kGammaD + 1.0) * rK);
        const double B = (kGammaD - 1.0) / (kGammaD + 1.0) * pK;
        const double ipb = 1.0 / (p + B);
        const double q = sqrt(A * ipb);
        f = (p - pK) * q;
        fd = q * (1.0 - 0.5 * (p - pK) * ipb);
    } else if (p == pK) {
        f = 0.0;
        fd = 1.0 / (rK * aK);
    } else {
        const double pratio = p / pK;
        const double w = rroot7(pratio), w2 = w * w, w6 = w2 * w2 * w2;   // pratio^(-1/7), ^(-6/7)
        f = 2.0 * aK / (kGammaD - 1.0) * (pratio * w6 - 1.0);
        fd = (1.0 / (rK * aK)) * w6;
    }
}

// head/riemann.hpp:361-443 (PVRS guess, <= 20 Newton steps, halving guard)
static __device__ __noinline__ bool exact_star(const PrimD& L, const PrimD& R, double& p_star,
                                        double& u_star) {
    const double pv = 0.5 * (L.p + R.p) - 0.125 * (R.un - L.un) * (L.r + R.r) * (L.a + R.a);
    p_star = fmax(1.0e-12, pv);
    for (int iter = 0; iter < 20; ++iter) {
        double fL, fR, dL, dR;
        exact_pressure_function(p_star, L.r, L.p, L.a, fL, dL);
        exact_pressure_function(p_star, R.r, R.p, R.a, fR, dR);
        const double f = fL + fR + (R.un - L.un);
        const double fd = dL + dR;
        if (fabs(fd) < 1.0e-14) return false;
        const double p_old = p_star;
        p_star = p_old - f / fd;
        if (!(fabs(p_star) < INFINITY) || p_star <= 0.0) p_star = 0.5 * p_old;
        // |dp| / (mean p + 1e-14) < 1e-8, as a product (the mean is positive)
        if (fabs(p_star - p_old) < 1.0e-8 * (0.5 * (p_star + p_old) + 1.0e-14)) break;
    }
    if (!(fabs(p_star) < INFINITY) || p_star <= 0.0) return false;
    double fL, fR, dL, dR;
    exact_pressure_function(p_star, L.r, L.p, L.a, fL, dL);
    exact_pressure_function(p_star, R.r, R.p, R.a, fR, dR);
    u_star = 0.5 * (L.un + R.un + fR - fL);
    return fabs(u_star) < INFINITY;
}

// The FP32 form's p* and u*: Newton's iteration of exact_star in FP32 to a
// relative step of 1e-5, then one FP64 Newton step from that root, with u*
// from the FP64 pressure functions linearised there.  The FP32 root is good
// to about 1e-6 relative (the sum fL + fR + du cancels in FP32), and the
// FP64 step is accepted only when it is at most 1e-5 of p*, so p* lands
// within 1e-10 of the FP64 iteration's own root (4e-11 at most over 262k
// random problems, 1e-12 typically) and u* closer: well inside the FP32
// rounding of both.  Two FP64 pressure function evaluations
// per face replace about ten.  Any case off this route (a non-positive or
// non-finite iterate, no convergence within 12 steps, f' below 1e-14, an
// FP64 step above 1e-5 of p*) runs the FP64 iteration.
struct StarD { double p, u; bool ok; };

struct SideF {   // one side's constants for the FP32 pressure function
    float r, p, a, A, B, ip, iz;   // A, B of the shock branch, 1/p, 1/(rho a)
};
__device__ __forceinline__ SideF side_f(float r, float p, float a) {
    const float g = gam<float>();
    return SideF{r, p, a, (2.0f / (g + 1.0f)) * Ar<float>::rcp(r), ((g - 1.0f) / (g + 1.0f)) * p,
                 Ar<float>::rcp(p), Ar<float>::rcp(r * a)};
}
__device__ __forceinline__ void exact_pressure_function(float p, const SideF& K, float& f, float& fd) {
    if (p > K.p) {
        const float ipb = Ar<float>::rcp(p + K.B);
        const float q = Ar<float>::sqrt_(K.A * ipb);
        f = (p - K.p) * q;
        fd = q * (1.0f - 0.5f * (p - K.p) * ipb);
    } else if (p == K.p) {
        f = 0.0f;
        fd = K.iz;
    } else {
        // z - 1 = (p/pK)^(1/7) - 1 from p - pK directly: accurate where p is
        // near pK and the difference z - 1 would cancel
        const float d = (p - K.p) * K.ip;                       // p/pK - 1
        const float zm1 = expm1f(log1pf(d) * (1.0f / 7.0f));
        f = (2.0f / (gam<float>() - 1.0f)) * K.a * zm1;
        fd = K.iz * (1.0f + zm1) * Ar<float>::rcp(1.0f + d);   // (p/pK)^(-6/7) / (rho a)
    }
}

// Scalar arguments: a reference to the caller's face states would make the
// caller keep them in local memory at every face.
static __device__ __noinline__ StarD exact_star_mixed(float rL, float uL, float pL, float aL, float rR, float uR,
                                                      float pR, float aR) {
    const SideF FL = side_f(rL, pL, aL), FR = side_f(rR, pR, aR);
    const float du = uR - uL;
    float p = fmaxf(1.0e-12f, 0.5f * (pL + pR) - 0.125f * du * (rL + rR) * (aL + aR));
    bool conv = false;
    for (int iter = 0; iter < 12; ++iter) {
        float fL, fR, dL, dR;
        exact_pressure_function(p, FL, fL, dL);
        exact_pressure_function(p, FR, fR, dR);
        const float pn = p - (fL + fR + du) * Ar<float>::rcp(dL + dR);
        if (!(pn > 0.0f && pn < INFINITY)) break;
        conv = fabsf(pn - p) < 1.0e-5f * (0.5f * (pn + p));
        p = pn;
        if (conv) break;
    }
    StarD st{0.0, 0.0, false};
    if (conv) {
        const double p0 = p;
        double fL, fR, dL, dR;
        exact_pressure_function(p0, rL, pL, aL, fL, dL);
        exact_pressure_function(p0, rR, pR, aR, fR, dR);
        const double fd = dL + dR;
        const double dp = -(fL + fR + ((double)uR - (double)uL)) / fd;
        // |f''| p / (2 f') is below 1 on both branches, so a step of at most
        // 1e-5 p0 leaves p0 + dp within 1e-10 of the root
        if (!(fabs(fd) < 1.0e-14) && fabs(dp) <= 1.0e-5 * p0) {
            st.p = p0 + dp;
            st.u = 0.5 * ((double)uL + (double)uR + (fR + dR * dp) - (fL + dL * dp));
            st.ok = fabs(st.u) < INFINITY;
            if (st.ok) return st;
        }
    }
    const PrimD L{(double)rL, (double)uL, 0.0, (double)pL, (double)aL};
    const PrimD R{(double)rR, (double)uR, 0.0, (double)pR, (double)aR};
    st.ok = exact_star(L, R, st.p, st.u);
    return st;
}

// head/riemann.hpp:445-591 sampled at xi = 0.  sgn = +1 samples the left
// wave family, -1 the right one (mirror image: un -> -un).
template <class T>
__device__ __forceinline__ void exact_sample(const Prim<T>& V, T a, T p_star, T u_star, T sgn,
                                             T& rho, T& un, T& p) {
    const T g = gam<T>();
    const T unK = sgn * V.un;     // mirrored normal velocity
    const T us = sgn * u_star;
    rho = V.r; un = unK; p = V.p;
    if (p_star > V.p) {
        const T pr = p_star / V.p;
        const T S = unK - a * Ar<T>::sqrt_((g + T(1)) / (T(2) * g) * pr + (g - T(1)) / (T(2) * g));
        if (!(T(0) <= S)) {
            const T k = (g - T(1)) / (g + T(1));
            rho = V.r * ((pr + k) / (k * pr + T(1)));
            un = us;
            p = p_star;
        }
    } else {
        const T pr = p_star / V.p;
        const T w = rroot7(pr), w2 = w * w;
        const T z = pr * (w2 * w2 * w2);                      // pr^(1/7) = pr^((g-1)/(2g))
        const T a_star = a * z;
        const T SH = unK - a;
        const T ST = us - a_star;
        if (T(0) <= SH) {
        } else if (T(0) >= ST) {
            rho = V.r * pow5(z);                              // pr^(5/7) = pr^(1/g)
            un = us;
            p = p_star;
        } else {
            const T af = T(2) / (g + T(1)) * (a + T(0.5) * (g - T(1)) * unK);
            un = T(2) / (g + T(1)) * (a + T(0.5) * (g - T(1)) * unK);
            const T ar = af / a;
            const T ar5 = pow5(ar);                           // ar^(2/(g-1))
            rho = V.r * ar5;
            p = V.p * (ar5 * (ar * ar));                      // ar^(2g/(g-1))
        }
    }
    un = sgn * un;
}

__device__ __forceinline__ bool same_bits(float a, float b) { return __float_as_uint(a) == __float_as_uint(b); }
__device__ __forceinline__ bool same_bits(double a, double b) {
    return __double_as_longlong(a) == __double_as_longlong(b);
}

// Identical left and right states -- every face of a uniform region, where
// both face states equal the cell state.  There exact_star and exact_sample
// compute, step by step: the PVRS guess p* = p, f(p*) = 0 (the p = p_K
// branch), so Newton stops at once with u* = u, and the sample returns the
// state itself (u = -0 comes back as +0).  The caller takes (rho, u, p)
// directly.  In IEEE arithmetic these are the full route's sampled bits
// (checked on 10^6 random states in FP64 and FP32).  In the FP32 form the
// full route's fast division can leave p*/p an ulp away from 1, which the
// direct route avoids.  The test excludes the cases where the full path
// takes another route: a PVRS guess below the 1e-12 floor, and f' below
// 1e-14.
template <class T> __device__ __forceinline__ bool exact_uniform(const Prim<T>& VL, const Prim<T>& VR, T aL) {
    if (!(same_bits(VL.r, VR.r) && same_bits(VL.un, VR.un) && same_bits(VL.ut, VR.ut) && same_bits(VL.p, VR.p)))
        return false;
    const double r = VL.r, u = VL.un, p = VL.p, a = aL;
    const double pv = 0.5 * (p + p) - 0.125 * (u - u) * (r + r) * (a + a);   // exact_star's PVRS guess
    if (!(pv == p) || !(p >= 1.0e-12)) return false;
    const double d = 1.0 / (r * a);                                        // f' of either side at p* = p
    return !(fabs(d + d) < 1.0e-14);
}

// FP32 states: the FP64 PVRS guess of two identical finite states is p
// exactly (every term is finite and u - u = 0), and the floor and f' tests
// become FP32 tests with a margin, so the direct route is taken only where
// the full route certainly passes them: p >= 1.0001e-12 implies
// p >= 1e-12, and rho a < 1.8e14 (rounded) implies 2 / (rho a) > 1e-14.
// This keeps the FP64 pipe, the exact solver's bottleneck, out of the test.
__device__ __forceinline__ bool exact_uniform(const Prim<float>& VL, const Prim<float>& VR, float aL) {
    if (!(same_bits(VL.r, VR.r) && same_bits(VL.un, VR.un) && same_bits(VL.ut, VR.ut) && same_bits(VL.p, VR.p)))
        return false;
    return VL.p >= 1.0001e-12f && VL.r * aL < 1.8e14f;
}

// head/riemann.hpp:601-644
template <class T>
__device__ __forceinline__ Cons<T> exact_flux(const Cons<T>& UL, const Prim<T>& VL,
                                              const Cons<T>& UR, const Prim<T>& VR) {
    if (!physical_riemann(VL) || !physical_riemann(VR)) return c_avg(flux(UL, VL), flux(UR, VR));
    const T aL = sound_speed(VL), aR = sound_speed(VR);
    T rho, un, p, ut;
    if (exact_uniform(VL, VR, aL)) {
        rho = VL.r;
        un = VL.un + T(0);   // the sampled u* of u = -0 is +0
        p = VL.p;
        ut = VL.ut;
    } else {
        double ps, us;
        if constexpr (sizeof(T) == 4) {
            const StarD st = exact_star_mixed(VL.r, VL.un, VL.p, aL, VR.r, VR.un, VR.p, aR);
            if (!st.ok) return hll_flux(UL, VL, UR, VR);
            ps = st.p;
            us = st.u;
        } else {
            const PrimD L{(double)VL.r, (double)VL.un, (double)VL.ut, (double)VL.p, (double)aL};
            const PrimD R{(double)VR.r, (double)VR.un, (double)VR.ut, (double)VR.p, (double)aR};
            if (!exact_star(L, R, ps, us)) return hll_flux(UL, VL, UR, VR);
        }
        const T p_star = T(ps), u_star = T(us);
        const bool left = us >= 0.0;
        if (left) exact_sample(VL, aL, p_star, u_star, T(1), rho, un, p);
        else exact_sample(VR, aR, p_star, u_star, T(-1), rho, un, p);
        ut = left ? VL.ut : VR.ut;
    }
    // make_conserved_from_normal_tangential (head/riemann.hpp:40-64)
    Cons<T> Us;
    Us.r = rho;
    Us.mn = rho * un;
    Us.mt = rho * ut;
    Us.e = p * inv_gm1<T>() + T(0.5) * rho * (un * un + ut * ut);
    const Prim<T> Vs = cons_to_prim(Us);
    if (!physical_riemann(Vs)) return hll_flux(UL, VL, UR, VR);
    return flux(Us, Vs);
}

template <int S, class T>
__device__ __forceinline__ Cons<T> riemann(const Cons<T>& UL, const Prim<T>& VL, const Cons<T>& UR,
                                           const Prim<T>& VR) {
    if constexpr (S == kHLLC) return hllc_flux(UL, VL, UR, VR);
    else if constexpr (S == kExact) return exact_flux(UL, VL, UR, VR);
    else if constexpr (S == kFORCE) return force_flux(UL, VL, UR, VR);
    else return hll_flux(UL, VL, UR, VR);
}

// ---------------------------------------------------------------------------
// src/cpu/solver_cpu.cpp:22-99  minmod-limited MUSCL-Hancock reconstruction
// ---------------------------------------------------------------------------
// minmod(a, b): 0 when a*b <= 0, else the argument of smaller magnitude
// (src/cpu/solver_cpu.cpp:22-28); for same-sign arguments min(a,b) (a > 0)
// or max(a,b) (a < 0) equals copysign(min(|a|,|b|), a) exactly.
template <class T> __device__ __forceinline__ T minmod(T a, T b) {
    // = max(0, min(a, b)) + min(0, max(a, b)): both terms vanish for
    // arguments of opposite sign (or a zero), otherwise one of them is the
    // argument nearer zero.  (The reference's test a*b > 0 also rejects
    // same-sign pairs whose product underflows, below 1e-308 in FP64.)
    return Ar<T>::fmax_(T(0), Ar<T>::fmin_(a, b)) + Ar<T>::fmin_(T(0), Ar<T>::fmax_(a, b));
}
// FP64: the same selection on the integer pipes, off the narrow FP64 pipe.
// Equal sign bits and a smaller magnitude (the bit patterns without the
// sign order like the magnitudes) pick the argument; the value is that of
// the form above for every non-NaN pair, up to the sign of a zero result.
template <> __device__ __forceinline__ double minmod<double>(double a, double b) {
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    const unsigned long long ma = (unsigned long long)ia & 0x7fffffffffffffffull;
    const unsigned long long mb = (unsigned long long)ib & 0x7fffffffffffffffull;
    const long long r = ma < mb ? ia : ib;
    return (ia ^ ib) >= 0 ? __longlong_as_double(r) : 0.0;
}

// Face states of one cell: the half-step-evolved left/right boundary states
// and their primitives.
template <class T> struct Face { Cons<T> U; Prim<T> V; };

// Reconstruct cell c from its neighbours' primitives (m, c, p) with
// hl = dt/(2 dx).  Outputs the evolved left (L) and right (R) states.
template <class T>
__device__ __forceinline__ void reconstruct(const Prim<T>& Wm, const Prim<T>& Wc, const Prim<T>& Wp,
                                            T hl, Face<T>& L, Face<T>& R) {
    Prim<T> s;
    s.r = minmod(xsub(Wc.r, Wm.r), xsub(Wp.r, Wc.r));
    s.un = minmod(xsub(Wc.un, Wm.un), xsub(Wp.un, Wc.un));
    s.ut = minmod(xsub(Wc.ut, Wm.ut), xsub(Wp.ut, Wc.ut));
    s.p = minmod(xsub(Wc.p, Wm.p), xsub(Wp.p, Wc.p));
    const T h = T(0.5);
    Prim<T> WL{xfms(h, s.r, Wc.r), xfms(h, s.un, Wc.un), xfms(h, s.ut, Wc.ut), xfms(h, s.p, Wc.p), T(0)};
    Prim<T> WR{xfma(h, s.r, Wc.r), xfma(h, s.un, Wc.un), xfma(h, s.ut, Wc.ut), xfma(h, s.p, Wc.p), T(0)};
    if (!physical_recon(WL)) WL = Wc;
    if (!physical_recon(WR)) WR = Wc;
    const Cons<T> UL = prim_to_cons(WL), UR = prim_to_cons(WR);
    Prim<T> VUL, VUR;
    if constexpr (sizeof(T) == 8) {
        // FP64: the reference re-derives the primitives of the rebuilt
        // conserved states inside physical_flux; keep that round trip.
        VUL = cons_to_prim(UL);
        VUR = cons_to_prim(UR);
    } else {
        // FP32: use the primitives the states were built from.
        VUL = WL; VUL.ir = Ar<T>::rcp(WL.r);
        VUR = WR; VUR.ir = Ar<T>::rcp(WR.r);
    }
    const Cons<T> FL = flux(UL, VUL), FR = flux(UR, VUR);
    const Cons<T> d{xmul(hl, xsub(FR.r, FL.r)), xmul(hl, xsub(FR.mn, FL.mn)), xmul(hl, xsub(FR.mt, FL.mt)),
                    xmul(hl, xsub(FR.e, FL.e))};
    const Cons<T> cl{xsub(UL.r, d.r), xsub(UL.mn, d.mn), xsub(UL.mt, d.mt), xsub(UL.e, d.e)};
    const Cons<T> cr{xsub(UR.r, d.r), xsub(UR.mn, d.mn), xsub(UR.mt, d.mt), xsub(UR.e, d.e)};
    const Prim<T> Vcl = cons_to_prim(cl), Vcr = cons_to_prim(cr);
    const bool okL = physical_recon(Vcl), okR = physical_recon(Vcr);
    L.U = okL ? cl : UL;
    L.V = okL ? Vcl : VUL;
    R.U = okR ? cr : UR;
    R.V = okR ? Vcr : VUR;
}

// ---------------------------------------------------------------------------
// Fast path.  The common case of every branch above, computed straight-line
// with the arithmetic regrouped for fused multiply-adds; `slow` is set
// whenever any of the reference's fallback branches (or the FP32 form's FP64
// pressure island) could change the result, and such a lane recomputes the
// cell with the full functions above.  Regroupings used (exact in real
// arithmetic, rounding differs in the last bits):
//   kinetic energy   rho|u|^2/2 = (m_n u_n + m_t u_t)/2
//   pressure         p = (g-1) E - (g-1)/2 (m_n u_n + m_t u_t)
//   half step        U -/+ (dt/2dx)(F_R - F_L) as one FMA per component
//   HLLC star state  E* = [(S-u) E + (S*-u)(q S* + p)] / (S - S*), q = rho (S-u)
// ---------------------------------------------------------------------------
// Physicality tests of primitives that came out of c2p_fast.  They need no
// separate test of u_n and u_t: the pressure is E(g-1) - (g-1)/2 (m_n u_n +
// m_t u_t), so a non-finite momentum or velocity (u = m / rho with rho above
// the floor) makes p NaN or -inf, which fails p > floor, and NaN in rho or p
// fails the comparisons.  A state with rho or E = +inf passes; it can only
// come from a state that is already non-finite, whose step reports
// EU_ERR_NONPHYSICAL through the y-sweep's finiteness check of its outputs.
template <class T> __device__ __forceinline__ bool phys_above(const Prim<T>& V, T floor) {
    return (V.r > floor) & (V.p > floor);
}
// FP32: min(rho, p) > floor with a NaN-propagating min (PTX min.NaN) is the
// pair of tests above, NaN included, in one fewer instruction.
__device__ __forceinline__ float min_nan(float a, float b) {
    float d;
    asm("min.NaN.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
    return d;
}
template <> __device__ __forceinline__ bool phys_above<float>(const Prim<float>& V, float floor) {
    return min_nan(V.r, V.p) > floor;
}
// FP64: the same tests on the integer pipes (Ar<double>::gt).
template <> __device__ __forceinline__ bool phys_above<double>(const Prim<double>& V, double floor) {
    return Ar<double>::gt(V.r, floor) & Ar<double>::gt(V.p, floor);
}
// physical_recon, with the 1e-12 floors (src/cpu/solver_cpu.cpp:39-43)
template <class T> __device__ __forceinline__ bool phys_recon_fast(const Prim<T>& V) {
    return phys_above(V, T(kRhoFloorD));
}
// physical_riemann (head/riemann.hpp:74-81)
template <class T> __device__ __forceinline__ bool phys_riemann_fast(const Prim<T>& V) {
    return phys_above(V, T(0));
}
// A cell whose limited face states are physical for any minmod slope: with
// finite neighbours of non-negative rho and p, minmod keeps the face values
// of rho and p at or above half the centre value, so rho, p > 4e-12 leaves
// them above the 1e-12 floors (src/cpu/solver_cpu.cpp:83-87).
template <class T> __device__ __forceinline__ bool nice_cell(const Prim<T>& V) {
    return phys_above(V, T(4.0e-12));
}

// cons_to_prim of a cell state, with the rounding fixed by explicit fused
// multiply-adds so that the fast path and the full path (cell_full) give the
// same bits: a cell's primitives never depend on which path computed them,
// which keeps every output independent of where a line segment starts.
template <class T> __device__ __forceinline__ Prim<T> c2p_arith(const Cons<T>& U, T& t) {
    Prim<T> V;
    V.ir = Ar<T>::rcp(U.r);
    V.r = U.r;
    V.un = U.mn * V.ir;
    V.ut = U.mt * V.ir;
    t = Ar<T>::fma_(U.mt, V.ut, U.mn * V.un);          // twice the kinetic energy
    V.p = Ar<T>::fma_(T(-0.5 * kGm1D), t, gm1<T>() * U.e);
    return V;
}

// FP32: every operation written out with its rounding (round to nearest,
// subnormals flushed), so that the one-cell form below and the two-cell
// packed form (c2p_rows) give the same bits lane by lane: IEEE operations
// with one rounding mode are exact per lane whether issued alone or as an
// f32x2 pair.
__device__ __forceinline__ float mul_rn_ftz(float a, float b) {
    float d;
    asm("mul.rn.ftz.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
    return d;
}
__device__ __forceinline__ float fma_rn_ftz(float a, float b, float c) {
    float d;
    asm("fma.rn.ftz.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ unsigned long long pk2(float a, float b) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk2(unsigned long long v, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ unsigned long long mul2_rn_ftz(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("mul.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long fma2_rn_ftz(unsigned long long a, unsigned long long b,
                                                      unsigned long long c) {
    unsigned long long d;
    asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
template <> __device__ __forceinline__ Prim<float> c2p_arith<float>(const Cons<float>& U, float& t) {
    Prim<float> V;
    V.ir = Ar<float>::rcp(U.r);
    V.r = U.r;
    V.un = mul_rn_ftz(U.mn, V.ir);
    V.ut = mul_rn_ftz(U.mt, V.ir);
    t = fma_rn_ftz(U.mt, V.ut, mul_rn_ftz(U.mn, V.un));
    V.p = fma_rn_ftz(float(-0.5 * kGm1D), t, mul_rn_ftz(gm1<float>(), U.e));
    return V;
}

// cons_to_prim without the FP64 island; flags the states that need it.
template <class T> __device__ __forceinline__ Prim<T> c2p_fast(const Cons<T>& U, bool& slow) {
    T t;
    const Prim<T> V = c2p_arith(U, t);
    if constexpr (sizeof(T) == 4) slow |= t > U.e;     // kinetic > E/2: FP64 recovery
    return V;
}

// c2p_fast of two cells at once.  FP32: the two cells' operations as f32x2
// pairs (half the issued instructions), bit for bit the one-cell form.
template <class T>
__device__ __forceinline__ void c2p_rows(const Cons<T>& A, const Cons<T>& B, Prim<T>& WA, Prim<T>& WB, bool& sa,
                                         bool& sb) {
    WA = c2p_fast(A, sa);
    WB = c2p_fast(B, sb);
}
template <>
__device__ __forceinline__ void c2p_rows<float>(const Cons<float>& A, const Cons<float>& B, Prim<float>& WA,
                                                Prim<float>& WB, bool& sa, bool& sb) {
    WA.ir = Ar<float>::rcp(A.r);
    WB.ir = Ar<float>::rcp(B.r);
    WA.r = A.r;
    WB.r = B.r;
    const unsigned long long ir = pk2(WA.ir, WB.ir), mn = pk2(A.mn, B.mn), mt = pk2(A.mt, B.mt);
    const unsigned long long un = mul2_rn_ftz(mn, ir), ut = mul2_rn_ftz(mt, ir);
    const unsigned long long t = fma2_rn_ftz(mt, ut, mul2_rn_ftz(mn, un));
    const unsigned long long p = fma2_rn_ftz(pk2(float(-0.5 * kGm1D), float(-0.5 * kGm1D)), t,
                                         mul2_rn_ftz(pk2(gm1<float>(), gm1<float>()), pk2(A.e, B.e)));
    upk2(un, WA.un, WB.un);
    upk2(ut, WA.ut, WB.ut);
    upk2(p, WA.p, WB.p);
    float ta, tb;
    upk2(t, ta, tb);
    sa |= ta > A.e;     // kinetic > E/2: FP64 recovery (c2p_fast)
    sb |= tb > B.e;
}

// The same primitives with the FP64 island applied (full path).
template <class T> __device__ __forceinline__ Prim<T> c2p_cell(const Cons<T>& U) {
    T t;
    Prim<T> V = c2p_arith(U, t);
    if constexpr (sizeof(T) == 4)
        if (t > U.e) V.p = pressure_fp64(U.r, U.mn, U.mt, U.e);
    return V;
}

// Conserved state and normal flux of a face state given in primitives.
template <class T>
__device__ __forceinline__ void face_state(const Prim<T>& W, Cons<T>& U, Cons<T>& F) {
    U.r = W.r;
    U.mn = W.r * W.un;
    U.mt = W.r * W.ut;
    U.e = W.p * inv_gm1<T>() + T(0.5) * (U.mt * W.ut + U.mn * W.un);
    F.r = U.mn;
    F.mn = U.mn * W.un + W.p;
    F.mt = U.mt * W.un;
    F.e = (U.e + W.p) * W.un;
}

// Reconstruct the centre cell c of (c-1, c, c+1) and evolve its face states
// by half a step.  The left difference dm = W(c) - W(c-1) is given (a
// marching line carries it from the previous cell, whose right difference
// it is) and the right difference dp = W(c+1) - W(c) is returned.  `nice`
// must say that all three cells pass nice_cell().
// (reconstruct_fast_1: this form for every precision; reconstruct_fast: the
// same, with the FP32 specialisation below that pairs the two faces.)
template <class T>
__device__ __forceinline__ void reconstruct_fast_1(const Prim<T>& dm, const Prim<T>& Wc, const Prim<T>& Wp, T hl,
                                                   bool nice, Face<T>& L, Face<T>& R, bool& slow, Prim<T>& dp) {
    dp = Prim<T>{Wp.r - Wc.r, Wp.un - Wc.un, Wp.ut - Wc.ut, Wp.p - Wc.p, T(0)};
    Prim<T> s;
    s.r = minmod(dm.r, dp.r);
    s.un = minmod(dm.un, dp.un);
    s.ut = minmod(dm.ut, dp.ut);
    s.p = minmod(dm.p, dp.p);
    const Prim<T> WL{Wc.r - T(0.5) * s.r, Wc.un - T(0.5) * s.un, Wc.ut - T(0.5) * s.ut, Wc.p - T(0.5) * s.p, T(0)};
    const Prim<T> WR{Wc.r + T(0.5) * s.r, Wc.un + T(0.5) * s.un, Wc.ut + T(0.5) * s.ut, Wc.p + T(0.5) * s.p, T(0)};
    Cons<T> UL, FL, UR, FR;
    face_state(WL, UL, FL);
    face_state(WR, UR, FR);
    const T dr = FR.r - FL.r, dmn = FR.mn - FL.mn, dmt = FR.mt - FL.mt, de = FR.e - FL.e;
    L.U = Cons<T>{UL.r - hl * dr, UL.mn - hl * dmn, UL.mt - hl * dmt, UL.e - hl * de};
    R.U = Cons<T>{UR.r - hl * dr, UR.mn - hl * dmn, UR.mt - hl * dmt, UR.e - hl * de};
    L.V = c2p_fast(L.U, slow);
    R.V = c2p_fast(R.U, slow);
    slow |= !(nice && phys_recon_fast(L.V) && phys_recon_fast(R.V));
}
template <class T>
__device__ __forceinline__ void reconstruct_fast(const Prim<T>& dm, const Prim<T>& Wc, const Prim<T>& Wp, T hl,
                                                 bool nice, Face<T>& L, Face<T>& R, bool& slow, Prim<T>& dp) {
    reconstruct_fast_1(dm, Wc, Wp, hl, nice, L, R, slow, dp);
}

// FP32: the same reconstruction with the left and right face states held as
// (left, right) pairs of one 64-bit register pair, so that every operation
// the two faces share -- their conserved states and fluxes, and the
// primitives of the evolved states -- is one packed instruction
// (fma/mul/add.rn.f32x2, sm_100 and later) instead of two.  Per cell that is
// 15 fewer issued instructions in a kernel bound by instruction issue.  The
// limiter, the flux differences and the half step stay scalar (their
// operands are a half of a pair or a value both faces share).
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 f2s(float a) { return make_float2(a, a); }

template <>
__device__ __forceinline__ void reconstruct_fast<float>(const Prim<float>& dm, const Prim<float>& Wc,
                                                          const Prim<float>& Wp, float hl, bool nice, Face<float>& L,
                                                          Face<float>& R, bool& slow, Prim<float>& dp) {
    dp = Prim<float>{Wp.r - Wc.r, Wp.un - Wc.un, Wp.ut - Wc.ut, Wp.p - Wc.p, 0.0f};
    const float sr = minmod(dm.r, dp.r), sun = minmod(dm.un, dp.un);
    const float sut = minmod(dm.ut, dp.ut), sp = minmod(dm.p, dp.p);
    // face primitives (left, right) = centre -/+ slope / 2
    const float2 r = f2(Wc.r - 0.5f * sr, Wc.r + 0.5f * sr);
    const float2 un = f2(Wc.un - 0.5f * sun, Wc.un + 0.5f * sun);
    const float2 ut = f2(Wc.ut - 0.5f * sut, Wc.ut + 0.5f * sut);
    const float2 p = f2(Wc.p - 0.5f * sp, Wc.p + 0.5f * sp);
    // conserved states and normal fluxes of both faces
    const float2 mn = __fmul2_rn(r, un), mt = __fmul2_rn(r, ut);
    const float2 kin2 = __ffma2_rn(mt, ut, __fmul2_rn(mn, un));            // twice the kinetic energy
    const float2 e = __ffma2_rn(f2s(0.5f), kin2, __fmul2_rn(p, f2s(inv_gm1<float>())));
    const float2 fmn = __ffma2_rn(mn, un, p);
    const float2 fmt = __fmul2_rn(mt, un);
    const float2 fe = __fmul2_rn(__fadd2_rn(e, p), un);
    // half step, both faces by the same flux difference
    const float dr = mn.y - mn.x, dmn = fmn.y - fmn.x, dmt = fmt.y - fmt.x, de = fe.y - fe.x;
    const float2 cr = f2(r.x - hl * dr, r.y - hl * dr);
    const float2 cmn = f2(mn.x - hl * dmn, mn.y - hl * dmn);
    const float2 cmt = f2(mt.x - hl * dmt, mt.y - hl * dmt);
    const float2 ce = f2(e.x - hl * de, e.y - hl * de);
    // primitives of the evolved states (c2p_arith on both at once)
    const float2 ir = f2(Ar<float>::rcp(cr.x), Ar<float>::rcp(cr.y));
    const float2 vun = __fmul2_rn(cmn, ir), vut = __fmul2_rn(cmt, ir);
    const float2 t = __ffma2_rn(cmt, vut, __fmul2_rn(cmn, vun));
    const float2 vp = __ffma2_rn(f2s(float(-0.5 * kGm1D)), t, __fmul2_rn(f2s(gm1<float>()), ce));
    L.U = Cons<float>{cr.x, cmn.x, cmt.x, ce.x};
    R.U = Cons<float>{cr.y, cmn.y, cmt.y, ce.y};
    L.V = Prim<float>{cr.x, vun.x, vut.x, vp.x, ir.x};
    R.V = Prim<float>{cr.y, vun.y, vut.y, vp.y, ir.y};
    slow |= (t.x > ce.x) | (t.y > ce.y);          // FP64 pressure island (c2p_fast)
    // phys_recon_fast(L.V) && phys_recon_fast(R.V) as one NaN-propagating min
    slow |= !(nice && min_nan(min_nan(cr.x, vp.x), min_nan(cr.y, vp.y)) > float(kRhoFloorD));
}

template <class T> __device__ __forceinline__ Cons<T> nflux(const Cons<T>& U, const Prim<T>& V) {
    return Cons<T>{U.mn, U.mn * V.un + V.p, U.mt * V.un, (U.e + V.p) * V.un};
}

// Riemann fluxes for physical inputs (the face states of reconstruct_fast).
template <class T>
__device__ __forceinline__ Cons<T> hll_fast(const Cons<T>& UL, const Prim<T>& VL, const Cons<T>& UR,
                                            const Prim<T>& VR, bool& slow) {
    const Cons<T> FL = nflux(UL, VL), FR = nflux(UR, VR);
    const T aL = sound_speed(VL), aR = sound_speed(VR);
    const T SL = Ar<T>::fmin_(VL.un - aL, VR.un - aR);
    const T SR = Ar<T>::fmax_(VL.un + aL, VR.un + aR);
    const T den = SR - SL;
    const T id = Ar<T>::rcp(den), ss = SL * SR;
    const Cons<T> Fh{(SR * FL.r - SL * FR.r + ss * (UR.r - UL.r)) * id,
                     (SR * FL.mn - SL * FR.mn + ss * (UR.mn - UL.mn)) * id,
                     (SR * FL.mt - SL * FR.mt + ss * (UR.mt - UL.mt)) * id,
                     (SR * FL.e - SL * FR.e + ss * (UR.e - UL.e)) * id};
    const bool upL = SL >= T(0), upR = SR <= T(0);
    slow |= !(upL || upR || !(Ar<T>::fabs_(den) < T(1.0e-14)));
    return upL ? FL : (upR ? FR : Fh);
}

// HLLC for physical inputs.  The upwind cases SL >= 0 / SR <= 0 return the
// flux of the upwind side; that side is also the side of the contact
// (left iff S* >= 0) whenever the star state is valid (rho* > 0 puts S*
// strictly inside the fan), so one flux F_K of the side K = left/right of S*
// serves all three cases: F = F_K + S_eff (U*_K - U_K), S_eff = 0 upwind.
// Any inconsistency (S* outside the fan, tiny denominators, non-finite
// star state) flags the lane for the full path.
template <class T>
__device__ __forceinline__ Cons<T> hllc_fast(const Cons<T>& UL, const Prim<T>& VL, const Cons<T>& UR,
                                             const Prim<T>& VR, bool& slow) {
    const T aL = sound_speed(VL), aR = sound_speed(VR);
    const T unL = VL.un, unR = VR.un;
    const T SL = Ar<T>::fmin_(unL - aL, unR - aR);
    const T SR = Ar<T>::fmax_(unL + aL, unR + aR);
    const T sL = SL - unL, sR = SR - unR;
    const T qL = VL.r * sL, qR = VR.r * sR;
    const T numerator = (VR.p - VL.p) + qL * unL - qR * unR;
    const T denominator = qL - qR;
    const T Sstar = numerator * Ar<T>::rcp(denominator);
    const bool left = Sstar >= T(0);
    const Cons<T> U = left ? UL : UR;
    const T p = left ? VL.p : VR.p;
    const T un = left ? unL : unR;
    const T ut = left ? VL.ut : VR.ut;
    const T S = left ? SL : SR;
    const T sK = left ? sL : sR;
    const T q = left ? qL : qR;
    const T dS = S - Sstar;
    const T idS = Ar<T>::rcp(dS);
    const T rho_star = q * idS;
    const T E_star = (sK * U.e + (Sstar - un) * (q * Sstar + p)) * idS;
    const bool upL = SL >= T(0), upR = SR <= T(0);
    const T Se = (upL || upR) ? T(0) : S;
    // !(|den| < 1e-14) && !(|dS| < 1e-14) as one test of the smaller
    // magnitude: fmin returns the other argument for one NaN, and a NaN
    // passes its own test, so the two forms agree for every input
    const bool ok = !(Ar<T>::fmin_(Ar<T>::fabs_(denominator), Ar<T>::fabs_(dS)) < T(1.0e-14)) &&
                    Ar<T>::fabs_(Sstar + rho_star + E_star) < T(INFINITY) && rho_star > T(0) &&
                    !(upL && !left) && !(upR && left);
    slow |= !ok;
    // the tangential momentum flux is u_t times the mass flux on either
    // side of the contact (rho u_n u_t upwind, rho* S* u_t in the star state)
    const T Fr = U.mn + Se * (rho_star - U.r);
    return Cons<T>{Fr, (U.mn * un + p) + Se * (rho_star * Sstar - U.mn), ut * Fr,
                   (U.e + p) * un + Se * (E_star - U.e)};
}

template <class T>
__device__ __forceinline__ Cons<T> force_fast(const Cons<T>& UL, const Prim<T>& VL, const Cons<T>& UR,
                                              const Prim<T>& VR, bool& slow) {
    const Cons<T> FL = nflux(UL, VL), FR = nflux(UR, VR);
    const Cons<T> Fc = c_avg(FL, FR);
    const T aL = sound_speed(VL), aR = sound_speed(VR);
    const T alpha = Ar<T>::fmax_(Ar<T>::fabs_(VL.un) + aL, Ar<T>::fabs_(VR.un) + aR);
    const T ha = T(0.5) * alpha;
    const T hia = T(0.5) * Ar<T>::rcp(alpha);
    const Cons<T> Flf{Fc.r - ha * (UR.r - UL.r), Fc.mn - ha * (UR.mn - UL.mn),
                      Fc.mt - ha * (UR.mt - UL.mt), Fc.e - ha * (UR.e - UL.e)};
    const Cons<T> Ua = c_avg(UL, UR);
    const Cons<T> Uri{Ua.r - hia * (FR.r - FL.r), Ua.mn - hia * (FR.mn - FL.mn),
                      Ua.mt - hia * (FR.mt - FL.mt), Ua.e - hia * (FR.e - FL.e)};
    const Prim<T> Vri = c2p_fast(Uri, slow);
    slow |= !(Ar<T>::finite(alpha) && alpha > T(1.0e-14) && phys_riemann_fast(Vri));
    return c_avg(Flf, nflux(Uri, Vri));
}

template <int S, class T>
__device__ __forceinline__ Cons<T> riemann_fast(const Cons<T>& UL, const Prim<T>& VL, const Cons<T>& UR,
                                                const Prim<T>& VR, bool& slow) {
    if constexpr (S == kHLLC) return hllc_fast(UL, VL, UR, VR, slow);
    else if constexpr (S == kFORCE) return force_fast(UL, VL, UR, VR, slow);
    else if constexpr (S == kHLL) return hll_fast(UL, VL, UR, VR, slow);
    else return exact_flux(UL, VL, UR, VR);   // the exact solver always takes its full path
}

// Largest signal speed max(|u|, |v|) + a of a conserved state (the CFL
// reduction, src/cpu/solver_cpu.cpp:295-300); NaN for a non-finite state.
template <class T> __device__ __forceinline__ T signal_speed_fast(const Cons<T>& U) {
    // head/physics.hpp:39-45 with p from (g-1) E - (g-1)/2 |m|^2 / rho
    const T ir = Ar<T>::rcp(U.r);
    const T t = U.mt * U.mt + U.mn * U.mn;
    const T p = gm1<T>() * U.e - T(0.5 * kGm1D) * (t * ir);
    const T a = Ar<T>::sqrt_(gam<T>() * p * ir);
    return Ar<T>::fmax_(Ar<T>::fabs_(U.mn), Ar<T>::fabs_(U.mt)) * ir + a;
}

// FP32 signal speed for the CFL reduction in lane form (lanes.cuh):
// max(|u_n|, |u_t|) + a = (max(|m_n|, |m_t|) + rho a) / rho with
// (rho a)^2 = gamma (gamma-1) (rho E - |m|^2/2), so the pressure needs no
// division.  NaN (or +inf) for a non-finite or negative-pressure state, as
// signal_speed_fast.  Every FP32 y-sweep pass takes this form, one cell
// (V = float) or two rows at a time (V = F2) with every rounding explicit,
// so that a cell's speed, and with it the step's dt, does not depend on
// which pass computed the cell.
template <class V> __device__ __forceinline__ V speed_v(const Cons<V>& U) {
    const V m2 = vfma(U.mt, U.mt, vmul(U.mn, U.mn));
    const V q = vfma(splat<V>(-0.5f), m2, vmul(U.e, U.r));
    const V ra = vsqrt(vmul(splat<V>(float(kGammaD * kGm1D)), q));
    return vmul(vadd(vmax(vabs(U.mn), vabs(U.mt)), ra), vrcp(U.r));
}
__device__ __forceinline__ float2 signal_speed_rows(const Cons<float>& A, const Cons<float>& B) {
    const F2 sp = speed_v(Cons<F2>{mk2(A.r, B.r), mk2(A.mn, B.mn), mk2(A.mt, B.mt), mk2(A.e, B.e)});
    return make_float2(lo(sp), hi(sp));
}

// Full-logic recomputation of one cell (out of line; taken only by lanes
// whose fast path flagged a fallback).
template <class T> struct CellOut {
    Prim<T> W;
    Face<T> L, R;
    Cons<T> F;
    bool r_phys;   // R.V is physical (the next cell's fast Riemann needs it)
};

// full = true: the cell's reconstruction flagged a fallback -- recompute
// its primitives, face states and flux with the full logic (W(c-2) is
// W(c-1) - dm).  full = false: only the face flagged one -- keep the
// fast-path primitives and face states (W, L, R) and recompute the flux.
template <class T, int S>
__device__ __noinline__ CellOut<T> cell_full(Cons<T> U, Prim<T> dm, Prim<T> Wm1, Face<T> Rp, T hl, bool full,
                                             Prim<T> W, Face<T> L, Face<T> R) {
    CellOut<T> o;
    if (full) {
        const Prim<T> Wm2{Wm1.r - dm.r, Wm1.un - dm.un, Wm1.ut - dm.ut, Wm1.p - dm.p, T(0)};   // W(c-2)
        o.W = c2p_cell(U);
        reconstruct(Wm2, Wm1, o.W, hl, o.L, o.R);
        o.r_phys = physical_riemann(o.R.V);
    } else {
        o.W = W;
        o.L = L;
        o.R = R;
        o.r_phys = true;
    }
    o.F = riemann<S>(Rp.U, Rp.V, o.L.U, o.L.V);
    return o;
}

// Largest signal speed max(|un|+a, |ut|+a) of a conserved state
// (src/cpu/solver_cpu.cpp:295-300); NaN for a non-finite state.
template <class T> __device__ __forceinline__ T max_signal_speed(const Cons<T>& U) {
    const Prim<T> V = cons_to_prim(U);
    const T a = sound_speed(V);
    const T sx = Ar<T>::fabs_(V.un) + a, sy = Ar<T>::fabs_(V.ut) + a;
    return (sx < sy) ? sy : sx;
}

}  // namespace eu
