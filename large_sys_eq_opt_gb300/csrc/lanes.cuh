// lanes.cuh -- FP32 arithmetic with every rounding written out, on one value
// (float) or on a pair of values held in one 64-bit register pair (F2: the
// f32x2 add/sub/mul/fma instructions of sm_100 and later).
//
// Each operation is one IEEE operation, rounded to nearest with subnormals
// flushed, issued through inline PTX so that the compiler neither fuses nor
// splits it.  An IEEE operation gives the same bits whether it runs alone or
// as one half of an f32x2 instruction, so code written once against these
// overloads computes, lane by lane, the same bits for V = float as for
// V = F2 (the y-sweep's CFL speeds: two rows at a time in the fast pass, one
// cell at a time in the fallback pass), and the same bits in every kernel it
// is compiled into (the full-logic path).
//
// One exception to "neither fuses": measured on sm_103a, ptxas fuses a
// mul.rn.f32x2 whose factor is a splat (the same value in both halves) into
// a following add/sub.rn.f32x2, whatever the rounding modifier or -fmad say;
// a general mul.rn.f32x2, and every scalar .rn operation, stay unfused.  So a
// packed product with a splat factor must not feed a packed add or subtract
// directly (it may feed an fma, a compare or a scalar operation).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace eu {

struct F2 { unsigned long long v; };   // (lo, hi) = (first, second) element
struct M2 { bool a, b; };              // per-element predicates of an F2 comparison

template <class V> struct MaskT;
template <> struct MaskT<float> { using type = bool; };
template <> struct MaskT<F2> { using type = M2; };
template <class V> using MaskOf = typename MaskT<V>::type;

__device__ __forceinline__ F2 mk2(float a, float b) {
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void sp2(F2 x, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x.v));
}
__device__ __forceinline__ float lo(F2 x) { float a, b; sp2(x, a, b); return a; }
__device__ __forceinline__ float hi(F2 x) { float a, b; sp2(x, a, b); return b; }

template <class V> __device__ __forceinline__ V splat(float c);
template <> __device__ __forceinline__ float splat<float>(float c) { return c; }
template <> __device__ __forceinline__ F2 splat<F2>(float c) { return mk2(c, c); }

// ---- one value ----
__device__ __forceinline__ float vadd(float a, float b) {
    float d;
    asm("add.rn.ftz.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
    return d;
}
__device__ __forceinline__ float vsub(float a, float b) {
    float d;
    asm("sub.rn.ftz.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
    return d;
}
__device__ __forceinline__ float vmul(float a, float b) {
    float d;
    asm("mul.rn.ftz.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
    return d;
}
__device__ __forceinline__ float vfma(float a, float b, float c) {
    float d;
    asm("fma.rn.ftz.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
// approximate reciprocal and square root (PTX rcp.approx / sqrt.approx)
__device__ __forceinline__ float vrcp(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float vsqrt(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float vmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float vmax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ float vabs(float a) { return fabsf(a); }
__device__ __forceinline__ bool vgt(float a, float b) { return a > b; }
__device__ __forceinline__ bool vge(float a, float b) { return a >= b; }
__device__ __forceinline__ bool vlt(float a, float b) { return a < b; }
__device__ __forceinline__ bool vle(float a, float b) { return a <= b; }
__device__ __forceinline__ float sel(bool m, float a, float b) { return m ? a : b; }
__device__ __forceinline__ bool m_and(bool a, bool b) { return a & b; }
__device__ __forceinline__ bool m_or(bool a, bool b) { return a | b; }
__device__ __forceinline__ bool m_not(bool a) { return !a; }

// ---- two values ----
__device__ __forceinline__ F2 vadd(F2 a, F2 b) {
    F2 d;
    asm("add.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ F2 vsub(F2 a, F2 b) {
    F2 d;
    asm("sub.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ F2 vmul(F2 a, F2 b) {   // see the splat rule above
    F2 d;
    asm("mul.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
    return d;
}
__device__ __forceinline__ F2 vfma(F2 a, F2 b, F2 c) {
    F2 d;
    asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(d.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return d;
}
// element-wise operations without an f32x2 form
#define EU_LANES_UNARY(name)                                  \
    __device__ __forceinline__ F2 name(F2 x) {                \
        float a, b;                                           \
        sp2(x, a, b);                                         \
        return mk2(name(a), name(b));                         \
    }
#define EU_LANES_BINARY(name)                                 \
    __device__ __forceinline__ F2 name(F2 x, F2 y) {          \
        float a, b, c, d;                                     \
        sp2(x, a, b);                                         \
        sp2(y, c, d);                                         \
        return mk2(name(a, c), name(b, d));                   \
    }
#define EU_LANES_CMP(name)                                    \
    __device__ __forceinline__ M2 name(F2 x, F2 y) {          \
        float a, b, c, d;                                     \
        sp2(x, a, b);                                         \
        sp2(y, c, d);                                         \
        return M2{name(a, c), name(b, d)};                    \
    }
EU_LANES_UNARY(vrcp)
EU_LANES_UNARY(vsqrt)
EU_LANES_UNARY(vabs)
EU_LANES_BINARY(vmin)
EU_LANES_BINARY(vmax)
EU_LANES_CMP(vgt)
EU_LANES_CMP(vge)
EU_LANES_CMP(vlt)
EU_LANES_CMP(vle)
#undef EU_LANES_UNARY
#undef EU_LANES_BINARY
#undef EU_LANES_CMP
__device__ __forceinline__ F2 sel(M2 m, F2 x, F2 y) {
    float a, b, c, d;
    sp2(x, a, b);
    sp2(y, c, d);
    return mk2(m.a ? a : c, m.b ? b : d);
}
__device__ __forceinline__ M2 m_and(M2 x, M2 y) { return M2{x.a && y.a, x.b && y.b}; }
__device__ __forceinline__ M2 m_or(M2 x, M2 y) { return M2{x.a || y.a, x.b || y.b}; }
__device__ __forceinline__ M2 m_not(M2 x) { return M2{!x.a, !x.b}; }

}  // namespace eu
