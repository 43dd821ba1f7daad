// sweeps.cuh -- the fused x- and y-sweep kernels of the MUSCL-Hancock split
// step (src/cpu/solver_cpu.cpp:400-499 restated for sm_103a).
//
// Data layout in HBM (SoA planes, 2-cell ghost frame):
//   state buffers S0/S1 : interior (i, j) at column i+kSOff (6), row j+2
//   Utmp                : interior (i, j) at column i+kTOff (8), row j+2
// The x-sweep finalises a cell two cells behind the newest one it reads; the
// two extra columns of Utmp put each output in the Utmp column equal to the
// S column of the newest input, and both offsets keep every box and every
// warp-wide row store on a 32-byte sector boundary.
//
// Execution model: every lane owns one grid line (a row in the x-sweep, a
// column in the y-sweep) and marches along it; the 5-cell stencil window
// (two primitive states, two conserved states, the last face state and the
// last face flux) slides through registers, so each cell is converted and
// reconstructed once and each face solved once, with no cross-lane traffic.
// Every warp is an independent unit with its own shared-memory stages and
// mbarriers: lane 0 streams the next boxes of all four field planes into
// shared memory with TMA (cp.async.bulk.tensor.3d) while the warp computes.
//   x-sweep : 32 rows per warp; boxes of 32 rows x 32 bytes, stored with the
//             32-byte swizzle so that 16-byte row reads are bank-conflict free.
//   y-sweep : 32 columns per warp; boxes of 36 columns x RY rows.  Its
//             epilogue reduces the maximum signal speed (warp shuffle max ->
//             one atomic per warp) and the last warp to finish computes the
//             next dt on the device.
#pragma once
#include "eu_internal.h"
#include "euler_numerics.cuh"
#include "tma_pipe.cuh"

namespace eu {

// ---------------------------------------------------------------------------
// The marching stencil window of one line
// ---------------------------------------------------------------------------
// push(U_c) takes the next cell c of the line and returns the updated cell
// c-2: cell c-1 is reconstructed from (c-2, c-1, c) and half-step evolved
// (src/cpu/solver_cpu.cpp:68-99), the face (c-2 | c-1) is solved
// (head/riemann.hpp:650-672) and cell c-2 is updated with its two face
// fluxes (src/cpu/solver_cpu.cpp:452-453, :489-490).
template <class T, int S> struct Line {
    Prim<T> dm, Wm1;    // W(c-1) - W(c-2), primitives of cell c-1 (1/rho unused)
    Cons<T> Um1, Um2;   // conserved states of cells c-1 and c-2
    Cons<T> Fm;         // flux F(c-5/2) through the left face of cell c-2
    Face<T> Rp;         // evolved right face state of cell c-2
    bool nice2, nice1;  // cells c-2, c-1 pass nice_cell()
    bool rp_phys;       // Rp is physical (always true when it came from the fast path)

    __device__ __forceinline__ void reset() {
        dm = Prim<T>{}; Wm1 = Prim<T>{}; Um1 = Cons<T>{}; Um2 = Cons<T>{}; Fm = Cons<T>{};
        Rp = Face<T>{};
        nice2 = nice1 = false;
        rp_phys = false;
    }

    // Start of a line at cell U0: the window as if U0 were repeated to the
    // left (zero slopes, faces equal to the cell).  Only the first outputs'
    // warm-up sees these values, and no output depends on them; they just
    // keep the first pushes from raising fallback flags on garbage.
    __device__ __forceinline__ void prime(const Cons<T>& U0) {
        bool isl = false;
        const Prim<T> W = c2p_fast(U0, isl);
        dm = Prim<T>{}; Wm1 = W;
        Um1 = U0;
        Um2 = U0;
        Fm = Cons<T>{};
        Rp.U = U0;
        Rp.V = W;
        nice2 = nice1 = nice_cell(W);
        rp_phys = phys_riemann_fast(W);
    }

    // The conservative update of cell c-2, U(c-2) - lam (F(c-3/2) - F(c-5/2))
    // (src/cpu/solver_cpu.cpp:452-453, :489-490), in the reference's order
    // of operations: equal fluxes leave a cell's state exactly as it was, so
    // a uniform region stays uniform to the last bit (the exact solver's
    // identical-states route depends on that).  Shifts the window's
    // conserved states on to cell c.
    __device__ __forceinline__ Cons<T> update(const Cons<T>& F, T lam, const Cons<T>& U) {
        Cons<T> N;
        if constexpr (sizeof(T) == 4) {
            const float nl = -lam;
            N = Cons<T>{vfma(nl, vsub(F.r, Fm.r), Um2.r), vfma(nl, vsub(F.mn, Fm.mn), Um2.mn),
                        vfma(nl, vsub(F.mt, Fm.mt), Um2.mt), vfma(nl, vsub(F.e, Fm.e), Um2.e)};
        } else {
            N = Cons<T>{Um2.r - lam * (F.r - Fm.r), Um2.mn - lam * (F.mn - Fm.mn), Um2.mt - lam * (F.mt - Fm.mt),
                        Um2.e - lam * (F.e - Fm.e)};
        }
        Fm = F;
        Um2 = Um1;
        Um1 = U;
        return N;
    }
    // SLOW = true: a cell flagged by its own reconstruction is recomputed in
    // full; a cell whose only flag is the face (a non-physical left face
    // state, a Riemann fallback) keeps its fast-path primitives and face
    // states and recomputes only the flux.
    // SLOW = false: the fast path only; the flags are returned (fi: the
    // cell's own FP64 pressure island, fc: its reconstruction, ff: its face)
    // and the caller redoes the work with SLOW = true when one matters.
    template <bool SLOW>
    __device__ __forceinline__ Cons<T> step(const Cons<T>& U, T hl, T lam, bool& fi, bool& fc, bool& ff) {
        bool isl = false;
        const Prim<T> W = c2p_fast(U, isl);
        return step_w<SLOW>(U, W, isl, hl, lam, fi, fc, ff);
    }
    // step() with the cell's c2p_fast primitives W and island flag isl given
    // (computed ahead, two cells at a time).
    template <bool SLOW>
    __device__ __forceinline__ Cons<T> step_w(const Cons<T>& U, Prim<T> W, bool isl, T hl, T lam, bool& fi,
                                              bool& fc, bool& ff) {
        bool slow_cell = false, slow_face = !rp_phys;
        const bool nice = nice_cell(W);
        Face<T> L, R;
        Prim<T> dp;
        if constexpr (S == kExact) reconstruct_fast_1(dm, Wm1, W, hl, nice && nice1 && nice2, L, R, slow_cell, dp);
        else reconstruct_fast(dm, Wm1, W, hl, nice && nice1 && nice2, L, R, slow_cell, dp);
        Cons<T> F = riemann_fast<S>(Rp.U, Rp.V, L.U, L.V, slow_face);
        bool r_phys = true;
        Prim<T> dnext = dp;   // W(c) - W(c-1) for the next cell
        if constexpr (SLOW) {
            slow_cell |= isl;
            if (__builtin_expect(slow_cell | slow_face, 0)) {
                // W(c-2) is rebuilt inside the out-of-line call (measured 1.2%
                // faster than building it here: same instruction count, the
                // call site holds fewer values live)
                const CellOut<T> o = cell_full<T, S>(U, dm, Wm1, Rp, hl, slow_cell, W, L, R);
                W = o.W; L = o.L; R = o.R; F = o.F;
                r_phys = o.r_phys;
                dnext = Prim<T>{W.r - Wm1.r, W.un - Wm1.un, W.ut - Wm1.ut, W.p - Wm1.p, T(0)};
            }
        } else {
            fi |= isl;
            fc |= slow_cell;
            ff |= slow_face;
        }
        const Cons<T> N = update(F, lam, U);
        dm = dnext;
        Wm1 = W;
        Rp = R;
        nice2 = nice1; nice1 = nice;
        rp_phys = r_phys;
        return N;
    }
    __device__ __forceinline__ Cons<T> push(const Cons<T>& U, T hl, T lam) {
        bool a = false, b = false, c = false;
        return step<true>(U, hl, lam, a, b, c);
    }
    // The fast path only, with the cell's primitives W given (c2p_fast of U,
    // computed ahead for two rows at a time) and one flag for every
    // fallback the push could need (the cell's FP64 pressure island included
    // by the caller); the y-sweep's fast pass, after warm4().  The previous
    // right face is then always a physical one from reconstruct_fast, so the
    // flag rp_phys carries for the full path is not needed here.
    __device__ __forceinline__ Cons<T> step_fast(const Cons<T>& U, const Prim<T>& W, T hl, T lam, bool& flag) {
        const bool nice = nice_cell(W);
        Face<T> L, R;
        Prim<T> dp;
        bool slow = false;
        reconstruct_fast(dm, Wm1, W, hl, nice && nice1 && nice2, L, R, slow, dp);
        const Cons<T> F = riemann_fast<S>(Rp.U, Rp.V, L.U, L.V, slow);
        flag |= slow;
        const Cons<T> N = update(F, lam, U);
        dm = dp;
        Wm1 = W;
        Rp = R;
        nice2 = nice1; nice1 = nice;
        return N;
    }
    // The four warm-up pushes of a line primed at row r0-2 (rows r0-2 .. r0+1,
    // primitives W = c2p_fast(U) given), doing only the work that reaches an
    // output: the first output (row r0, at the next push) needs the slopes
    // W(r0-1) - W(r0-2) and W(r0) - W(r0-1), the reconstructions of cells
    // r0-1 and r0 and the flux F(r0-1/2).  The reconstructions of cells r0-3
    // and r0-2 start from the primed copy, and the fluxes F(r0-7/2) ..
    // F(r0-3/2) and the updates of rows r0-4 .. r0-1 only feed outputs the
    // task does not store, so they are skipped together with their fallback
    // flags; the window then holds what four step_fast pushes leave in it.
    __device__ __forceinline__ void warm4(const Cons<T> (&U)[4], const Prim<T> (&W)[4], T hl, bool& flag) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const bool nice = nice_cell(W[q]);
            dm = Prim<T>{W[q].r - Wm1.r, W[q].un - Wm1.un, W[q].ut - Wm1.ut, W[q].p - Wm1.p, T(0)};
            Wm1 = W[q];
            Um2 = Um1;
            Um1 = U[q];
            nice2 = nice1; nice1 = nice;
        }
#pragma unroll
        for (int q = 2; q < 4; ++q) {
            const bool nice = nice_cell(W[q]);
            Face<T> L, R;
            Prim<T> dp;
            bool slow = false;
            reconstruct_fast(dm, Wm1, W[q], hl, nice && nice1 && nice2, L, R, slow, dp);
            if (q == 3) Fm = riemann_fast<S>(Rp.U, Rp.V, L.U, L.V, slow);   // F(r0-1/2)
            flag |= slow;
            dm = dp;
            Wm1 = W[q];
            Um2 = Um1;
            Um1 = U[q];
            Rp = R;
            nice2 = nice1; nice1 = nice;
        }
    }
};

// Vector loads/stores of VEC consecutive elements (16 B, 8 B or scalar).
template <class T, int V> __device__ __forceinline__ void ld_vec(const T* p, T (&o)[V]) {
    if constexpr (V == 1) {
        o[0] = p[0];
    } else if constexpr (sizeof(T) * V == 16) {
        if constexpr (sizeof(T) == 4) {
            const float4 x = *reinterpret_cast<const float4*>(p);
            o[0] = x.x; o[1] = x.y; o[2] = x.z; o[3] = x.w;
        } else {
            const double2 x = *reinterpret_cast<const double2*>(p);
            o[0] = x.x; o[1] = x.y;
        }
    } else if constexpr (sizeof(T) == 4 && V == 2) {
        const float2 x = *reinterpret_cast<const float2*>(p);
        o[0] = x.x; o[1] = x.y;
    } else {
#pragma unroll
        for (int v = 0; v < V; ++v) o[v] = p[v];
    }
}
template <class T, int V> __device__ __forceinline__ void st_vec(T* p, const T (&o)[V]) {
    if constexpr (V == 1) {
        p[0] = o[0];
    } else if constexpr (sizeof(T) * V == 16) {
        if constexpr (sizeof(T) == 4) {
            *reinterpret_cast<float4*>(p) = make_float4(o[0], o[1], o[2], o[3]);
        } else {
            *reinterpret_cast<double2*>(p) = make_double2(o[0], o[1]);
        }
    } else if constexpr (sizeof(T) == 4 && V == 2) {
        *reinterpret_cast<float2*>(p) = make_float2(o[0], o[1]);
    } else {
#pragma unroll
        for (int v = 0; v < V; ++v) p[v] = o[v];
    }
}

// Store VEC cells (fields in (r, mn, mt, e) order) to row `row`, starting at
// column `col`, into planes (p0..p3); only slots with mask bit set.
template <class T, int V>
__device__ __forceinline__ void store_cells(const Planes<T>& P, long long row, long long col,
                                            const Cons<T> (&N)[V], unsigned mask, int pmn, int pmt,
                                            bool negate_mt) {
    T* base = P.base + row * P.pitch + col;
    T r[V], mn[V], mt[V], en[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
        r[v] = N[v].r; mn[v] = N[v].mn; mt[v] = negate_mt ? -N[v].mt : N[v].mt; en[v] = N[v].e;
    }
    if (mask == (1u << V) - 1u) {
        st_vec<T, V>(base, r);
        st_vec<T, V>(base + pmn * P.plane, mn);
        st_vec<T, V>(base + pmt * P.plane, mt);
        st_vec<T, V>(base + 3 * P.plane, en);
    } else {
#pragma unroll
        for (int v = 0; v < V; ++v)
            if (mask & (1u << v)) {
                base[v] = r[v];
                base[pmn * P.plane + v] = mn[v];
                base[pmt * P.plane + v] = mt[v];
                base[3 * P.plane + v] = en[v];
            }
    }
}

template <class T>
__device__ __forceinline__ void store_cell(const Planes<T>& P, long long row, long long col,
                                           const Cons<T>& N, int pmn, int pmt, bool negate_mt) {
    T* base = P.base + row * P.pitch + col;
    base[0] = N.r;
    base[pmn * P.plane] = N.mn;
    base[pmt * P.plane] = negate_mt ? -N.mt : N.mt;
    base[3 * P.plane] = N.e;
}

// Device-side end of a step, run by the last warp to arrive
// (last-block-done pattern: atomics and fences only, no waiting).
static __device__ __noinline__ void finalize_step(Ctl* c, int advance, int out_index) {
    __threadfence();
    const unsigned long long bits = atomicAdd(&c->smax_bits, 0ull);
    const double smax = __longlong_as_double((long long)bits);
    c->smax_bits = 0ull;
    c->arrive = 0u;
    c->smax = smax;
    if (advance) {
        const double t_new = c->t + c->dt;        // scripts/cpu/main_cpu.cpp:241
        if (c->dt_log && c->step < c->dt_log_cap) c->dt_log[c->step] = c->dt;
        c->t = t_new;
        c->step += 1;
        c->cur = out_index;
        unsigned int req = 0u;                    // scripts/cpu/main_cpu.cpp:244-261
        while (c->next_snap < c->nsnap && t_new >= c->snap_target[c->next_snap]) {
            req |= 1u << c->next_snap;
            c->snap_time[c->next_snap] = t_new;
            c->snap_step[c->next_snap] = c->step;
            c->next_snap += 1;
        }
        c->snap_req = req;
    }
    if (c->mode == kModeFrozen) {
        const long long k = c->step - c->frozen_base;
        if (k < c->n_frozen) c->dt = c->frozen[k];
        else c->done = 1;
    } else {
        // src/cpu/solver_cpu.cpp:304-308 and scripts/cpu/main_cpu.cpp:221-228
        if (!(smax > 0.0) || !(smax < INFINITY)) {
            c->status |= kStatusNonPhysical;
            c->done = 1;
        } else {
            double dt = c->cfl_dmin / smax;
            if (c->mode == kModeCfl && c->t + dt > c->t_end) dt = c->t_end - c->t;
            c->dt = dt;
        }
        if (c->mode == kModeCfl && !(c->t < c->t_end)) c->done = 1;
    }
    if (c->step >= c->max_steps) c->done = 1;
    if (c->status & kStatusTimeout) c->done = 1;
    __threadfence();
}

// Warp-level end of a launch: fold the warp's maximum signal speed into the
// grid maximum and let the last warp finalise the step.
template <class T>
__device__ __forceinline__ void warp_arrive(Ctl* ctl, T smax, bool bad, bool timed_out, int lane,
                                            unsigned int ntasks, int advance, int out_index) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) smax = Ar<T>::fmax_(smax, __shfl_xor_sync(0xffffffffu, smax, o));
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
        if (bad) atomicOr(&ctl->status, (int)kStatusNonFinite);
        if (timed_out) atomicOr(&ctl->status, (int)kStatusTimeout);
        const double m = (double)smax;
        if (m > 0.0 && m < INFINITY) atomicMax(&ctl->smax_bits, (unsigned long long)__double_as_longlong(m));
        __threadfence();
        const unsigned int prev = atomicAdd(&ctl->arrive, 1u);
        if (prev == ntasks - 1u) finalize_step(ctl, advance, out_index);
    }
}

// ---------------------------------------------------------------------------
// x-sweep: Uold (S buffer) -> Utmp.  One warp per (32-row group, x-segment),
// one row per lane.  src/cpu/solver_cpu.cpp:206-238 + :437-461
//
// Box k holds S columns [m0 + CX k, m0 + CX (k+1)) of 32 rows, CX = 32 bytes
// of columns, m0 = s0 + kSOff + 2 - CX.  The cell updated when S column c is
// pushed is interior column c - kSOff - 2, which sits in Utmp column c:
// every output lands in the shared-memory slot its input came from, so the
// box is overwritten in place and written back with one TMA store of whole
// 32-byte rows.  Box 0 only warms the stencil window up; boxes 1.. hold
// exactly this segment's outputs (clipped by the store map at the edges).
// ---------------------------------------------------------------------------
// Per-warp mbarrier phases: bit s is the parity the next wait on stage s
// expects.  A warp initialises its barriers once and carries the bits from
// task to task (a persistent warp runs many tasks on the same barriers).
// A single-task launch (PERSIST = false) derives the parity from the box
// index instead, as its barriers start fresh.
template <bool PERSIST>
__device__ __forceinline__ bool stage_wait(uint64_t* bar, int s, int k, int stages, uint32_t& phase) {
    if constexpr (!PERSIST) {
        return mbar_wait_bounded(smem_u32(&bar[s]), (uint32_t)((k / stages) & 1));
    } else {
        const bool ok = mbar_wait_bounded(smem_u32(&bar[s]), (phase >> s) & 1u);
        if (ok) phase ^= 1u << s;
        return ok;
    }
}

// One x-sweep task (one warp): 32 rows x one segment of columns.  Returns
// true when a bounded wait expired (the task is abandoned after draining the
// boxes in flight).
template <class T, int S, int STAGES, bool PERSIST>
__device__ __forceinline__ bool x_task(const CUtensorMap* tm, const CUtensorMap* tm_out, const SweepArgs<T>& a,
                                       int task, T* buf, uint64_t* bar, uint32_t& phase, int lane) {
    constexpr int CX = 32 / sizeof(T);          // columns per box: 32-byte rows
    constexpr int HV = CX / 2;                  // cells per 16-byte half row
    constexpr int STAGE = 4 * 32 * CX;          // elements: 4 fields x 32 rows x CX
    constexpr uint32_t STAGE_BYTES = STAGE * sizeof(T);
    static_assert(STAGE_BYTES % 1024 == 0, "32-byte swizzle needs 1 KB-aligned stage buffers");
    static_assert(kTOff == kSOff + 2, "outputs must land in their input's column");
    Ctl* ctl = a.ctl;
    const int rg = task / a.nseg;                // 32-row group
    const int s0 = (task - rg * a.nseg) * a.seg; // first interior column of the segment
    const int e = min(s0 + a.seg, a.nx);
    const int m0 = s0 + kSOff + 2 - CX;          // first S column marched
    const int nst = 1 + (e - s0 + CX - 1) / CX;  // warm-up box + output boxes
    const int j = rg * 32 + lane;                // interior row of this lane
    const bool row_ok = j < a.ny;
    const double lam_d = __ldcg(&ctl->dt) / a.d; // dt/dx
    const T lam = T(lam_d);
    const T hl = T(0.5 * lam_d);
    const unsigned int req = __ldcg(&ctl->snap_req);
    T* snap = (req && a.snap) ? a.snap + (long long)(__ffs(req) - 1) * a.snap_stride : nullptr;

    if (lane == 0) {
        tma_prefetch_desc(tm);
        tma_prefetch_desc(tm_out);
    }
    auto issue = [&](int k) {
        const int s = k % STAGES;
        const uint32_t b = smem_u32(&bar[s]);
        mbar_arrive_expect_tx(b, STAGE_BYTES);
        tma_load_3d(smem_u32(buf + s * STAGE), tm, b, m0 + k * CX, rg * 32 + 2, 0);
    };
    if (lane == 0) {
        const int np = min(STAGES, nst);
        for (int k = 0; k < np; ++k) issue(k);
    }

    // rows 0, 1, ny-2, ny-1 also feed the y-ghost rows of Utmp
    const bool has_ghost = row_ok && (j <= 1 || j >= a.ny - 2);

    Line<T, S> line;
    line.reset();
    const int swz = (lane >> 2) & 1;             // 32-byte swizzle: 16 B chunk ^= row bit 2
    bool timed_out = false;
    int kfail = nst;
    for (int k = 0; k < nst; ++k) {
        const int s = k % STAGES;
        if (!stage_wait<PERSIST>(bar, s, k, STAGES, phase)) {
            timed_out = true;
            kfail = k;
            break;
        }
        T* rowp = buf + s * STAGE + lane * CX;
        if (snap && row_ok) {                    // the input state is a requested snapshot
            for (int c = 0; c < CX; ++c) {
                const int is = m0 + k * CX + c - kSOff;
                if (is >= s0 && is < e) {
                    const T* q = rowp + (((c / HV) ^ swz) * HV) + (c % HV);
                    T* p = snap + (long long)j * a.nx + is;
                    p[0] = q[0]; p[a.snap_plane] = q[32 * CX]; p[2 * a.snap_plane] = q[64 * CX];
                    p[3 * a.snap_plane] = q[96 * CX];
                }
            }
        }
        // Box 0 holds interior columns s0+2-CX .. s0+1; the first output
        // (column s0, pushed with column s0+2) needs the window from column
        // s0-2 on, so the line is primed there (as the y-sweep's) and the
        // columns before it are not pushed at all (FP32: the first half of
        // box 0).  A line started from nothing would also send its first two
        // cells through the out-of-line full path.
        constexpr int kWarmHalf = (CX - 4) / HV;
#pragma unroll 1
        for (int h = k == 0 ? kWarmHalf : 0; h < 2; ++h) {
            T* q = rowp + ((h ^ swz) * HV);
            T r[HV], mn[HV], mt[HV], en[HV];
            ld_vec<T, HV>(q, r);
            ld_vec<T, HV>(q + 32 * CX, mn);
            ld_vec<T, HV>(q + 64 * CX, mt);
            ld_vec<T, HV>(q + 96 * CX, en);
            if (k == 0 && h == kWarmHalf) line.prime(Cons<T>{r[0], mn[0], mt[0], en[0]});
            if constexpr (sizeof(T) == 4 && S != kExact) {
                // FP32: the cells' primitives two at a time (packed), then the
                // pushes (not for the exact solver: it spilled)
                Prim<T> W[HV];
                bool isl[HV];
#pragma unroll
                for (int v = 0; v < HV; v += 2) {
                    isl[v] = isl[v + 1] = false;
                    c2p_rows(Cons<T>{r[v], mn[v], mt[v], en[v]}, Cons<T>{r[v + 1], mn[v + 1], mt[v + 1], en[v + 1]},
                             W[v], W[v + 1], isl[v], isl[v + 1]);
                }
#pragma unroll
                for (int v = 0; v < HV; ++v) {
                    bool a = false, b = false, c = false;
                    const Cons<T> N = line.template step_w<true>(Cons<T>{r[v], mn[v], mt[v], en[v]}, W[v], isl[v],
                                                                 hl, lam, a, b, c);
                    r[v] = N.r; mn[v] = N.mn; mt[v] = N.mt; en[v] = N.e;
                }
            } else {
#pragma unroll
                for (int v = 0; v < HV; ++v) {
                    const Cons<T> N = line.push(Cons<T>{r[v], mn[v], mt[v], en[v]}, hl, lam);
                    r[v] = N.r; mn[v] = N.mn; mt[v] = N.mt; en[v] = N.e;
                }
            }
            st_vec<T, HV>(q, r);                  // outputs overwrite their inputs in place
            st_vec<T, HV>(q + 32 * CX, mn);
            st_vec<T, HV>(q + 64 * CX, mt);
            st_vec<T, HV>(q + 96 * CX, en);
        }
        if (has_ghost && k > 0) {                 // y-ghost rows of Utmp (few lanes)
            // transmissive sides copy the edge row into both ghost layers,
            // reflective sides mirror rows 0/1 (ny-1/ny-2) with rho*v negated
            int g0 = -1, g1 = -1, g2 = -1, g3 = -1;
            bool n0 = false, n2 = false;
            if (a.bc_lo == kBcReflective) {
                if (j == 0) { g0 = 1; n0 = true; }
                if (j == 1) { g0 = 0; n0 = true; }
            } else if (j == 0) {
                g0 = 1; g1 = 0;
            }
            if (a.bc_hi == kBcReflective) {
                if (j == a.ny - 1) { g2 = a.ny + 2; n2 = true; }
                if (j == a.ny - 2) { g2 = a.ny + 3; n2 = true; }
            } else if (j == a.ny - 1) {
                g2 = a.ny + 2; g3 = a.ny + 3;
            }
            for (int c = 0; c < CX; ++c) {
                const int col = m0 + k * CX + c;
                if (col - kTOff >= a.nx) break;
                const T* q = rowp + (((c / HV) ^ swz) * HV) + (c % HV);
                const Cons<T> N{q[0], q[32 * CX], q[64 * CX], q[96 * CX]};
                if (g0 >= 0) store_cell(a.out, g0, col, N, 1, 2, n0);
                if (g1 >= 0) store_cell(a.out, g1, col, N, 1, 2, false);
                if (g2 >= 0) store_cell(a.out, g2, col, N, 1, 2, n2);
                if (g3 >= 0) store_cell(a.out, g3, col, N, 1, 2, false);
            }
        }
        fence_proxy_async_smem();                 // make the in-place writes visible to TMA
        __syncwarp();
        if (lane == 0) {
            if (k > 0) {
                tma_store_3d(tm_out, smem_u32(buf + s * STAGE), m0 + k * CX, rg * 32 + 2, 0);
                bulk_commit();
            }
            // refill the buffer of box k-1 (its store, if any, is the older group)
            if (k > 0 && k - 1 + STAGES < nst) {
                bulk_wait_read1();
                issue(k - 1 + STAGES);
            }
        }
        __syncwarp();
    }
    if (lane == 0) bulk_wait0();
    if (timed_out) {
        // drain the boxes still in flight (bounded), then report
        const int last = min(kfail + STAGES, nst);
        for (int k = kfail + 1; k < last; ++k) (void)stage_wait<PERSIST>(bar, k % STAGES, k, STAGES, phase);
    }
    return timed_out;
}

// x-sweep: Uold (S buffer) -> Utmp, one task per warp.
template <class T, int S, int STAGES, int NW, int MINB>
__global__ void __launch_bounds__(NW * 32, MINB)
    sweep_x_kernel(const __grid_constant__ CUtensorMap tm, const __grid_constant__ CUtensorMap tm_out,
                   const SweepArgs<T> a) {
    constexpr int STAGE = 4 * 32 * (32 / sizeof(T));
    constexpr uint32_t STAGE_BYTES = STAGE * sizeof(T);
    extern __shared__ __align__(1024) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int task = blockIdx.x * NW + warp;
    if (task >= a.ntasks) return;
    Ctl* ctl = a.ctl;
    if (__ldcg(&ctl->done)) return;

    // stage buffers on a 1 KB boundary (the launch reserves 1 KB of slack)
    unsigned char* base = smem + ((1024u - (smem_u32(smem) & 1023u)) & 1023u);
    T* buf = reinterpret_cast<T*>(base) + (size_t)warp * STAGES * STAGE;
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + (size_t)NW * STAGES * STAGE_BYTES) + warp * STAGES;
    if (lane == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(smem_u32(&bar[s]), 1);
        fence_mbar_init();
    }
    __syncwarp();
    uint32_t phase = 0;
    if (x_task<T, S, STAGES, false>(&tm, &tm_out, a, task, buf, bar, phase, lane) && lane == 0)
        atomicOr(&ctl->status, (int)kStatusTimeout);
}

// ---------------------------------------------------------------------------
// y-sweep: Utmp -> Unew (S buffer), with the fused CFL reduction.  One warp
// per (row segment, group of 32 S columns), one column per lane; the input
// box is BW >= 34 Utmp columns wide because Utmp's interior sits two columns
// right of the S interior.  Box k holds Utmp rows [r0 + RY k, r0 + RY k + RY)
// (RY = 8 in FP32, 4 in FP64) and is processed in groups of 4 rows; a cell
// is final four rows after it enters, so row group j+1 of the segment yields
// the output rows [r0 + 4j, r0 + 4j + 4) (group 0 only warms the window up),
// staged in shared memory and written with one TMA store of whole 128-byte
// rows per group.  A box of 8 rows halves the per-box work (barrier wait,
// TMA load, masks, abort vote) against boxes of 4.  The store map ends at the last 16-byte boundary
// before the right ghost columns (TMA stores clip at 16-byte granularity);
// columns past it, and group 0 whose box would also cover the left ghost
// columns, are stored directly.
// src/cpu/solver_cpu.cpp:247-279 + :474-498
// ---------------------------------------------------------------------------
// max(a, b) that returns NaN when either is NaN (PTX max.NaN).
__device__ __forceinline__ float max_nan(float a, float b) {
    float d;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
    return d;
}

// Result of one y-sweep task for the step's epilogue.
template <class T> struct YOut {
    T smax;
    bool bad, timed_out;
};

// One pass of a y-sweep task (one warp): 32 S columns x one segment of rows.
// FAST = true runs the fast path only and gives up (aborted = true, nothing
// of the box in hand stored, boxes in flight drained) as soon as any lane
// flags a fallback that can reach an output; the caller then reruns the
// task with FAST = false, whose push handles every fallback.  Keeping the
// out-of-line fallback call out of the hot loop is worth about a third of
// the y-sweep's time; outputs do not depend on which pass produced them.
template <class T, int S, int RY, int BW, int STAGES, bool FAST>
__device__ __forceinline__ YOut<T> y_pass(const CUtensorMap* tm, const CUtensorMap* tm_out, const SweepArgs<T>& a,
                                          int task, T* buf, T* obuf, uint64_t* bar, uint32_t& phase, int lane,
                                          bool& aborted) {
    constexpr int LAG = kYLag;                   // rows of one output box
    constexpr int HB = RY / LAG;                 // output boxes per input box
    constexpr int STAGE = 4 * RY * BW;           // input box: 4 fields x RY rows x BW columns
    constexpr uint32_t STAGE_BYTES = STAGE * sizeof(T);
    constexpr int OSTAGE = 4 * LAG * 32;         // output box: 4 fields x LAG rows x 32 columns
    constexpr uint32_t OSTAGE_BYTES = OSTAGE * sizeof(T);
    static_assert(STAGE_BYTES % 128 == 0 && OSTAGE_BYTES % 128 == 0, "stage buffers must stay 128-byte aligned");
    static_assert(BW >= 32 + kTOff - kSOff, "box too narrow");
    static_assert(RY % LAG == 0, "an input box holds whole output boxes");
    Ctl* ctl = a.ctl;
    const int rs = task / a.nseg;                // row segment
    const int g = task - rs * a.nseg;            // group of 32 S columns
    const int r0 = rs * a.seg;                   // first interior output row (a multiple of LAG)
    const int e = min(r0 + a.seg, a.ny);
    const int nob = (e - r0 + LAG - 1) / LAG;    // output boxes of this task
    const int nst = ((nob + 1) * LAG + RY - 1) / RY;   // input boxes: LAG warm-up rows + the output rows
    const int sc = g * 32 + lane;                // S column of this lane
    const int i = sc - kSOff;                    // its interior column
    const bool col_ok = i >= 0 && i < a.nx;
    // Lanes that store without TMA: all of group 0 (its box would cover the
    // left ghost columns) and the columns past the store map's 16-byte end.
    const bool direct = g == 0 || sc >= a.wclip;
    const double lam_d = __ldcg(&ctl->dt) / a.d; // dt/dy
    const T lam = T(lam_d);
    const T hl = T(0.5 * lam_d);
    aborted = false;

    if (lane == 0) {
        tma_prefetch_desc(tm);
        tma_prefetch_desc(tm_out);
    }
    auto issue = [&](int k) {
        const int s = k % STAGES;
        const uint32_t b = smem_u32(&bar[s]);
        mbar_arrive_expect_tx(b, STAGE_BYTES);
        tma_load_3d(smem_u32(buf + s * STAGE), tm, b, g * 32, r0 + k * RY, 0);
    };
    if (lane == 0) {
        const int np = min(STAGES, nst);
        for (int k = 0; k < np; ++k) issue(k);
    }

    Line<T, S> line;
    line.reset();
    T smax = T(0), ssum = T(0);
    const bool edge = col_ok && (i <= 1 || i >= a.nx - 2);   // writes x-ghost columns
    const bool special = __any_sync(0xffffffffu, direct || edge);
    bool timed_out = false;
    int kfail = nst;
    for (int k = 0; k < nst; ++k) {
        const int s = k % STAGES;
        if (!stage_wait<true>(bar, s, k, STAGES, phase)) {
            timed_out = true;
            kfail = k;
            break;
        }
        const T* sbox = buf + s * STAGE + lane + (kTOff - kSOff);
        // FP32 fast pass: the cells of a row group are converted to
        // primitives two rows at a time (packed), and the outputs' signal
        // speeds likewise (not for the exact solver, whose register-heavy
        // Riemann call spilled with four rows' primitives held ahead)
        constexpr bool kRows = FAST && sizeof(T) == 4 && S != kExact;
        bool flag = false;
        if (k == 0)   // window of the line's first cell (see Line::prime)
            line.prime(Cons<T>{sbox[0], sbox[2 * RY * BW], sbox[RY * BW], sbox[3 * RY * BW]});
#pragma unroll 1
        for (int h = 0; h < HB; ++h) {
            const int j = k * HB + h - 1;         // output box of this row group (-1: warm-up)
            if (j >= nob) break;                  // past the task's last output row (warp-uniform)
            const T* sb = sbox + h * LAG * BW;    // the group's rows; fields RY * BW apart
            T* ob = obuf + (j & 1) * OSTAGE + lane;
            if (j >= 2 && lane == 0) bulk_wait_read1();   // output buffer j&1 was stored for box j-2
            __syncwarp();
            const int ir0 = r0 + j * LAG;         // interior row of this group's first output
            // Masks over the group's rows (bit rr): pushes whose flags can
            // reach an output (all of the warm-up group, then up to the
            // segment's last row), and pushes that yield an output of this
            // task.  Testing a constant bit per unrolled row measured 2.6%
            // faster than comparing row indices per cell.
            const int nlive = j < 0 ? LAG : e - ir0;
            const unsigned live_mask = nlive >= LAG ? (1u << LAG) - 1u : (nlive > 0 ? (1u << nlive) - 1u : 0u);
            const int nout = j < 0 ? 0 : min(LAG, e - ir0);
            const unsigned out_mask =
                !col_ok ? 0u : (nout >= LAG ? (1u << LAG) - 1u : (nout > 0 ? (1u << nout) - 1u : 0u));
            Cons<T> Ub[LAG];
            Prim<T> Wb[LAG];
            bool ib[LAG];
            if constexpr (kRows) {
#pragma unroll
                for (int rr = 0; rr < LAG; ++rr) {
                    Ub[rr] = Cons<T>{sb[rr * BW], sb[(2 * RY) * BW + rr * BW], sb[RY * BW + rr * BW],
                                     sb[(3 * RY) * BW + rr * BW]};
                    ib[rr] = false;
                }
#pragma unroll
                for (int rr = 0; rr < LAG; rr += 2) c2p_rows(Ub[rr], Ub[rr + 1], Wb[rr], Wb[rr + 1], ib[rr], ib[rr + 1]);
                if (j < 0) {   // the warm-up group (warp-uniform): every row's pressure island matters
                    static_assert(LAG == 4, "warm4 takes the four warm-up rows");
                    flag |= ib[0] | ib[1] | ib[2] | ib[3];
                    line.warm4(Ub, Wb, hl, flag);
                    continue;
                }
            }
            Cons<T> Nprev{};
#pragma unroll
            for (int rr = 0; rr < LAG; ++rr) {
                // normal momentum of the y-sweep is rho*v (plane 2)
                Cons<T> N;
                if constexpr (kRows) {
                    // a flag matters unless the push lies past the task's
                    // last output row (no later output depends on it)
                    bool f = ib[rr];
                    N = line.step_fast(Ub[rr], Wb[rr], hl, lam, f);
                    flag |= f & (((live_mask >> rr) & 1u) != 0u);
                } else {
                    const Cons<T> U{sb[rr * BW], sb[(2 * RY) * BW + rr * BW], sb[RY * BW + rr * BW],
                                    sb[(3 * RY) * BW + rr * BW]};
                    if constexpr (FAST) {
                        bool fi = false, fc = false, ff = false;
                        N = line.template step<false>(U, hl, lam, fi, fc, ff);
                        flag |= (fi | fc | ff) & (((live_mask >> rr) & 1u) != 0u);
                    } else {
                        N = line.push(U, hl, lam);
                    }
                }
                ob[rr * 32] = N.r;
                ob[(LAG + rr) * 32] = N.mt;
                ob[(2 * LAG + rr) * 32] = N.mn;
                ob[(3 * LAG + rr) * 32] = N.e;
                const int ir = ir0 + rr;
                const bool out_ok = ((out_mask >> rr) & 1u) != 0u;
                if constexpr (kRows) {
                    if (rr & 1) {             // the speeds of rows rr-1 and rr
                        // selects, not branches: a speed is >= 0 or NaN, so
                        // 0 stands in for a row without an output
                        const float2 sp = signal_speed_rows(Nprev, N);
                        const float s0 = ((out_mask >> (rr - 1)) & 1u) ? sp.x : 0.0f;
                        const float s1 = out_ok ? sp.y : 0.0f;
                        smax = max_nan(smax, max_nan(s0, s1));
                    } else {
                        Nprev = N;
                    }
                } else {
                    T sp;
                    if constexpr (sizeof(T) == 4) sp = speed_v<float>(N);   // the fast pass's form, per cell
                    else sp = signal_speed_fast(N);
                    if (out_ok) {
                        if constexpr (sizeof(T) == 4) {
                            smax = max_nan(smax, sp);     // NaN propagates: checked once at the end
                        } else {
                            ssum += sp;                   // NaN / inf propagate: checked once at the end
                            smax = Ar<T>::fmax_(smax, sp);
                        }
                    }
                }
                if (special) {                        // warp-uniform: few warps store anything directly
                    if (out_ok && direct) store_cell(a.out, ir + 2, sc, N, 2, 1, false);
                    if (out_ok && edge) {             // x-ghost columns of Unew read by the next x-sweep
                        if (i == 0) {
                            if (a.bc_lo == kBcReflective) store_cell(a.out, ir + 2, kSOff - 1, N, 2, 1, true);
                            else { store_cell(a.out, ir + 2, kSOff - 1, N, 2, 1, false);
                                   store_cell(a.out, ir + 2, kSOff - 2, N, 2, 1, false); }
                        }
                        if (i == 1 && a.bc_lo == kBcReflective) store_cell(a.out, ir + 2, kSOff - 2, N, 2, 1, true);
                        if (i == a.nx - 1) {
                            if (a.bc_hi == kBcReflective) store_cell(a.out, ir + 2, a.nx + kSOff, N, 2, 1, true);
                            else { store_cell(a.out, ir + 2, a.nx + kSOff, N, 2, 1, false);
                                   store_cell(a.out, ir + 2, a.nx + kSOff + 1, N, 2, 1, false); }
                        }
                        if (i == a.nx - 2 && a.bc_hi == kBcReflective)
                            store_cell(a.out, ir + 2, a.nx + kSOff + 1, N, 2, 1, true);
                    }
                }
            }
            if (j >= 0) {   // store the group's outputs (an aborted pass's are rewritten by the full pass)
                fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0 && g != 0 && g * 32 < a.wclip) {
                    tma_store_3d(tm_out, smem_u32(obuf + (j & 1) * OSTAGE), g * 32, ir0 + 2, 0);
                    bulk_commit();
                }
            }
        }
        if constexpr (FAST) {
            if (__any_sync(0xffffffffu, flag && col_ok)) {
                aborted = true;
                kfail = k;
                break;
            }
        }
        fence_proxy_async_smem();
        __syncwarp();                             // every lane is done with stage s
        if (lane == 0 && k + STAGES < nst) issue(k + STAGES);
    }
    if (lane == 0) bulk_wait0();
    if (timed_out || aborted) {
        // drain the boxes still in flight (bounded)
        const int last = min(kfail + STAGES, nst);
        for (int k = kfail + 1; k < last; ++k) (void)stage_wait<true>(bar, k % STAGES, k, STAGES, phase);
    }
    const bool bad = sizeof(T) == 4 ? !(smax < T(INFINITY)) : !(Ar<T>::fabs_(ssum) < T(INFINITY));
    return YOut<T>{smax, bad, timed_out};
}

// The full pass, out of line so that its code stays out of the fast loop.
template <class T, int S, int RY, int BW, int STAGES>
__device__ __noinline__ YOut<T> y_task_full(const CUtensorMap* tm, const CUtensorMap* tm_out, const SweepArgs<T>& a,
                                            int task, T* buf, T* obuf, uint64_t* bar, uint32_t* phase, int lane) {
    bool unused = false;
    return y_pass<T, S, RY, BW, STAGES, false>(tm, tm_out, a, task, buf, obuf, bar, *phase, lane, unused);
}

// One y-sweep task: the fast pass, and the full pass when the fast one gave
// up.  Barrier phases are carried in `phase` across both passes.
template <class T, int S, int RY, int BW, int STAGES>
__device__ __forceinline__ YOut<T> y_task(const CUtensorMap* tm, const CUtensorMap* tm_out, const SweepArgs<T>& a,
                                          int task, T* buf, T* obuf, uint64_t* bar, uint32_t& phase, int lane) {
    bool aborted = false;
    YOut<T> o = y_pass<T, S, RY, BW, STAGES, true>(tm, tm_out, a, task, buf, obuf, bar, phase, lane, aborted);
    if (aborted && !o.timed_out) o = y_task_full<T, S, RY, BW, STAGES>(tm, tm_out, a, task, buf, obuf, bar, &phase, lane);
    return o;
}

// y-sweep: Utmp -> Unew (S buffer), with the fused CFL reduction.  The
// launch holds one CTA per resident slot and its warps take tasks from the
// handle's work list (Ctl::ytask_next) until it is empty, so a warp that
// finishes early starts the next task at once instead of waiting for its
// CTA's other warps (measured 0.7% faster than one task per warp at 8192^2,
// bit-identical; the x-sweep gains nothing from it).  Each warp folds its
// tasks' signal speeds, and the last warp to leave the list resets it for
// the next launch.
template <class T, int S, int RY, int BW, int STAGES, int NW, int MINB>
__global__ void __launch_bounds__(NW * 32, MINB)
    sweep_y_kernel(const __grid_constant__ CUtensorMap tm, const __grid_constant__ CUtensorMap tm_out,
                   const SweepArgs<T> a) {
    constexpr int STAGE = 4 * RY * BW;
    constexpr uint32_t STAGE_BYTES = STAGE * sizeof(T);
    constexpr int OSTAGE = 4 * kYLag * 32;
    constexpr uint32_t OSTAGE_BYTES = OSTAGE * sizeof(T);
    extern __shared__ __align__(1024) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    Ctl* ctl = a.ctl;
    if (__ldcg(&ctl->done)) return;

    unsigned char* base = smem + ((1024u - (smem_u32(smem) & 1023u)) & 1023u);
    T* buf = reinterpret_cast<T*>(base) + (size_t)warp * STAGES * STAGE;
    T* obuf = reinterpret_cast<T*>(base + (size_t)NW * STAGES * STAGE_BYTES) + (size_t)warp * 2 * OSTAGE;
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + (size_t)NW * (STAGES * STAGE_BYTES + 2 * OSTAGE_BYTES)) +
                    warp * STAGES;
    if (lane == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(smem_u32(&bar[s]), 1);
        fence_mbar_init();
    }
    __syncwarp();
    uint32_t phase = 0;
    T smax = T(0);
    bool bad = false, timed_out = false;
    for (;;) {
        int task = 0;
        if (lane == 0) task = (int)atomicAdd(&ctl->ytask_next, 1u);
        task = __shfl_sync(0xffffffffu, task, 0);
        if (task >= a.ntasks) break;
        const YOut<T> o = y_task<T, S, RY, BW, STAGES>(&tm, &tm_out, a, task, buf, obuf, bar, phase, lane);
        if constexpr (sizeof(T) == 4) smax = max_nan(smax, o.smax);   // NaN propagates to the final check
        else smax = fmax(smax, o.smax);
        bad |= o.bad;
        timed_out |= o.timed_out;
    }
    const unsigned int nwarps = gridDim.x * NW;
    if (lane == 0) {
        __threadfence();
        if (atomicAdd(&ctl->ytask_exit, 1u) == nwarps - 1u) {   // every warp is past the list
            ctl->ytask_next = 0u;
            ctl->ytask_exit = 0u;
            __threadfence();
        }
    }
    warp_arrive<T>(ctl, smax, bad, timed_out, lane, nwarps, a.finalize, a.out_index);
}

// ---------------------------------------------------------------------------
// Ensemble step: the x- and y-sweep tasks of many independent grids
// (instances with their own sizes, boundaries, parameters and dt) in one
// persistent launch.  Every warp dequeues tasks from one work list -- all
// x-sweep tasks first, instance by instance, then all y-sweep tasks -- and
// runs them with the same task bodies as the single-grid kernels, so every
// instance's result is bit-for-bit that of its own launches.  A y-sweep task
// of instance q waits (bounded acquire spin) until all of q's x-sweep tasks
// have published their Utmp writes; every x-sweep task was dequeued before
// any y-sweep task and none of them waits, so the wait always ends.  Each
// instance's last y-sweep warp finalises that instance's step (t, step,
// next dt from its own CFL reduction) exactly as in a single-grid launch.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int ens_find(const int* off, int n, int t) {
    int lo = 0, hi = n;                          // off[lo] <= t < off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= t) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <class T, int S, int SX, int RY, int BWY, int SY, int NW, int MINB>
__global__ void __launch_bounds__(NW * 32, MINB) ensemble_kernel(const __grid_constant__ EnsArgs<T> e) {
    constexpr int CX = 32 / sizeof(T);
    constexpr size_t XB = (size_t)SX * 4 * 32 * CX * sizeof(T);
    constexpr size_t YSTAGE = (size_t)4 * RY * BWY * sizeof(T);
    constexpr size_t YB = SY * YSTAGE + 2 * (size_t)4 * kYLag * 32 * sizeof(T);
    constexpr size_t WB = ((XB > YB ? XB : YB) + 1023) / 1024 * 1024;   // per-warp region
    constexpr int NB = SX > SY ? SX : SY;
    static_assert(YSTAGE % 128 == 0, "y output staging must stay 128-byte aligned");
    extern __shared__ __align__(1024) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* base = smem + ((1024u - (smem_u32(smem) & 1023u)) & 1023u);
    unsigned char* wb = base + (size_t)warp * WB;
    uint64_t* bar = reinterpret_cast<uint64_t*>(base + (size_t)NW * WB) + warp * NB;
    if (lane == 0) {
        for (int s = 0; s < NB; ++s) mbar_init(smem_u32(&bar[s]), 1);
        fence_mbar_init();
    }
    __syncwarp();
    uint32_t phase = 0;
    const int total = e.total_x + e.total_y;
    for (;;) {
        int t = 0;
        if (lane == 0) t = (int)atomicAdd(&e.sched->next, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= total) break;
        if (t < e.total_x) {
            const int q = ens_find(e.x_off, e.ninst, t);
            const EnsInst<T>& I = e.inst[q];
            Ctl* ctl = I.xa.ctl;
            if (!__ldcg(&ctl->done)) {
                const int cur = __ldcg(&ctl->cur);
                const bool to = x_task<T, S, SX, true>(&I.tm_x[cur], &I.tm_xo, I.xa, t - e.x_off[q],
                                                       reinterpret_cast<T*>(wb), bar, phase, lane);
                if (to && lane == 0) atomicOr(&ctl->status, (int)kStatusTimeout);
            }
            // publish this task's Utmp writes (TMA stores completed by the
            // task's final bulk wait, ghost rows by plain stores)
            __threadfence();
            __syncwarp();
            if (lane == 0) {
                fence_proxy_async_global();
                __threadfence();
                atomicAdd(&e.sched->xdone[q], 1u);
            }
        } else {
            const int ty = t - e.total_x;
            const int q = ens_find(e.y_off, e.ninst, ty);
            const EnsInst<T>& I = e.inst[q];
            Ctl* ctl = I.xa.ctl;
            if (__ldcg(&ctl->done)) continue;
            int ok = 1;
            if (lane == 0) {
                ok = wait_count_bounded(&e.sched->xdone[q], (unsigned)(I.xa.ntasks + e.wait_extra)) ? 1 : 0;
                fence_proxy_async_global();
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
            const int cur = __ldcg(&ctl->cur);
            const SweepArgs<T>& a = I.ya[1 - cur];
            YOut<T> o{T(0), false, true};
            if (ok)
                o = y_task<T, S, RY, BWY, SY>(&I.tm_y, &I.tm_yo[1 - cur], a, ty - e.y_off[q],
                                                     reinterpret_cast<T*>(wb),
                                                     reinterpret_cast<T*>(wb + SY * YSTAGE), bar, phase, lane);
            warp_arrive<T>(ctl, o.smax, o.bad, o.timed_out, lane, (unsigned)a.ntasks, a.finalize, a.out_index);
        }
    }
}

// Dynamic shared memory of the ensemble kernel.
template <class T, int SX, int RY, int BWY, int SY, int NW> constexpr size_t ensemble_smem() {
    constexpr int CX = 32 / sizeof(T);
    constexpr size_t XB = (size_t)SX * 4 * 32 * CX * sizeof(T);
    constexpr size_t YB = SY * (size_t)4 * RY * BWY * sizeof(T) + 2 * (size_t)4 * kYLag * 32 * sizeof(T);
    constexpr size_t WB = ((XB > YB ? XB : YB) + 1023) / 1024 * 1024;
    constexpr int NB = SX > SY ? SX : SY;
    return 1024 + NW * WB + NW * NB * sizeof(uint64_t);
}

// ---------------------------------------------------------------------------
// First-order Godunov step (src/cpu/solver_cpu.cpp:315-369): four interface
// fluxes per cell from the unreconstructed neighbours, one thread per cell,
// ghosts of the input read as given; the caller refills the output's ghost
// frame afterwards (the reference ends with apply_transmissive_boundary).
// ---------------------------------------------------------------------------
template <class T, int S>
__global__ void __launch_bounds__(256) first_order_kernel(Planes<T> in, Planes<T> out, int nx, int ny,
                                                          double dtdx, double dtdy) {
    const long long total = (long long)nx * ny;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(idx / nx), i = (int)(idx - (long long)j * nx);
        const T* c = in.base + (long long)(j + 2) * in.pitch + (i + kSOff);
        auto ld = [&](long long off) {
            const T* q = c + off;
            return Cons<T>{q[0], q[in.plane], q[2 * in.plane], q[3 * in.plane]};
        };
        const Cons<T> U = ld(0), W = ld(-1), E_ = ld(1), Sd = ld(-in.pitch), Nd = ld(in.pitch);
        // x faces in (n, t) = (rho u, rho v); y faces in (n, t) = (rho v, rho u)
        auto swp = [](const Cons<T>& a) { return Cons<T>{a.r, a.mt, a.mn, a.e}; };
        const Cons<T> Fxp = riemann<S>(U, cons_to_prim(U), E_, cons_to_prim(E_));
        const Cons<T> Fxm = riemann<S>(W, cons_to_prim(W), U, cons_to_prim(U));
        const Cons<T> Uy = swp(U), Ny = swp(Nd), Sy = swp(Sd);
        const Cons<T> Gp = riemann<S>(Uy, cons_to_prim(Uy), Ny, cons_to_prim(Ny));
        const Cons<T> Gm = riemann<S>(Sy, cons_to_prim(Sy), Uy, cons_to_prim(Uy));
        const T ax = T(dtdx), ay = T(dtdy);
        T* o = out.base + (long long)(j + 2) * out.pitch + (i + kSOff);
        o[0] = (U.r - ax * (Fxp.r - Fxm.r)) - ay * (Gp.r - Gm.r);
        o[out.plane] = (U.mn - ax * (Fxp.mn - Fxm.mn)) - ay * (Gp.mt - Gm.mt);
        o[2 * out.plane] = (U.mt - ax * (Fxp.mt - Fxm.mt)) - ay * (Gp.mn - Gm.mn);
        o[3 * out.plane] = (U.e - ax * (Fxp.e - Fxm.e)) - ay * (Gp.e - Gm.e);
    }
}

}  // namespace eu
