// sweeps.cuh -- the fused x- and y-sweep kernels of the MUSCL-Hancock split
// step (src/cpu/solver_cpu.cpp:400-499 restated for sm_103a).
//
// Data layout in HBM (SoA planes, 2-cell ghost frame):
//   state buffers S0/S1 : interior (i, j) at column i+2, row j+2
//   Utmp                : interior (i, j) at column i+4, row j+2
// The extra two columns of Utmp absorb the x-sweep's two-cell output lag so
// that every lane of both sweeps stores whole 16-byte vectors.
//
// Execution model: every warp is an independent marching unit with its own
// shared-memory stages and mbarriers.  Lane 0 streams boxes of the input
// planes into shared memory with TMA (cp.async.bulk.tensor.3d, all four
// fields in one box) while the warp computes on earlier boxes.  Each lane
// owns VEC adjacent cells; the stencil state slides through registers along
// the march direction, so each cell is reconstructed once and each face
// solved once.  Nothing is written back except the updated cells (and the
// ghost lines the next sweep reads):
//   x-sweep : warp marches along one row, W = 32*VEC cells per box; the
//             neighbour values cross lanes by warp shuffles and cross boxes
//             through lane 0's carry registers.
//   y-sweep : warp covers 32*VEC columns and marches up a row segment, RY rows
//             per box; no shuffles at all.  Its epilogue reduces the maximum
//             signal speed (warp shuffle max -> one atomic per warp) and the
//             last warp to finish computes the next dt on the device.
#pragma once
#include "eu_internal.h"
#include "euler_numerics.cuh"
#include "tma_pipe.cuh"

namespace eu {

// ---------------------------------------------------------------------------
// warp helpers
// ---------------------------------------------------------------------------
template <class T> __device__ __forceinline__ T shfl_rot(T v, int lane) {
    return __shfl_sync(0xffffffffu, v, (lane + 31) & 31);
}

// Value held by the owner of the previous cells: lane-1, or for lane 0 the
// value lane 31 held in the previous box (kept in `carry`).
template <class T> __device__ __forceinline__ T prev_of(T v, T& carry, int lane) {
    const T r = shfl_rot(v, lane);
    const T out = (lane == 0) ? carry : r;
    carry = r;
    return out;
}
template <class T>
__device__ __forceinline__ Cons<T> prev_of(const Cons<T>& v, Cons<T>& c, int lane) {
    return Cons<T>{prev_of(v.r, c.r, lane), prev_of(v.mn, c.mn, lane), prev_of(v.mt, c.mt, lane),
                   prev_of(v.e, c.e, lane)};
}
// Primitive without 1/rho (the reconstruction never reads it).
template <class T>
__device__ __forceinline__ Prim<T> prev_prim4(const Prim<T>& v, Prim<T>& c, int lane) {
    return Prim<T>{prev_of(v.r, c.r, lane), prev_of(v.un, c.un, lane), prev_of(v.ut, c.ut, lane),
                   prev_of(v.p, c.p, lane), T(0)};
}
template <class T>
__device__ __forceinline__ Face<T> prev_face(const Face<T>& v, Face<T>& c, int lane) {
    Face<T> o;
    o.U = prev_of(v.U, c.U, lane);
    o.V = Prim<T>{prev_of(v.V.r, c.V.r, lane), prev_of(v.V.un, c.V.un, lane),
                  prev_of(v.V.ut, c.V.ut, lane), prev_of(v.V.p, c.V.p, lane),
                  prev_of(v.V.ir, c.V.ir, lane)};
    return o;
}

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
// x-sweep: Uold (S buffer) -> Utmp.  One warp per (row, x-segment).
// src/cpu/solver_cpu.cpp:206-238 + :437-461
// ---------------------------------------------------------------------------
template <class T, int S, int VEC, int STAGES, int NW>
__global__ void __launch_bounds__(NW * 32)
    sweep_x_kernel(const __grid_constant__ CUtensorMap tm, const SweepArgs<T> a) {
    constexpr int W = 32 * VEC;
    constexpr int STAGE = 4 * W;
    constexpr uint32_t STAGE_BYTES = STAGE * sizeof(T);
    extern __shared__ __align__(128) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int task = blockIdx.x * NW + warp;
    if (task >= a.ntasks) return;
    Ctl* ctl = a.ctl;
    if (__ldcg(&ctl->done)) return;

    T* buf = reinterpret_cast<T*>(smem) + (size_t)warp * STAGES * STAGE;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + (size_t)NW * STAGES * STAGE_BYTES) + warp * STAGES;

    const int j = task / a.nseg;                 // interior row
    const int s0 = (task - j * a.nseg) * a.seg;  // first interior column of this task
    const int e = min(s0 + a.seg, a.nx);
    const int nchunks = (e + 4 - s0 + W - 1) / W;
    const double lam_d = __ldcg(&ctl->dt) / a.d;  // dt/dx
    const T lam = T(lam_d);
    const T hl = T(0.5 * lam_d);
    const unsigned int req = __ldcg(&ctl->snap_req);
    T* snap = (req && a.snap) ? a.snap + (long long)(__ffs(req) - 1) * a.snap_stride : nullptr;

    if (lane == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(smem_u32(&bar[s]), 1);
        fence_mbar_init();
        tma_prefetch_desc(&tm);
    }
    __syncwarp();
    auto issue = [&](int k) {
        const int s = k % STAGES;
        const uint32_t b = smem_u32(&bar[s]);
        mbar_arrive_expect_tx(b, STAGE_BYTES);
        tma_load_3d(smem_u32(buf + s * STAGE), &tm, b, s0 + k * W, j + 2, 0);
    };
    if (lane == 0) {
        const int np = min(STAGES, nchunks);
        for (int k = 0; k < np; ++k) issue(k);
    }

    // Ghost rows of Utmp fed by this row (the y-ghosts the y-sweep reads):
    // transmissive sides copy the edge row into both layers, reflective
    // sides mirror rows 0/1 (ny-1/ny-2) with rho*v negated.
    int grow[4];
    bool gneg[4];
    int nghost = 0;
    if (a.bc_lo == kBcReflective) {
        if (j == 0) { grow[nghost] = 1; gneg[nghost++] = true; }
        if (j == 1) { grow[nghost] = 0; gneg[nghost++] = true; }
    } else if (j == 0) {
        grow[nghost] = 1; gneg[nghost++] = false;
        grow[nghost] = 0; gneg[nghost++] = false;
    }
    if (a.bc_hi == kBcReflective) {
        if (j == a.ny - 1) { grow[nghost] = a.ny + 2; gneg[nghost++] = true; }
        if (j == a.ny - 2) { grow[nghost] = a.ny + 3; gneg[nghost++] = true; }
    } else if (j == a.ny - 1) {
        grow[nghost] = a.ny + 2; gneg[nghost++] = false;
        grow[nghost] = a.ny + 3; gneg[nghost++] = false;
    }

    Prim<T> cW1{}, cW2{};
    Cons<T> cU1{}, cU2{}, cF{};
    Face<T> cR{};
    bool timed_out = false;
    int kfail = nchunks;
    for (int k = 0; k < nchunks; ++k) {
        const int s = k % STAGES;
        if (!mbar_wait_bounded(smem_u32(&bar[s]), (uint32_t)((k / STAGES) & 1))) {
            timed_out = true;
            kfail = k;
            break;
        }
        Cons<T> Ux[VEC + 2];
        {
            const T* sb = buf + s * STAGE + lane * VEC;
            T r[VEC], mn[VEC], mt[VEC], en[VEC];
            ld_vec<T, VEC>(sb, r);
            ld_vec<T, VEC>(sb + W, mn);
            ld_vec<T, VEC>(sb + 2 * W, mt);
            ld_vec<T, VEC>(sb + 3 * W, en);
#pragma unroll
            for (int v = 0; v < VEC; ++v) Ux[v + 2] = Cons<T>{r[v], mn[v], mt[v], en[v]};
        }
        __syncwarp();
        if (lane == 0 && k + STAGES < nchunks) {
            fence_proxy_async_smem();
            issue(k + STAGES);
        }
        const int c0 = s0 + k * W + lane * VEC;  // S-buffer column of slot 0

        if (snap) {  // the input state is a requested snapshot
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                const int ic = c0 + v - 2;
                if (ic >= s0 && ic < e) {
                    T* q = snap + (long long)j * a.nx + ic;
                    q[0] = Ux[v + 2].r;
                    q[a.snap_plane] = Ux[v + 2].mn;
                    q[2 * a.snap_plane] = Ux[v + 2].mt;
                    q[3 * a.snap_plane] = Ux[v + 2].e;
                }
            }
        }

        // primitives of this box's cells; neighbours from the previous owner
        Prim<T> Wx[VEC + 2];
#pragma unroll
        for (int v = 0; v < VEC; ++v) Wx[v + 2] = cons_to_prim(Ux[v + 2]);
        Wx[1] = prev_prim4(Wx[VEC + 1], cW1, lane);
        Wx[0] = prev_prim4(Wx[VEC], cW2, lane);
        Ux[1] = prev_of(Ux[VEC + 1], cU1, lane);
        Ux[0] = prev_of(Ux[VEC], cU2, lane);

        // slot v reconstructs cell c0+v-1, solves face (c0+v-2 | c0+v-1) and
        // updates cell c0+v-2
        Face<T> L[VEC], R[VEC];
#pragma unroll
        for (int v = 0; v < VEC; ++v) reconstruct(Wx[v], Wx[v + 1], Wx[v + 2], hl, L[v], R[v]);
        const Face<T> Rm = prev_face(R[VEC - 1], cR, lane);
        Cons<T> F[VEC];
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
            const Face<T>& left = (v == 0) ? Rm : R[v - 1];
            F[v] = riemann<S>(left.U, left.V, L[v].U, L[v].V);
        }
        const Cons<T> Fm = prev_of(F[VEC - 1], cF, lane);
        Cons<T> N[VEC];
        unsigned mask = 0u;
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
            const Cons<T>& fm = (v == 0) ? Fm : F[v - 1];
            // src/cpu/solver_cpu.cpp:452-453
            N[v] = Cons<T>{Ux[v].r - lam * (F[v].r - fm.r), Ux[v].mn - lam * (F[v].mn - fm.mn),
                           Ux[v].mt - lam * (F[v].mt - fm.mt), Ux[v].e - lam * (F[v].e - fm.e)};
            const int ic = c0 + v - 4;
            if (ic >= s0 && ic < e) mask |= 1u << v;
        }
        if (mask) {
            store_cells<T, VEC>(a.out, j + 2, c0, N, mask, 1, 2, false);
            for (int q = 0; q < nghost; ++q) store_cells<T, VEC>(a.out, grow[q], c0, N, mask, 1, 2, gneg[q]);
        }
    }
    if (timed_out) {
        // drain the boxes still in flight (bounded), then report
        const int last = min(kfail + STAGES, nchunks);
        for (int k = kfail + 1; k < last; ++k)
            (void)mbar_wait_bounded(smem_u32(&bar[k % STAGES]), (uint32_t)((k / STAGES) & 1));
        if (lane == 0) atomicOr(&ctl->status, (int)kStatusTimeout);
    }
}

// ---------------------------------------------------------------------------
// y-sweep: Utmp -> Unew (S buffer), with the fused CFL reduction.  One warp
// per (row segment, column group).  src/cpu/solver_cpu.cpp:247-279 + :474-498
// ---------------------------------------------------------------------------
template <class T, int S, int VEC, int RY, int BW, int OFF, int STAGES, int NW>
__global__ void __launch_bounds__(NW * 32)
    sweep_y_kernel(const __grid_constant__ CUtensorMap tm, const SweepArgs<T> a) {
    constexpr int WY = 32 * VEC;
    constexpr int STAGE = 4 * RY * BW;
    constexpr uint32_t STAGE_BYTES = STAGE * sizeof(T);
    static_assert(4 - OFF + WY <= BW, "box too narrow");
    extern __shared__ __align__(128) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int task = blockIdx.x * NW + warp;
    if (task >= a.ntasks) return;
    Ctl* ctl = a.ctl;
    if (__ldcg(&ctl->done)) return;

    T* buf = reinterpret_cast<T*>(smem) + (size_t)warp * STAGES * STAGE;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + (size_t)NW * STAGES * STAGE_BYTES) + warp * STAGES;

    const int rs = task / a.nseg;                // row segment
    const int g = task - rs * a.nseg;            // column group
    const int r0 = rs * a.seg;                   // first interior output row
    const int e = min(r0 + a.seg, a.ny);
    const int nrows = e + 4 - r0;
    const int nst = (nrows + RY - 1) / RY;
    const int i0 = g * WY - OFF + lane * VEC;    // interior column of slot 0
    const double lam_d = __ldcg(&ctl->dt) / a.d;
    const T lam = T(lam_d);
    const T hl = T(0.5 * lam_d);

    if (lane == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(smem_u32(&bar[s]), 1);
        fence_mbar_init();
        tma_prefetch_desc(&tm);
    }
    __syncwarp();
    auto issue = [&](int k) {
        const int s = k % STAGES;
        const uint32_t b = smem_u32(&bar[s]);
        mbar_arrive_expect_tx(b, STAGE_BYTES);
        tma_load_3d(smem_u32(buf + s * STAGE), &tm, b, g * WY, r0 + k * RY, 0);
    };
    if (lane == 0) {
        const int np = min(STAGES, nst);
        for (int k = 0; k < np; ++k) issue(k);
    }

    unsigned colmask = 0u;
#pragma unroll
    for (int v = 0; v < VEC; ++v)
        if (i0 + v >= 0 && i0 + v < a.nx) colmask |= 1u << v;

    Prim<T> Wm2[VEC], Wm1[VEC];
    Cons<T> Um2[VEC], Um1[VEC], Fp[VEC];
    Face<T> Rp[VEC];
#pragma unroll
    for (int v = 0; v < VEC; ++v) {
        Wm2[v] = Prim<T>{}; Wm1[v] = Prim<T>{}; Um2[v] = Cons<T>{}; Um1[v] = Cons<T>{};
        Fp[v] = Cons<T>{}; Rp[v] = Face<T>{};
    }
    T smax = T(0);
    bool bad = false, timed_out = false;
    int kfail = nst;
    for (int k = 0; k < nst; ++k) {
        const int s = k % STAGES;
        if (!mbar_wait_bounded(smem_u32(&bar[s]), (uint32_t)((k / STAGES) & 1))) {
            timed_out = true;
            kfail = k;
            break;
        }
        Cons<T> U[RY][VEC];
#pragma unroll
        for (int rr = 0; rr < RY; ++rr) {
            const T* sb = buf + s * STAGE + rr * BW + (4 - OFF) + lane * VEC;
            T r[VEC], mu[VEC], mv[VEC], en[VEC];
            ld_vec<T, VEC>(sb, r);
            ld_vec<T, VEC>(sb + RY * BW, mu);
            ld_vec<T, VEC>(sb + 2 * RY * BW, mv);
            ld_vec<T, VEC>(sb + 3 * RY * BW, en);
#pragma unroll
            for (int v = 0; v < VEC; ++v) U[rr][v] = Cons<T>{r[v], mv[v], mu[v], en[v]};  // n = y
        }
        __syncwarp();
        if (lane == 0 && k + STAGES < nst) {
            fence_proxy_async_smem();
            issue(k + STAGES);
        }
#pragma unroll
        for (int rr = 0; rr < RY; ++rr) {
            const int R = r0 + k * RY + rr;      // Utmp row of the freshest cells
            Cons<T> N[VEC];
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
                const Prim<T> W = cons_to_prim(U[rr][v]);
                Face<T> L, Rn;
                reconstruct(Wm2[v], Wm1[v], W, hl, L, Rn);           // cell row R-1
                const Cons<T> F = riemann<S>(Rp[v].U, Rp[v].V, L.U, L.V);  // face (R-2 | R-1)
                // src/cpu/solver_cpu.cpp:489-490, cell row R-2
                N[v] = Cons<T>{Um2[v].r - lam * (F.r - Fp[v].r), Um2[v].mn - lam * (F.mn - Fp[v].mn),
                               Um2[v].mt - lam * (F.mt - Fp[v].mt), Um2[v].e - lam * (F.e - Fp[v].e)};
                Wm2[v] = Wm1[v]; Wm1[v] = W;
                Um2[v] = Um1[v]; Um1[v] = U[rr][v];
                Rp[v] = Rn; Fp[v] = F;
            }
            const int ir = R - 4;                // interior row of N
            if (ir >= r0 && ir < e && colmask) {
                store_cells<T, VEC>(a.out, ir + 2, i0 + 2, N, colmask, 2, 1, false);
#pragma unroll
                for (int v = 0; v < VEC; ++v) {
                    if (!(colmask & (1u << v))) continue;
                    const T sp = max_signal_speed(N[v]);
                    bad |= !(sp < T(INFINITY));
                    smax = Ar<T>::fmax_(smax, sp);
                    // x-ghost columns of Unew read by the next x-sweep
                    const int ic = i0 + v;
                    if (ic == 0) {
                        if (a.bc_lo == kBcReflective) store_cell(a.out, ir + 2, 1, N[v], 2, 1, true);
                        else { store_cell(a.out, ir + 2, 1, N[v], 2, 1, false);
                               store_cell(a.out, ir + 2, 0, N[v], 2, 1, false); }
                    }
                    if (ic == 1 && a.bc_lo == kBcReflective) store_cell(a.out, ir + 2, 0, N[v], 2, 1, true);
                    if (ic == a.nx - 1) {
                        if (a.bc_hi == kBcReflective) store_cell(a.out, ir + 2, a.nx + 2, N[v], 2, 1, true);
                        else { store_cell(a.out, ir + 2, a.nx + 2, N[v], 2, 1, false);
                               store_cell(a.out, ir + 2, a.nx + 3, N[v], 2, 1, false); }
                    }
                    if (ic == a.nx - 2 && a.bc_hi == kBcReflective)
                        store_cell(a.out, ir + 2, a.nx + 3, N[v], 2, 1, true);
                }
            }
        }
    }
    if (timed_out) {
        const int last = min(kfail + STAGES, nst);
        for (int k = kfail + 1; k < last; ++k)
            (void)mbar_wait_bounded(smem_u32(&bar[k % STAGES]), (uint32_t)((k / STAGES) & 1));
    }
    warp_arrive<T>(ctl, smax, bad, timed_out, lane, (unsigned)a.ntasks, a.finalize, a.out_index);
}

}  // namespace eu
