// Per-revolution thermal kernels, batched over solves.
//
// One revolution of the reference (inertiadifference,
// 3905/Thermal/NominalPole/main.cpp:1473-1557) advances every non-converged
// facet through NTAU steps of FTCS conduction + a Newton-Raphson radiative
// surface boundary.  Its self-heating flux reads only previous-revolution
// surface temperatures (main.cpp:1505-1527), so the revolution splits into
//
//   k_selfheat_w   W[f][s] = eps*sigma*T_{r-1}[s][f]^4          (transpose)
//   k_selfheat_q   Q[s][f] = sum_k W[g_k][s] * vf_k  (list order)  -- A6
//                  (FAST: the tensor-core product of atpm_spmm_tc.cu)
//   k_conduction   depth column in registers, NTAU steps, Newton BC -- A1
//                  (FAST: over the active-facet list once at most half a
//                  solve is active)
//   k_tail_mode, k_conduction_warp   FAST late revolutions: one warp per
//                  active facet once the batch has few of them
//   k_converge     shape_converged (main.cpp:1876-1909)             -- A4
//                  (+ the active-facet lists and row-block activity)
//   k_advance      revolution counter / stop rule (main.cpp:2522-2539)
//
// All of them read the per-solve control word and return at once for solves
// that have stopped, so the same launch sequence (or a captured graph of it)
// can be replayed until every solve in the batch is done.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "atpm_internal.h"

namespace atpm {

// ------------------------------------------------------------------ arithmetic
template <int MODE> struct Ar;
template <> struct Ar<MODE_REF> {
    using R = float;
    static __device__ __forceinline__ R add(R a, R b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ R sub(R a, R b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ R mul(R a, R b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ R div(R a, R b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ R fabs_(R a) { return fabsf(a); }
};
template <> struct Ar<MODE_FP64> {
    using R = double;
    static __device__ __forceinline__ R add(R a, R b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ R sub(R a, R b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ R mul(R a, R b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ R div(R a, R b) { return __ddiv_rn(a, b); }
    static __device__ __forceinline__ R fabs_(R a) { return fabs(a); }
};
template <> struct Ar<MODE_FAST> {
    using R = float;
    static __device__ __forceinline__ R add(R a, R b) { return a + b; }
    static __device__ __forceinline__ R sub(R a, R b) { return a - b; }
    static __device__ __forceinline__ R mul(R a, R b) { return a * b; }
    static __device__ __forceinline__ R div(R a, R b) { return a / b; }
    static __device__ __forceinline__ R fabs_(R a) { return fabsf(a); }
};

__device__ __forceinline__ float pow_fix(const PowTab& t, float x, float v, int* status) {
    return pow_table_fix(t, x, v, status);
}

template <int MODE> struct Pw;
template <> struct Pw<MODE_REF> {
    static __device__ __forceinline__ float p4(const PowTab& t, float x, int* st) { return pow_fix(t, x, dev_pow4(x), st); }
    static __device__ __forceinline__ float p3(const PowTab& t, float x, int* st) { return pow_fix(t, x, dev_pow3(x), st); }
};
template <> struct Pw<MODE_FP64> {
    static __device__ __forceinline__ double p4(const PowTab&, double x, int*) {
        double t2 = __dmul_rn(x, x);
        return __dmul_rn(t2, t2);
    }
    static __device__ __forceinline__ double p3(const PowTab&, double x, int*) { return __dmul_rn(__dmul_rn(x, x), x); }
};
template <> struct Pw<MODE_FAST> {
    static __device__ __forceinline__ float p4(const PowTab&, float x, int*) { float t2 = x * x; return t2 * t2; }
    static __device__ __forceinline__ float p3(const PowTab&, float x, int*) { return x * x * x; }
};

// per-mode scalar views of DevSolve
template <int MODE> struct Sc {
    using R = typename Ar<MODE>::R;
    R ti, oma, es, es4, m1, r, tacc, tacc10, esw;
    __device__ __forceinline__ void load(const DevSolve& s) {
        if constexpr (MODE == MODE_FP64) {
            ti = s.ti_d; oma = s.oma_d; es = s.es_d; es4 = s.es4_d; m1 = s.m1_d; r = s.r_d;
            tacc = s.tacc_d; tacc10 = s.tacc10_d; esw = s.es_w_d;
        } else {
            ti = s.ti; oma = s.oma; es = s.es; es4 = s.es4; m1 = s.m1; r = s.r;
            tacc = s.tacc; tacc10 = s.tacc10; esw = s.es_w;
        }
    }
    // facet f's own rotation rate (the secondary of a non-synchronous binary)
    __device__ __forceinline__ void body(const DevSolve& s, int f) {
        if (f < s.fsplit) return;
        if constexpr (MODE == MODE_FP64) { m1 = s.m1_2_d; r = s.r2_d; }
        else { m1 = s.m1_2; r = s.r2; }
    }
};

// ------------------------------------------------------------- self-heating
// W[f][s] = (eps*sigma) * T[s][f]^4 over a 32x32 tile, transposed in shared memory
template <int MODE>
__global__ void __launch_bounds__(256) k_selfheat_w(Batch b) {
    using A = Ar<MODE>;
    using R = typename A::R;
    const int4 t = b.wmap[blockIdx.x];
    const DevSolve& sv = b.tab[t.x];
    if (!sv.ctl->active || sv.nnz == 0) return;
    __shared__ R sm[32][33];
    const int nf = sv.nf, ntau = sv.ntau;
    const R* T = static_cast<const R*>(sv.stemp1);
    R* W = static_cast<R*>(sv.W);
    Sc<MODE> c;
    c.load(sv);
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int s = t.z + j, f = t.y + threadIdx.x;
        R v = R(0);
        if (s < ntau && f < nf) v = A::mul(c.esw, Pw<MODE>::p4(b.p4, T[(size_t)s * nf + f], sv.status));
        sm[j][threadIdx.x] = v;
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int f = t.y + j, s = t.z + threadIdx.x;
        if (f < nf && s < ntau) W[(size_t)f * ntau + s] = sm[threadIdx.x][j];
    }
}

// Q[s][f] = sum over f's list of W[g][s] * vf, accumulated in list order
// (main.cpp:1519-1529).  Warp w of the block owns facet f0+w, lane l owns
// step s0+l, so the list loop is warp-uniform and every W load is a
// coalesced 128-byte row segment.
template <int MODE>
__global__ void __launch_bounds__(1024) k_selfheat_q(Batch b) {
    using A = Ar<MODE>;
    using R = typename A::R;
    const int4 t = b.wmap[blockIdx.x];
    const DevSolve& sv = b.tab[t.x];
    if (!sv.ctl->active) return;
    __shared__ R sm[32][33];
    const int nf = sv.nf, ntau = sv.ntau;
    const int f = t.y + threadIdx.y, s = t.z + threadIdx.x;
    const bool inst = (MODE == MODE_FP64) ? (sv.ti_d == 0.0) : (sv.ti == 0.0f);
    R q = R(0);
    if (f < nf && s < ntau && (inst || !sv.freeze || !sv.conv[f])) {
        const R* W = static_cast<const R*>(sv.W);
        const int k1 = sv.dep_ptr[f + 1];
        for (int k = sv.dep_ptr[f]; k < k1; ++k) {
            const int g = __ldg(&sv.dep_idx[k]);
            const R v = (R)__ldg(&sv.dep_vf[k]);
            q = A::add(q, A::mul(W[(size_t)g * ntau + s], v));
        }
    }
    sm[threadIdx.y][threadIdx.x] = q;
    __syncthreads();
    const int so = t.z + threadIdx.y, fo = t.y + threadIdx.x;
    if (so < ntau && fo < nf) static_cast<R*>(sv.Q)[(size_t)so * nf + fo] = sm[threadIdx.x][threadIdx.y];
}

// --------------------------------------------------------------- conduction
// One thread owns one facet's depth column (NX+1 nodes in registers) for a
// whole revolution.  Per step it reads E, Q and the previous-revolution
// surface temperature (coalesced across the warp), applies the FTCS update of
// main.cpp:1510-1515, the Newton boundary of main.cpp:1533-1542 and the
// Neumann bottom of main.cpp:1549, and records whether |stemp1-stemp0| >= TACC
// (the shape_converged test) so no stemp history has to be re-read.
template <int MODE, int NX>
__device__ __forceinline__ void column_revolution(const DevSolve& sv, const Batch& b, int f) {
    using A = Ar<MODE>;
    using R = typename A::R;
    const int nf = sv.nf, ntau = sv.ntau;
    Sc<MODE> c;
    c.load(sv);
    c.body(sv, f);
    R* temp = static_cast<R*>(sv.temp);
    const R* E = static_cast<const R*>(sv.E);
    const R* Q = static_cast<const R*>(sv.Q);
    R* S0 = static_cast<R*>(sv.stemp0);
    R* S1 = static_cast<R*>(sv.stemp1);
    R T[NX + 1];
#pragma unroll
    for (int i = 0; i <= NX; ++i) T[i] = temp[(size_t)i * nf + f];
    bool hot = false;
    const int cap = sv.newton_cap;
    int flags = 0;
    for (int s = 0; s < ntau; ++s) {
        const size_t o = (size_t)s * nf + f;
        const R old = S1[o];
        S0[o] = old;
        R t0 = T[0];
#pragma unroll
        for (int i = 1; i < NX; ++i) {
            const R t1 = T[i];
            T[i] = A::add(T[i], A::mul(c.r, A::add(A::sub(T[i + 1], A::mul(R(2), T[i])), t0)));
            t0 = t1;
        }
        const R a = A::add(A::mul(c.oma, E[o]), Q[o]);
        R TR0 = T[0], TR1 = T[0], DT = R(1);
        int it = 0;
        while (DT >= c.tacc10) {
            if (it == cap) { flags |= ST_NEWTON_CAP; break; }
            const R sbc = A::sub(A::add(a, A::mul(c.m1, A::sub(T[1], TR0))),
                                 A::mul(c.es, Pw<MODE>::p4(b.p4, TR0, sv.status)));
            const R sbcd = A::add(c.m1, A::mul(c.es4, Pw<MODE>::p3(b.p3, TR0, sv.status)));
            TR1 = A::add(TR0, A::div(sbc, sbcd));
            DT = A::fabs_(A::sub(TR1, TR0));
            TR0 = TR1;
            ++it;
        }
        T[0] = TR1;
        S1[o] = TR1;
        T[NX] = T[NX - 1];
        hot = hot || (A::fabs_(A::sub(TR1, old)) >= c.tacc);
        if (!isfinite(TR1)) flags |= ST_NONFINITE;
    }
#pragma unroll
    for (int i = 0; i <= NX; ++i) temp[(size_t)i * nf + f] = T[i];
    sv.hot[f] = hot ? 1 : 0;
    if (flags) atomicOr(sv.status, flags);
}

// FAST + tensor-core self-heating: eps*sigma*T^4 of the new surface
// temperature goes straight into the hi/lo BF16 tiles the next revolution's
// product reads (atpm_spmm_tc.cu), so no separate pass re-reads stemp1.
// FAST arithmetic is written with explicitly rounded operations (the _rn
// intrinsics are never contracted into a multiply-add), so the scalar, the
// warp-per-facet and the paired forms of the sweep round alike, operation by
// operation, whatever the compiler schedules.
// eps sigma T^4 (with the IR absorptivity folded into es_w)
__device__ __forceinline__ float fast_w(float es_w, float t) {
    const float t2 = __fmul_rn(t, t);
    return __fmul_rn(es_w, __fmul_rn(t2, t2));
}
// the BF16 pair of W: hi = bf16(w), lo = bf16(w - hi)
__device__ __forceinline__ __nv_bfloat16 w_lo(float w, __nv_bfloat16 hi) {
    return __float2bfloat16_rn(__fsub_rn(w, __bfloat162float(hi)));
}

__device__ __forceinline__ void store_w(const DevSolve& sv, int f, int s, float t) {
    const int N = sv.tc_n;
    const float w = fast_w(sv.es_w, t);
    __nv_bfloat16* W = static_cast<__nv_bfloat16*>(sv.Wb);
    const size_t base = ((size_t)(f >> 6) * sv.tc_nchunks + s / N) * (size_t)2 * N * 64;
    const uint32_t o = swz((uint32_t)(s % N), (uint32_t)(f & 63));
    const __nv_bfloat16 hi = __float2bfloat16_rn(w);
    W[base + o] = hi;
    W[base + (size_t)N * 64 + o] = w_lo(w, hi);
    if (sv.W32) sv.W32[(size_t)f * sv.w32_ld + s] = w;
}

// FAST precision: the same update, scheduled for the FP32 pipes.
//  * The column is advanced as offsets theta_i = T_i - T_ref from a per-facet
//    reference (the bottom node at the start of the revolution).  The FTCS
//    Laplacian is translation-invariant, so each step rounds to the ulp of
//    theta (a few K) instead of the ulp of T (~300 K): 10-100x less roundoff
//    than the reference's absolute FP32 update, which is what keeps the FAST
//    path within 0.01 K of FP64 over hundreds of revolutions.
//  * Node 1 is advanced first (the boundary solve needs it); the Newton
//    boundary runs two iterations unconditionally (more only while the change
//    is still >= TACC/10), and the update of nodes 2..NX-1 -- independent of
//    the boundary result -- sits in the same basic block, so the scheduler
//    overlaps it with the Newton dependency chain.
// per-thread asynchronous copies (cp.async, 4 bytes) for the step prefetch of
// the FAST sweep: each thread copies and later reads only its own words, so
// no block barrier is involved
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

constexpr int kFastPrefetch = 8;  // steps of forcing / flux / previous temperature in flight per facet

// One FTCS node update and one Newton step of the FAST sweep, shared by the
// thread-per-facet and the warp-per-facet forms so both round alike.
// (up + dn) - 2 t is formed as one fma: 2 t is exact, so this is the
// rounding of the plain expression
__device__ __forceinline__ float ftcs_node(float r, float up, float dn, float t) {
    return __fmaf_rn(r, __fmaf_rn(-2.0f, t, __fadd_rn(up, dn)), t);
}

// one Newton step on theta_0: sbc = (m1 (t1 - th) + a) - es TR^4 with the
// emission folded into one multiply-add
__device__ __forceinline__ float newton_fast(float th, float Tref, float t1, float a, float m1, float es, float es4,
                                             float& DT) {
    const float TR = __fadd_rn(Tref, th);
    const float t2 = __fmul_rn(TR, TR);
    const float sbc = __fmaf_rn(-es, __fmul_rn(t2, t2), __fmaf_rn(m1, __fsub_rn(t1, th), a));
    const float sbcd = __fmaf_rn(es4, __fmul_rn(t2, TR), m1);
    const float th1 = __fadd_rn(th, __fdividef(sbc, sbcd));
    DT = fabsf(__fsub_rn(th1, th));
    return th1;
}

template <int NX>
__device__ __forceinline__ void column_revolution_fast(const DevSolve& sv, int f) {
    const int nf = sv.nf, ntau = sv.ntau;
    const bool sec = f >= sv.fsplit;  // non-synchronous secondary: its own rotation rate
    const float r = sec ? sv.r2 : sv.r, oma = sv.oma, es = sv.es, es4 = sv.es4, m1 = sec ? sv.m1_2 : sv.m1,
                tacc = sv.tacc, tacc10 = sv.tacc10;
    float* temp = static_cast<float*>(sv.temp);
    const float* __restrict__ E = static_cast<const float*>(sv.E);
    const float* __restrict__ Q = static_cast<const float*>(sv.Q);
    float* __restrict__ S0 = static_cast<float*>(sv.stemp0);
    float* __restrict__ S1 = static_cast<float*>(sv.stemp1);
    float T[NX + 1];
    const float Tref = temp[(size_t)NX * nf + f];
    // W tile addressing, advanced incrementally (no per-step division)
    __nv_bfloat16* Wb = static_cast<__nv_bfloat16*>(sv.Wb);
    const int N = sv.tc_n;
    const size_t chunk = (size_t)2 * N * 64;
    size_t wrow = Wb ? (size_t)(f >> 6) * sv.tc_nchunks * chunk : 0;
    const uint32_t kc = (uint32_t)(f & 63) >> 3, k7 = (uint32_t)f & 7u;
    int wn = 0;
#pragma unroll
    for (int i = 0; i <= NX; ++i) T[i] = __fsub_rn(temp[(size_t)i * nf + f], Tref);
    bool hot = false;
    int flags = 0;
    const int cap = sv.newton_cap;
    // E, Q and the previous temperature of step s + kFastPrefetch are copied
    // into this thread's shared-memory slots while step s computes: in the
    // late revolutions a few active facets per SM cannot hide DRAM latency
    // behind other warps
    constexpr int D = kFastPrefetch;
    __shared__ float pre[D][3][128];
    // the last 8 values of eps sigma T^4, written to this facet's W32 row
    // as two 16-byte stores per 8 steps (one full 32-byte sector)
    __shared__ float w8[8][128];
    float* W32 = Wb ? sv.W32 : nullptr;
    float* w32row = W32 ? W32 + (size_t)f * sv.w32_ld : nullptr;
    const int lt = threadIdx.x;
    for (int j = 0; j < D; ++j) {
        if (j < ntau) {
            const size_t oj = (size_t)j * nf + f;
            cp_async4(&pre[j][0][lt], E + oj);
            cp_async4(&pre[j][1][lt], Q + oj);
            cp_async4(&pre[j][2][lt], S1 + oj);
        }
        cp_async_commit();
    }
    size_t o = (size_t)f;
    int slot = 0;
    for (int s = 0; s < ntau; ++s, o += nf) {
        cp_async_wait<D - 1>();  // the copies of step s have landed
        const float e = pre[slot][0][lt], q = pre[slot][1][lt], old = pre[slot][2][lt];
        S0[o] = old;
        const float t1 = T[1];
        T[1] = ftcs_node(r, T[2], T[0], t1);
        const float a = __fmaf_rn(oma, e, q);
        // Newton iterations 1 and 2 on theta_0 (T_0 = Tref + theta_0)
        float DT;
        float th1 = newton_fast(T[0], Tref, T[1], a, m1, es, es4, DT);
        if (DT >= tacc10) th1 = newton_fast(th1, Tref, T[1], a, m1, es, es4, DT);
        // remaining nodes (independent of the boundary result)
        float tm = t1;
#pragma unroll
        for (int i = 2; i < NX; ++i) {
            const float ti = T[i];
            T[i] = ftcs_node(r, T[i + 1], tm, ti);
            tm = ti;
        }
        int it = 2;
        while (DT >= tacc10) {
            if (it >= cap) { flags |= ST_NEWTON_CAP; break; }
            th1 = newton_fast(th1, Tref, T[1], a, m1, es, es4, DT);
            ++it;
        }
        T[0] = th1;
        const float Tsurf = __fadd_rn(Tref, th1);
        S1[o] = Tsurf;
        if (Wb) {
            const float w = fast_w(sv.es_w, Tsurf);
            const uint32_t off = (uint32_t)wn * 64u + ((kc ^ ((uint32_t)wn & 7u)) << 3) + k7;
            const __nv_bfloat16 hi = __float2bfloat16_rn(w);
            Wb[wrow + off] = hi;
            Wb[wrow + (size_t)N * 64 + off] = w_lo(w, hi);
            if (++wn == N) { wn = 0; wrow += chunk; }
            if (w32row) {
                w8[s & 7][lt] = w;
                if ((s & 7) == 7) {
                    float4* d = reinterpret_cast<float4*>(w32row + (s - 7));
                    d[0] = make_float4(w8[0][lt], w8[1][lt], w8[2][lt], w8[3][lt]);
                    d[1] = make_float4(w8[4][lt], w8[5][lt], w8[6][lt], w8[7][lt]);
                }
            }
        }
        T[NX] = T[NX - 1];
        hot = hot || (fabsf(__fsub_rn(Tsurf, old)) >= tacc);
        // refill the slot just read (its words are consumed) with step s + D
        if (s + D < ntau) {
            const size_t od = o + (size_t)D * nf;
            cp_async4(&pre[slot][0][lt], E + od);
            cp_async4(&pre[slot][1][lt], Q + od);
            cp_async4(&pre[slot][2][lt], S1 + od);
        }
        cp_async_commit();
        if (++slot == D) slot = 0;
    }
    cp_async_wait<0>();
    if (w32row)  // the steps after the last full group of 8
        for (int s = ntau & ~7; s < ntau; ++s) w32row[s] = w8[s & 7][lt];
    if (!isfinite(__fadd_rn(T[0], Tref))) flags |= ST_NONFINITE;
#pragma unroll
    for (int i = 0; i <= NX; ++i) temp[(size_t)i * nf + f] = __fadd_rn(Tref, T[i]);
    sv.hot[f] = hot ? 1 : 0;
    if (flags) atomicOr(sv.status, flags);
}

// FAST, two adjacent facets per thread.  The sweep is issue-bound, so the
// pair is advanced with the packed FP32 instructions (fma/add/mul .f32x2):
// each lane of a pair is the scalar sweep's operation sequence with the same
// roundings, so both facets end bit-identical to column_revolution_fast.  The
// two facets' words sit side by side in every [step][facet] and
// [depth][facet] array (f even, nf even), so their loads and stores are
// 8-byte accesses and the two W tile entries one BF16x2 store.  The Newton
// solve runs while either lane still needs a step; a lane that has stopped
// keeps its value (per-lane select), so each facet takes its own iterations.
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
// a - b with one rounding (b * -1 is exact), the value of __fsub_rn(a, b)
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }

__device__ __forceinline__ float2 ftcs_node2(float2 r, float2 up, float2 dn, float2 t) {
    return f2fma(r, f2fma(make_float2(-2.0f, -2.0f), t, f2add(up, dn)), t);
}

// newton_fast on both lanes (nes = -es)
__device__ __forceinline__ float2 newton_fast2(float2 th, float2 Tref, float2 t1, float2 a, float2 m1, float2 nes,
                                               float2 es4, float2& DT) {
    const float2 TR = f2add(Tref, th);
    const float2 t2 = f2mul(TR, TR);
    const float2 sbc = f2fma(nes, f2mul(t2, t2), f2fma(m1, f2sub(t1, th), a));
    const float2 sbcd = f2fma(es4, f2mul(t2, TR), m1);
    const float2 th1 = f2add(th, make_float2(__fdividef(sbc.x, sbcd.x), __fdividef(sbc.y, sbcd.y)));
    const float2 d = f2sub(th1, th);
    DT = make_float2(fabsf(d.x), fabsf(d.y));
    return th1;
}

__device__ __forceinline__ void cp_async8(float2* dst, const float* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}

template <int NX>
__device__ __forceinline__ void column_revolution_fast2(const DevSolve& sv, int f) {
    const int nf = sv.nf, ntau = sv.ntau;
    const bool sec0 = f >= sv.fsplit, sec1 = f + 1 >= sv.fsplit;
    const float2 r = make_float2(sec0 ? sv.r2 : sv.r, sec1 ? sv.r2 : sv.r);
    const float2 m1 = make_float2(sec0 ? sv.m1_2 : sv.m1, sec1 ? sv.m1_2 : sv.m1);
    const float2 oma = make_float2(sv.oma, sv.oma), nes = make_float2(-sv.es, -sv.es),
                 es4 = make_float2(sv.es4, sv.es4), esw = make_float2(sv.es_w, sv.es_w);
    const float tacc = sv.tacc, tacc10 = sv.tacc10;
    float* temp = static_cast<float*>(sv.temp);
    const float* __restrict__ E = static_cast<const float*>(sv.E);
    const float* __restrict__ Q = static_cast<const float*>(sv.Q);
    float* __restrict__ S0 = static_cast<float*>(sv.stemp0);
    float* __restrict__ S1 = static_cast<float*>(sv.stemp1);
    float2 T[NX + 1];
    const float2 Tref = *reinterpret_cast<const float2*>(temp + (size_t)NX * nf + f);
    __nv_bfloat16* Wb = static_cast<__nv_bfloat16*>(sv.Wb);
    const int N = sv.tc_n;
    const size_t chunk = (size_t)2 * N * 64;
    size_t wrow = Wb ? (size_t)(f >> 6) * sv.tc_nchunks * chunk : 0;
    const uint32_t kc = (uint32_t)(f & 63) >> 3, k7 = (uint32_t)f & 7u;  // f even: f + 1 is the next BF16
    int wn = 0;
#pragma unroll
    for (int i = 0; i <= NX; ++i) T[i] = f2sub(*reinterpret_cast<const float2*>(temp + (size_t)i * nf + f), Tref);
    bool hot0 = false, hot1 = false;
    int flags = 0;
    const int cap = sv.newton_cap;
    constexpr int D = kFastPrefetch;
    __shared__ float2 pre2[D][3][64];
    __shared__ float2 w8p[8][64];
    float* W32 = Wb ? sv.W32 : nullptr;
    float* w32r0 = W32 ? W32 + (size_t)f * sv.w32_ld : nullptr;
    float* w32r1 = W32 ? w32r0 + sv.w32_ld : nullptr;
    const int lt = threadIdx.x;
    for (int j = 0; j < D; ++j) {
        if (j < ntau) {
            const size_t oj = (size_t)j * nf + f;
            cp_async8(&pre2[j][0][lt], E + oj);
            cp_async8(&pre2[j][1][lt], Q + oj);
            cp_async8(&pre2[j][2][lt], S1 + oj);
        }
        cp_async_commit();
    }
    size_t o = (size_t)f;
    int slot = 0;
    for (int s = 0; s < ntau; ++s, o += nf) {
        cp_async_wait<D - 1>();
        const float2 e = pre2[slot][0][lt], q = pre2[slot][1][lt], old = pre2[slot][2][lt];
        *reinterpret_cast<float2*>(S0 + o) = old;
        const float2 t1 = T[1];
        T[1] = ftcs_node2(r, T[2], T[0], t1);
        const float2 a = f2fma(oma, e, q);
        float2 DT;
        float2 th1 = newton_fast2(T[0], Tref, T[1], a, m1, nes, es4, DT);
        {
            const bool n0 = DT.x >= tacc10, n1 = DT.y >= tacc10;
            if (n0 || n1) {
                float2 d2;
                const float2 t = newton_fast2(th1, Tref, T[1], a, m1, nes, es4, d2);
                if (n0) { th1.x = t.x; DT.x = d2.x; }
                if (n1) { th1.y = t.y; DT.y = d2.y; }
            }
        }
        float2 tm = t1;
#pragma unroll
        for (int i = 2; i < NX; ++i) {
            const float2 ti = T[i];
            T[i] = ftcs_node2(r, T[i + 1], tm, ti);
            tm = ti;
        }
        for (int it = 2;; ++it) {
            const bool n0 = DT.x >= tacc10, n1 = DT.y >= tacc10;
            if (!n0 && !n1) break;
            if (it >= cap) { flags |= ST_NEWTON_CAP; break; }
            float2 d2;
            const float2 t = newton_fast2(th1, Tref, T[1], a, m1, nes, es4, d2);
            if (n0) { th1.x = t.x; DT.x = d2.x; }
            if (n1) { th1.y = t.y; DT.y = d2.y; }
        }
        T[0] = th1;
        const float2 Tsurf = f2add(Tref, th1);
        *reinterpret_cast<float2*>(S1 + o) = Tsurf;
        if (Wb) {
            const float2 t2s = f2mul(Tsurf, Tsurf);
            const float2 w = f2mul(esw, f2mul(t2s, t2s));
            const uint32_t off = (uint32_t)wn * 64u + ((kc ^ ((uint32_t)wn & 7u)) << 3) + k7;
            const __nv_bfloat162 hi = __floats2bfloat162_rn(w.x, w.y);
            const float2 lo = f2sub(w, __bfloat1622float2(hi));
            *reinterpret_cast<__nv_bfloat162*>(Wb + wrow + off) = hi;
            *reinterpret_cast<__nv_bfloat162*>(Wb + wrow + (size_t)N * 64 + off) = __floats2bfloat162_rn(lo.x, lo.y);
            if (++wn == N) { wn = 0; wrow += chunk; }
            if (w32r0) {
                w8p[s & 7][lt] = w;
                if ((s & 7) == 7) {
                    float4* d0 = reinterpret_cast<float4*>(w32r0 + (s - 7));
                    float4* d1 = reinterpret_cast<float4*>(w32r1 + (s - 7));
                    d0[0] = make_float4(w8p[0][lt].x, w8p[1][lt].x, w8p[2][lt].x, w8p[3][lt].x);
                    d0[1] = make_float4(w8p[4][lt].x, w8p[5][lt].x, w8p[6][lt].x, w8p[7][lt].x);
                    d1[0] = make_float4(w8p[0][lt].y, w8p[1][lt].y, w8p[2][lt].y, w8p[3][lt].y);
                    d1[1] = make_float4(w8p[4][lt].y, w8p[5][lt].y, w8p[6][lt].y, w8p[7][lt].y);
                }
            }
        }
        T[NX] = T[NX - 1];
        const float2 dT = f2sub(Tsurf, old);
        hot0 = hot0 || (fabsf(dT.x) >= tacc);
        hot1 = hot1 || (fabsf(dT.y) >= tacc);
        if (s + D < ntau) {
            const size_t od = o + (size_t)D * nf;
            cp_async8(&pre2[slot][0][lt], E + od);
            cp_async8(&pre2[slot][1][lt], Q + od);
            cp_async8(&pre2[slot][2][lt], S1 + od);
        }
        cp_async_commit();
        if (++slot == D) slot = 0;
    }
    cp_async_wait<0>();
    if (w32r0)
        for (int s = ntau & ~7; s < ntau; ++s) {
            w32r0[s] = w8p[s & 7][lt].x;
            w32r1[s] = w8p[s & 7][lt].y;
        }
    const float2 t0 = f2add(T[0], Tref);
    if (!isfinite(t0.x) || !isfinite(t0.y)) flags |= ST_NONFINITE;
#pragma unroll
    for (int i = 0; i <= NX; ++i) *reinterpret_cast<float2*>(temp + (size_t)i * nf + f) = f2add(Tref, T[i]);
    sv.hot[f] = hot0 ? 1 : 0;
    sv.hot[f + 1] = hot1 ? 1 : 0;
    if (flags) atomicOr(sv.status, flags);
}

// FAST, late revolutions: one warp per active facet.  Lane l holds depth
// nodes 2l and 2l+1 (theta offsets, as above), and every lane also carries
// nodes 0..3, so a step's boundary chain (node 1, then the Newton solve)
// waits on no shuffle: the new node 3 and the next step's absorbed flux are
// shuffled while the Newton solve runs.  The bottom node is a copy of node
// NX-1 after every step, so node NX-1 reads its own old value for it and the
// bottom is written once, after the revolution.  The arithmetic is that of
// column_revolution_fast step for step.  Forcing, flux and the previous
// temperature come in blocks of 32 steps (lane j holds step s0 + j, the next
// block loading while this one runs); the step's outputs collect in the lane
// of that step and are stored once per block.
constexpr int kWarpNodes = 64;  // nodes 0..NX a warp can hold

template <int NX>
__device__ __forceinline__ void column_revolution_warp(const DevSolve& sv, int f) {
    static_assert(NX + 1 <= kWarpNodes, "two nodes per lane");
    static_assert(NX >= 4, "nodes 0..3 above the bottom node");
    constexpr unsigned FULL = 0xffffffffu;
    const int nf = sv.nf, ntau = sv.ntau;
    const int lane = threadIdx.x & 31;
    const bool sec = f >= sv.fsplit;
    const float r = sec ? sv.r2 : sv.r, oma = sv.oma, es = sv.es, es4 = sv.es4, m1 = sec ? sv.m1_2 : sv.m1,
                tacc = sv.tacc, tacc10 = sv.tacc10;
    float* temp = static_cast<float*>(sv.temp);
    const float* __restrict__ E = static_cast<const float*>(sv.E);
    const float* __restrict__ Q = static_cast<const float*>(sv.Q);
    float* __restrict__ S0 = static_cast<float*>(sv.stemp0);
    float* __restrict__ S1 = static_cast<float*>(sv.stemp1);
    __nv_bfloat16* Wb = static_cast<__nv_bfloat16*>(sv.Wb);
    const int N = sv.tc_n;
    const int na = 2 * lane, nb = 2 * lane + 1;
    const float Tref = temp[(size_t)NX * nf + f];
    float Ta = na <= NX ? __fsub_rn(temp[(size_t)na * nf + f], Tref) : 0.0f;
    float Tb = nb <= NX ? __fsub_rn(temp[(size_t)nb * nf + f], Tref) : 0.0f;
    bool hot = false;
    int flags = 0;
    const int cap = sv.newton_cap;
    // nodes 0..3 on every lane (lane 0 owns 0 and 1, lane 1 owns 2 and 3)
    float th_u = __shfl_sync(FULL, Ta, 0), t1_u = __shfl_sync(FULL, Tb, 0);
    float t2_u = __shfl_sync(FULL, Ta, 1), t3_u = __shfl_sync(FULL, Tb, 1);
    // lane j: (1 - A) E + Q and the previous surface temperature of step s0 + j
    float ca = 0.0f, co = 0.0f;
    if (lane < ntau) {
        const size_t o = (size_t)lane * nf + f;
        ca = __fmaf_rn(oma, E[o], Q[o]);
        co = S1[o];
    }
    for (int s0 = 0; s0 < ntau; s0 += 32) {
        float ne = 0.0f, nq = 0.0f, no = 0.0f;
        if (s0 + 32 + lane < ntau) {
            const size_t o = (size_t)(s0 + 32 + lane) * nf + f;
            ne = E[o];
            nq = Q[o];
            no = S1[o];
        }
        float ts = 0.0f;
        const int nstep = min(32, ntau - s0);
        float a = __shfl_sync(FULL, ca, 0);
#pragma unroll 4
        for (int j = 0; j < nstep; ++j) {
            const float old = __shfl_sync(FULL, co, j);
            const float a_next = __shfl_sync(FULL, ca, (j + 1) & 31);  // unused after the block's last step
            const float lft = __shfl_up_sync(FULL, Tb, 1);    // node na - 1
            const float rgt = __shfl_down_sync(FULL, Ta, 1);  // node nb + 1
            // nodes 2 .. NX-1 from old values; node NX-1 reads itself for the bottom
            float Ta_n = Ta, Tb_n = Tb;
            if (na >= 2 && na <= NX - 1) Ta_n = ftcs_node(r, Tb, lft, Ta);
            if (nb >= 2 && nb <= NX - 1) Tb_n = ftcs_node(r, nb == NX - 1 ? Tb : rgt, Ta, Tb);
            if (nb == NX) Tb_n = Ta_n;  // odd NX: the bottom copy beside node NX-1
            // nodes 1 and 2 on every lane (uniform values)
            const float t1n = ftcs_node(r, t2_u, th_u, t1_u);
            const float t2n = ftcs_node(r, t3_u, t1_u, t2_u);
            if (lane == 0) Tb_n = t1n;  // node 1, read by lane 1 next step
            const float t3n = __shfl_sync(FULL, Tb_n, 1);
            // the boundary solve on every lane
            float DT;
            float th1 = newton_fast(th_u, Tref, t1n, a, m1, es, es4, DT);
            if (DT >= tacc10) th1 = newton_fast(th1, Tref, t1n, a, m1, es, es4, DT);
            int it = 2;
            while (DT >= tacc10) {
                if (it >= cap) { flags |= ST_NEWTON_CAP; break; }
                th1 = newton_fast(th1, Tref, t1n, a, m1, es, es4, DT);
                ++it;
            }
            Ta = Ta_n;
            Tb = Tb_n;
            th_u = th1;
            t1_u = t1n;
            t2_u = t2n;
            t3_u = t3n;
            a = a_next;
            const float Tsurf = __fadd_rn(Tref, th1);
            if (lane == j) ts = Tsurf;
            hot = hot || (fabsf(__fsub_rn(Tsurf, old)) >= tacc);
        }
        if (lane < nstep) {
            const int s = s0 + lane;
            const size_t o = (size_t)s * nf + f;
            S0[o] = co;
            S1[o] = ts;
            if (Wb) {
                const float w = fast_w(sv.es_w, ts);
                const size_t base = ((size_t)(f >> 6) * sv.tc_nchunks + s / N) * (size_t)2 * N * 64;
                const uint32_t off = swz((uint32_t)(s % N), (uint32_t)(f & 63));
                const __nv_bfloat16 hi = __float2bfloat16_rn(w);
                Wb[base + off] = hi;
                Wb[base + (size_t)N * 64 + off] = w_lo(w, hi);
                if (sv.W32) sv.W32[(size_t)f * sv.w32_ld + s] = w;  // 32 lanes: one 128-byte row segment
            }
        }
        ca = __fmaf_rn(oma, ne, nq);
        co = no;
    }
    if (!isfinite(__fadd_rn(th_u, Tref))) flags |= ST_NONFINITE;
    if (lane == 0) Ta = th_u;  // node 0 lives in the uniform copy during the sweep
    if constexpr ((NX & 1) == 0) {
        const float bot = __shfl_sync(FULL, Tb, (NX - 1) >> 1);  // node NX-1
        if (lane == (NX >> 1)) Ta = bot;
    }
    if (na <= NX) temp[(size_t)na * nf + f] = __fadd_rn(Tref, Ta);
    if (nb <= NX) temp[(size_t)nb * nf + f] = __fadd_rn(Tref, Tb);
    if (lane == 0) {
        sv.hot[f] = hot ? 1 : 0;
        if (flags) atomicOr(sv.status, flags);
    }
}

// A revolution of the batch runs warp per facet when every active solve with
// a depth sweep (TI > 0) freezes converged facets, fits a warp's nodes and
// has the list of its active facets built for this revolution, and those
// lists hold at most b.tail_limit facets together.  k_tail_mode decides once
// per revolution (one warp over the solves) and leaves the answer in the
// batch's first solve (act_cnt[4]), where both conduction kernels read it:
// exactly one of them advances each facet.
__global__ void k_tail_mode(Batch b) {
    const int lane = threadIdx.x;
    bool ok = b.warp_tail != 0;
    int total = 0;
    for (int i = lane; i < b.n; i += 32) {
        const DevSolve& s = b.tab[i];
        if (!s.ctl->active || s.ti == 0.0f) continue;
        const int rev = s.ctl->rev;
        if (!s.freeze || s.nx + 1 > kWarpNodes || rev < 7 || s.act_cnt[2 + (rev & 1)] != rev) ok = false;
        else total += s.act_cnt[rev & 1];
    }
    ok = __all_sync(0xffffffffu, ok);
    for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
    if (lane == 0) b.tab[0].act_cnt[4] = (ok && total <= b.tail_limit) ? 1 : 0;
}

__device__ __forceinline__ bool warp_tail_now(const Batch& b) { return b.tab[0].act_cnt[4] != 0; }

// CTAs (4 warps each) per solve: in the late revolutions most active facets
// belong to the one or two solves of highest thermal inertia, so one solve
// may hold most of the batch's b.tail_limit facets (12 per SM, 1,824 on 152
// SMs); 384 x 4 = 1,536 warps give nearly every one of them its own warp, and
// the CTAs beyond a solve's list exit at once
constexpr int kSparseCtas = 384;

template <int NX>
__global__ void __launch_bounds__(128) k_conduction_warp(Batch b) {
    const int si = blockIdx.x / kSparseCtas;
    // the batch-wide decision first: one load, and most revolutions stop here
    if (si >= b.n || !b.warp_tail || !warp_tail_now(b)) return;
    const DevSolve& sv = b.tab[si];
    if (!sv.ctl->active || sv.ti == 0.0f) return;
    const int rev = sv.ctl->rev;
    if (rev < 7 || sv.act_cnt[2 + (rev & 1)] != rev || sv.act_cnt[rev & 1] == 0) return;
    if constexpr (NX + 1 <= kWarpNodes) {
        const int n = sv.act_cnt[rev & 1];
        const int* list = sv.act_list + (size_t)(rev & 1) * sv.nf;
        for (int k = (blockIdx.x % kSparseCtas) * 4 + (threadIdx.x >> 5); k < n; k += 4 * kSparseCtas)
            column_revolution_warp<NX>(sv, list[k]);
    }
}

// instequilibrium (main.cpp:1563-1612): every facet, every step, no depth
template <int MODE>
__device__ __forceinline__ void column_equilibrium(const DevSolve& sv, const Batch& b, int f) {
    using A = Ar<MODE>;
    using R = typename A::R;
    const int nf = sv.nf, ntau = sv.ntau;
    Sc<MODE> c;
    c.load(sv);
    const R* E = static_cast<const R*>(sv.E);
    const R* Q = static_cast<const R*>(sv.Q);
    R* S0 = static_cast<R*>(sv.stemp0);
    R* S1 = static_cast<R*>(sv.stemp1);
    bool hot = false;
    for (int s = 0; s < ntau; ++s) {
        const size_t o = (size_t)s * nf + f;
        const R old = S1[o];
        S0[o] = old;
        const R x = A::div(A::add(A::mul(c.oma, E[o]), Q[o]), c.es);
        R tn;
        if constexpr (MODE == MODE_FP64) tn = sqrt(sqrt(x));
        else if constexpr (MODE == MODE_REF) tn = pow_fix(b.pq, x, dev_qroot(x), sv.status);  // powf(x, 0.25f)
        else tn = dev_qroot(x);
        S1[o] = tn;
        if constexpr (MODE == MODE_FAST) {
            if (sv.Wb) store_w(sv, f, s, tn);
        }
        hot = hot || (A::fabs_(A::sub(tn, old)) >= c.tacc);
    }
    sv.hot[f] = hot ? 1 : 0;
}

// the solve sweeps its list of active facets this revolution (at most half
// of them active, freeze protocol, list built for this revolution)
__device__ __forceinline__ bool list_mode(const Batch& b, const DevSolve& sv) {
    const int rev = sv.ctl->rev;
    return b.warp_tail && sv.freeze && rev >= 7 && sv.act_cnt[2 + (rev & 1)] == rev && 2 * sv.act_cnt[rev & 1] <= sv.nf;
}
// the facet-range sweep of this solve runs as pairs (variant 4, even facet
// count) while at least 90 % of its facets are active: once facets freeze,
// pairs split and their other halves would fall to the scalar sweep, so the
// whole range goes back to it.  Both kernels read the same list count
// (written by the previous revolution's convergence test), so exactly one
// of them takes each facet.
__device__ __forceinline__ bool pairs_here(const Batch& b, const DevSolve& sv) {
    if (b.cond_variant != 4 || (sv.nf & 1)) return false;
    const int rev = sv.ctl->rev;
    // no count for this revolution (every facet active before revolution 7,
    // or no lists kept): pairs; split pairs fall to the scalar sweep
    if (!sv.freeze || rev < 7 || sv.act_cnt[2 + (rev & 1)] != rev) return true;
    return 10 * sv.act_cnt[rev & 1] >= 9 * sv.nf;
}

// MINB: minimum resident blocks per SM requested from the register allocator
// (FAST only; the variants trade registers for occupancy, picked at run time)
template <int MODE, int NX, int MINB = 1>
__global__ void __launch_bounds__(128, MINB) k_conduction(Batch b) {
    const int2 fb = b.fmap[blockIdx.x];
    const DevSolve& sv = b.tab[fb.x];
    if (!sv.ctl->active) return;
    if constexpr (MODE == MODE_FAST) {
        if (sv.ti != 0.0f) {
            if (warp_tail_now(b)) return;  // k_conduction_warp runs this revolution
            // at most half the facets active: the solve's blocks sweep its
            // list of active facets instead of its facet range, so active
            // facets fill whole warps and the remaining blocks exit
            const int rev = sv.ctl->rev;
            if (list_mode(b, sv)) {
                const int k = fb.y + threadIdx.x;
                if (k >= sv.act_cnt[rev & 1]) return;
                column_revolution_fast<NX>(sv, sv.act_list[(size_t)(rev & 1) * sv.nf + k]);
                return;
            }
        }
    }
    const int f = fb.y + threadIdx.x;
    if (f >= sv.nf) return;
    if constexpr (MODE == MODE_FAST) {
        // k_conduction_pairs sweeps the pairs whose facets are both active;
        // a facet whose partner is frozen is swept here
        if (sv.ti != 0.0f && pairs_here(b, sv) && !(sv.freeze && sv.conv[f ^ 1])) return;
    }
    const bool inst = (MODE == MODE_FP64) ? (sv.ti_d == 0.0) : (sv.ti == 0.0f);
    if (inst) { column_equilibrium<MODE>(sv, b, f); return; }
    if (sv.freeze && sv.conv[f]) return;
    if constexpr (MODE == MODE_FAST) {
        column_revolution_fast<NX>(sv, f);
    }
    else column_revolution<MODE, NX>(sv, b, f);
}

// FAST conduction variant 4: the facet-range sweep (every revolution before
// the active-list and warp-per-facet forms take over) as pairs of adjacent
// facets, 64 threads per 128-facet block.  Only pairs with both facets
// active are swept here: k_conduction, launched beside it, takes a facet
// whose partner is frozen (the freeze flags do not change during the sweep),
// and every facet of a solve with an odd facet count.
template <int NX>
__global__ void __launch_bounds__(64, 4) k_conduction_pairs(Batch b) {
    const int2 fb = b.fmap[blockIdx.x];
    const DevSolve& sv = b.tab[fb.x];
    if (!sv.ctl->active || sv.ti == 0.0f || !pairs_here(b, sv) || warp_tail_now(b) || list_mode(b, sv)) return;
    const int f = fb.y + 2 * threadIdx.x;
    if (f >= sv.nf || (sv.freeze && (sv.conv[f] || sv.conv[f + 1]))) return;
    column_revolution_fast2<NX>(sv, f);
}

// -------------------------------------------------------------- convergence
__global__ void __launch_bounds__(128) k_converge(Batch b) {
    const int2 fb = b.fmap[blockIdx.x];
    const DevSolve& sv = b.tab[fb.x];
    if (!sv.ctl->active) return;
    const int rev = sv.ctl->rev;
    if (rev <= 5) return;
    const int f = fb.y + threadIdx.x;
    int c = 0;
    if (f < sv.nf) {
        const bool ok = !sv.hot[f];
        if (ok) { sv.conv[f] = 1; c = 1; }
    }
    c = __syncthreads_count(c);
    if (threadIdx.x == 0 && c) atomicAdd(&sv.counts[rev], c);
    // row-block activity read by the next revolution's tensor-core product
    // (blocks of this kernel are the product's 128-facet row blocks)
    const int any = __syncthreads_or(f < sv.nf && !sv.conv[f]);
    if (threadIdx.x == 0) sv.rb_act[fb.y >> 7] = any ? 1 : 0;
    // list of the facets still active for the next revolution (FAST, freeze):
    // each block appends its active facets as one segment in facet order, so
    // a sweep over the list keeps runs of neighbouring facets together
    if (b.mode == MODE_FAST && sv.freeze) {
        __shared__ int wcnt[4], base;
        const bool act = f < sv.nf && !sv.conv[f];
        const unsigned m = __ballot_sync(0xffffffffu, act);
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (lane == 0) wcnt[warp] = __popc(m);
        __syncthreads();
        if (threadIdx.x == 0) {
            const int t = wcnt[0] + wcnt[1] + wcnt[2] + wcnt[3];
            base = t ? atomicAdd(&sv.act_cnt[(rev + 1) & 1], t) : 0;
            if (fb.y == 0) sv.act_cnt[2 + ((rev + 1) & 1)] = rev + 1;
        }
        __syncthreads();
        int off = base;
        for (int w = 0; w < warp; ++w) off += wcnt[w];
        if (act) sv.act_list[(size_t)((rev + 1) & 1) * sv.nf + off + __popc(m & ((1u << lane) - 1u))] = f;
    }
}

__global__ void k_advance(Batch b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.n) return;
    const DevSolve& sv = b.tab[i];
    Ctl* ctl = sv.ctl;
    if (!ctl->active) return;
    const int rev = ctl->rev;
    if (rev > 5) {
        const int n = sv.counts[rev];
        ctl->numconv = n;
        ctl->converged = (n == sv.nf) ? 1 : 0;
    } else {
        sv.counts[rev] = ctl->numconv;
    }
    // read by this revolution's conduction; k_converge of rev + 1 refills it
    sv.act_cnt[rev & 1] = 0;
    sv.act_cnt[2 + (rev & 1)] = -1;
    ctl->rev = rev + 1;
    if (ctl->converged || rev + 1 >= sv.revcap || (*sv.status & ST_NONFINITE)) ctl->active = 0;
}

// ------------------------------------------------------------- initial state
template <int MODE>
__global__ void k_initial_mean(DevSolve sv, void* out) {
    using A = Ar<MODE>;
    using R = typename A::R;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= sv.nf) return;
    const R* E = static_cast<const R*>(sv.E);
    const R inv = A::div(R(1), (R)sv.ntau);
    R t = R(0);
    for (int s = 0; s < sv.ntau; ++s) t = A::add(t, A::mul(inv, E[(size_t)s * sv.nf + f]));
    static_cast<R*>(out)[f] = t;
}

// initialisetemperatures (main.cpp:1455-1462): the facet's mean absorbed
// flux -> T0 = ((1 - A) mean / (eps sigma))^0.25 everywhere in its column
template <int MODE>
__global__ void k_fill_initial(DevSolve sv, const void* mean, PowTab pq) {
    using R = typename Ar<MODE>::R;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= sv.nf) return;
    const R m = static_cast<const R*>(mean)[f];
    R v;
    if constexpr (MODE == MODE_FP64) {
        v = sqrt(sqrt(__ddiv_rn(__dmul_rn(sv.oma_d, m), sv.es_d)));
    } else {
        const float x = __fdiv_rn(__fmul_rn(sv.oma, m), sv.es);
        v = (MODE == MODE_REF) ? pow_fix(pq, x, dev_qroot(x), sv.status) : dev_qroot(x);  // powf(x, 0.25f)
    }
    R* temp = static_cast<R*>(sv.temp);
    R* S0 = static_cast<R*>(sv.stemp0);
    R* S1 = static_cast<R*>(sv.stemp1);
    for (int i = 0; i <= sv.nx; ++i) temp[(size_t)i * sv.nf + f] = v;
    for (int s = 0; s < sv.ntau; ++s) { S0[(size_t)s * sv.nf + f] = v; S1[(size_t)s * sv.nf + f] = v; }
}

// FP64 energy balance of the current revolution: sums over facets and steps
// of absorbed flux (1-A)E + Q, emitted eps*sigma*T^4 and T.
template <int MODE>
__global__ void k_energy(DevSolve sv) {
    using R = typename Ar<MODE>::R;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    double ab = 0.0, em = 0.0, tm = 0.0;
    if (f < sv.nf) {
        const R* E = static_cast<const R*>(sv.E);
        const R* Q = static_cast<const R*>(sv.Q);
        const R* S1 = static_cast<const R*>(sv.stemp1);
        const double oma = 1.0 - (double)sv.alb_d, es = sv.es_d;
        for (int s = 0; s < sv.ntau; ++s) {
            const size_t o = (size_t)s * sv.nf + f;
            const double T = (double)S1[o];
            ab += oma * (double)E[o] + (double)Q[o];
            em += es * (T * T) * (T * T);
            tm += T;
        }
    }
    for (int d = 16; d > 0; d >>= 1) {
        ab += __shfl_down_sync(0xffffffffu, ab, d);
        em += __shfl_down_sync(0xffffffffu, em, d);
        tm += __shfl_down_sync(0xffffffffu, tm, d);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&sv.diag[0], ab);
        atomicAdd(&sv.diag[1], em);
        atomicAdd(&sv.diag[2], tm);
    }
}

// ------------------------------------------------------------------ launchers
#define NX_LIST(X) X(8) X(12) X(16) X(24) X(32) X(40) X(48) X(56) X(64)

bool conduction_nx_supported(int nx) {
#define NX_CASE(n) if (nx == n) return true;
    NX_LIST(NX_CASE)
#undef NX_CASE
    return false;
}

template <int MODE>
static int launch_rev_part(const Batch& b, int part, cudaStream_t st) {
    // FAST + tensor cores: the conduction sweep keeps W current (store_w), so
    // part 0 has nothing to do
    if (MODE == MODE_FAST && b.nq > 0 && part < 2) return part == 0 ? 0 : launch_spmm_tc(b, st);
    switch (part) {
        case 0: if (b.nw > 0) k_selfheat_w<MODE><<<b.nw, dim3(32, 8), 0, st>>>(b); break;
        case 1: if (b.nw > 0) k_selfheat_q<MODE><<<b.nw, dim3(32, 32), 0, st>>>(b); break;
        case 2:
            if (MODE == MODE_FAST) k_tail_mode<<<1, 32, 0, st>>>(b);
            if (MODE == MODE_FAST && b.cond_variant == 4) {
                switch (b.nx) {
#define NX_CASE(n)                                                \
    case n:                                                       \
        k_conduction<MODE, n, 3><<<b.nfb, 128, 0, st>>>(b);       \
        k_conduction_pairs<n><<<b.nfb, 64, 0, st>>>(b);           \
        break;
                    NX_LIST(NX_CASE)
#undef NX_CASE
                    default: return 1;
                }
            } else if (MODE == MODE_FAST && b.cond_variant == 3) {
                switch (b.nx) {
#define NX_CASE(n) case n: k_conduction<MODE, n, 3><<<b.nfb, 128, 0, st>>>(b); break;
                    NX_LIST(NX_CASE)
#undef NX_CASE
                    default: return 1;
                }
            } else if (MODE == MODE_FAST && b.cond_variant == 2) {
                switch (b.nx) {
#define NX_CASE(n) case n: k_conduction<MODE, n, 2><<<b.nfb, 128, 0, st>>>(b); break;
                    NX_LIST(NX_CASE)
#undef NX_CASE
                    default: return 1;
                }
            } else {
                switch (b.nx) {
#define NX_CASE(n) case n: k_conduction<MODE, n><<<b.nfb, 128, 0, st>>>(b); break;
                    NX_LIST(NX_CASE)
#undef NX_CASE
                    default: return 1;
                }
            }
            if (MODE == MODE_FAST) {
                const int wgrid = b.n * kSparseCtas;
                switch (b.nx) {
#define NX_CASE(n) case n: k_conduction_warp<n><<<wgrid, 128, 0, st>>>(b); break;
                    NX_LIST(NX_CASE)
#undef NX_CASE
                    default: return 1;
                }
            }
            break;
        case 3: k_converge<<<b.nfb, 128, 0, st>>>(b); break;
        case 4: k_advance<<<(b.n + 127) / 128, 128, 0, st>>>(b); break;
        default: return 1;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_revolution_part(const Batch& b, int part, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    switch (b.mode) {
        case MODE_REF: return launch_rev_part<MODE_REF>(b, part, st);
        case MODE_FP64: return launch_rev_part<MODE_FP64>(b, part, st);
        case MODE_FAST: return launch_rev_part<MODE_FAST>(b, part, st);
    }
    return 1;
}

int kernels_per_revolution(const Batch& b) {
    const bool tc = b.mode == MODE_FAST && b.nq > 0;
    // k_tc_compact + k_spmm_tc (+ k_spmm_rem, k_rem_add), or W + Q
    const int selfheat = tc ? 2 + (b.rem_nmb > 0 ? 2 : 0) : (b.nw > 0 ? 2 : 0);
    // + k_tail_mode, k_conduction_warp (+ k_conduction_pairs)
    const int conduction = b.mode == MODE_FAST ? (b.cond_variant == 4 ? 4 : 3) : 1;
    return selfheat + conduction + 2;                    // + k_converge, k_advance
}

int launch_revolution(const Batch& b, stream_t st) {
    for (int part = 0; part < 5; ++part) {
        const int rc = launch_revolution_part(b, part, st);
        if (rc) return rc;
    }
    return 0;
}

int launch_initial_mean(const DevSolve& s, void* out, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const int g = (s.nf + 127) / 128;
    switch (s.mode) {
        case MODE_REF: k_initial_mean<MODE_REF><<<g, 128, 0, st>>>(s, out); break;
        case MODE_FP64: k_initial_mean<MODE_FP64><<<g, 128, 0, st>>>(s, out); break;
        default: k_initial_mean<MODE_FAST><<<g, 128, 0, st>>>(s, out); break;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_fill_initial(const DevSolve& s, const void* mean, const PowTab& pq, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const int g = (s.nf + 127) / 128;
    switch (s.mode) {
        case MODE_REF: k_fill_initial<MODE_REF><<<g, 128, 0, st>>>(s, mean, pq); break;
        case MODE_FP64: k_fill_initial<MODE_FP64><<<g, 128, 0, st>>>(s, mean, pq); break;
        default: k_fill_initial<MODE_FAST><<<g, 128, 0, st>>>(s, mean, pq); break;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// Progress of every solve of a batch for one read-back: its control word,
// status word and the convergence counts of its last `window` revolutions
// (record of 5 + window ints per solve)
__global__ void k_progress(Batch b, int window, int* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.n) return;
    const DevSolve& s = b.tab[i];
    int* o = out + (size_t)i * (5 + window);
    const Ctl c = *s.ctl;
    o[0] = c.rev;
    o[1] = c.active;
    o[2] = c.converged;
    o[3] = c.numconv;
    o[4] = *s.status;
    for (int j = 0; j < window; ++j) {
        const int r = c.rev - window + j;
        o[5 + j] = (r >= 0 && r < s.revcap) ? s.counts[r] : 0;
    }
}

int launch_progress(const Batch& b, int window, int* out, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    k_progress<<<(b.n + 127) / 128, 128, 0, st>>>(b, window, out);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_energy_balance(const DevSolve& s, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const int g = (s.nf + 127) / 128;
    if (s.mode == MODE_FP64) k_energy<MODE_FP64><<<g, 128, 0, st>>>(s);
    else k_energy<MODE_REF><<<g, 128, 0, st>>>(s);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // namespace atpm
