// Crater (surface roughness) module: the kernels of the reference's Thermal
// GPU module (3905/Thermal/NominalPole/GPU_code.cu:152-594), rebuilt for
// GB300 with runtime sizes.
//
// Every facet carries a hemispherical crater of nsf (= 100) sub-facets.  The
// reference launches one kernel per time step (2 x NTAU launches and
// synchronisations per revolution, GPU_code.cu:982-998).  Here:
//
//   k_crater_shadow      sfcpartialshadow (152-210): 10x10 sub-points of each
//                        sub-facet against the analytic crater rim, every
//                        (facet, step) in one launch
//   k_crater_scatter     roughness_single/multiple_scattering (216-304):
//                        one block per (facet, step) batch, the 100x100
//                        crater view-factor matrix staged in shared memory
//   k_crater_revolution  finite_difference + boundary_condition (377-490)
//                        for a whole revolution in ONE launch: a block owns a
//                        facet, a thread owns a sub-facet's depth column in
//                        registers; the crater self-heating sum reads the
//                        other sub-facets' previous-revolution temperatures
//                        through shared memory
//   k_crater_equilibrium roughness_inst_equilibrium (496-548)
//   k_crater_converged   converged (554-594)
//
// REFERENCE precision evaluates every float expression in the GPU module's
// operand order without contraction, with this host's libm powf for x^4 and
// x^0.25 (the exception tables of atpm_powtab.cpp); it is bit-identical to
// the CPU restatement of the module the reference driver links for GPU-free
// runs.  FAST precision contracts and reorders.
#include <cuda_runtime.h>

#include "atpm_internal.h"

namespace atpm {

namespace {

template <int MODE> struct Ca;
template <> struct Ca<MODE_REF> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }
};
template <> struct Ca<MODE_FAST> {
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
    static __device__ __forceinline__ float div(float a, float b) { return a / b; }
    static __device__ __forceinline__ float sqrt_(float a) { return sqrtf(a); }
};

__device__ __forceinline__ float cpow4_exact(const PowTab& t, float x, int* st) {
    // x^4 corrected to this host's libm powf (atpm_powtab.cpp)
    return pow_table_fix(t, x, dev_pow4(x), st);
}

template <int MODE>
__device__ __forceinline__ float cpow4(const PowTab& t, float x, int* st) {
    if constexpr (MODE == MODE_REF) return cpow4_exact(t, x, st);
    else { const float x2 = x * x; return x2 * x2; }
}

}  // namespace

// sfcpartialshadow: each thread owns one (facet, step, sub-facet)
template <int MODE>
__global__ void __launch_bounds__(128) k_crater_shadow(CraterDev c) {
    using A = Ca<MODE>;
    const int nsf = c.nsf;
    const long long n = (long long)c.nf * c.ntau;
    const int j = threadIdx.x;
    for (long long fs = blockIdx.x; fs < n; fs += gridDim.x) {
        if (c.shadow[fs] != 1) continue;  // block-uniform
        if (j >= nsf) continue;
        const float* iv = c.illumvec + 3 * fs;
        // sun vector normalised by its x-y length (GPU_code.cu:177-181)
        const float s = A::sqrt_(A::add(A::mul(iv[0], iv[0]), A::mul(iv[1], iv[1])));
        const float sv0 = A::div(iv[0], s), sv1 = A::div(iv[1], s), sv2 = A::div(iv[2], s);
        const float a = A::div(fabsf(sv2), A::sqrt_(A::add(A::mul(sv0, sv0), A::mul(sv1, sv1))));
        float sh = c.sfc_shadow[fs * nsf + j];
        const float* v2 = c.cverts + 3 * c.cfac[3 * j + 2];
        const float* t0 = c.ctri + 6 * j;
        const float* t1 = t0 + 3;
        const float R = 10.0f;
        for (int p = 0; p != 100; ++p) {
            const float m0 = c.cmult[2 * p], m1 = c.cmult[2 * p + 1];
            float mp[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) mp[k] = A::add(A::add(v2[k], A::mul(m0, t0[k])), A::mul(m1, t1[k]));
            const float tc1 = A::add(A::mul(A::mul(-1.0f, sv1), mp[0]), A::mul(sv0, mp[1]));
            const float rad = A::sqrt_(A::sub(A::mul(R, R), A::mul(tc1, tc1)));
            const float tc0 = A::sub(A::add(A::mul(sv0, mp[0]), A::mul(sv1, mp[1])), rad);
            if (mp[2] <= A::mul(a, tc0) && sh != 0.0f) sh = A::sub(sh, A::div(1.0f, 100.0f));
            if (sh < 0.0f) sh = 0.0f;
        }
        c.sfc_shadow[fs * nsf + j] = sh;
    }
}

// single (multiple == 0) or single + Jacobi multiple scattering of one
// (facet, step) per block iteration
template <int MODE>
__global__ void __launch_bounds__(128) k_crater_scatter(CraterDev c, float solar, float acc, int multiple, int cap) {
    using A = Ca<MODE>;
    extern __shared__ float sm[];
    const int nsf = c.nsf;
    float* Vs = sm;                 // nsf*nsf
    float* ill = Vs + nsf * nsf;    // nsf
    float* pold = ill + nsf;        // nsf
    __shared__ int more;
    for (int k = threadIdx.x; k < nsf * nsf; k += blockDim.x) Vs[k] = c.V[k];
    __syncthreads();
    const long long n = (long long)c.nf * c.ntau;
    const int j = threadIdx.x;
    for (long long fs = blockIdx.x; fs < n; fs += gridDim.x) {
        const int f = (int)(fs / c.ntau);
        const float alb = c.albedo[f];
        const size_t o = (size_t)fs * nsf + j;
        float solarpower = 0.0f, tot = 0.0f;
        if (j < nsf) {
            const float sh = c.sfc_shadow[o], ia = c.illumangle[o], gi = c.RGI[o];
            ill[j] = A::add(A::mul(A::mul(solar, sh), ia), gi);
            solarpower = A::add(A::mul(A::mul(solar, ia), sh), gi);
        }
        __syncthreads();
        if (j < nsf) {
            tot = ill[j];
            for (int i = 0; i != nsf; ++i) tot = A::add(tot, A::mul(A::mul(Vs[i * nsf + j], alb), ill[i]));
            if (tot <= 0.0f) tot = 0.0f;
        }
        if (multiple) {
            float pnew = 0.0f;
            if (j < nsf) pold[j] = A::mul(alb, tot);
            __syncthreads();
            for (int it = 0; it < cap; ++it) {
                if (threadIdx.x == 0) more = 0;
                float sum = 0.0f;
                if (j < nsf) {
                    for (int i = 0; i != nsf; ++i) sum = A::add(sum, A::mul(Vs[i * nsf + j], pold[i]));
                    pnew = A::mul(alb, A::add(solarpower, sum));
                }
                __syncthreads();
                if (j < nsf) {
                    const float d = A::sub(pnew, pold[j]);
                    if (fabsf(d) > acc) more = 1;
                    pold[j] = pnew;
                }
                __syncthreads();
                const int m = more;
                __syncthreads();
                if (!m) break;
                if (it + 1 == cap && threadIdx.x == 0) atomicOr(c.status, ST_SCATTER_CAP);
            }
            tot = A::div(pnew, alb);
        }
        if (j < nsf) c.RI[o] = tot;
        __syncthreads();
    }
}

// one revolution of finite_difference + boundary_condition for every step:
// block = one facet, thread j = sub-facet j (its depth column in registers)
template <int MODE, int NX>
__global__ void __launch_bounds__(128) k_crater_revolution(CraterDev c, PowTab p4, float es, float es4, float m0,
                                                           float dz, float tacc, float tacc2) {
    using A = Ca<MODE>;
    extern __shared__ float sm[];
    const int nsf = c.nsf, ntau = c.ntau, f = blockIdx.x;
    if (c.conv[f]) return;  // block-uniform (sfc_converged)
    float* Vs = sm;                           // nsf*nsf
    float* W = Vs + ((nsf * nsf + 3) & ~3);   // nsf, 16-byte aligned: eps sigma T_prev^4 of this step
    for (int k = threadIdx.x; k < nsf * nsf; k += blockDim.x) Vs[k] = c.V[k];
    const int j = threadIdx.x;
    const bool act = j < nsf;
    const float alb = c.albedo[f];
    // the facet body's revolutions per model period scale the time step and
    // the skin factor (175706/Run-04/thermal_GPU.cu:448-450, 539); with none
    // given the expressions are the synchronous module's (GPU_code.cu:392-393)
    const float w2pi = c.numrevs ? A::mul(A::mul(2.0f, c.PI), c.numrevs[f]) : A::mul(2.0f, c.PI);
    const float m0f = c.numrevs ? A::div(A::div(w2pi, (float)ntau), A::mul(dz, dz)) : m0;
    const float m1 = A::div(A::mul(c.ti[f], A::sqrt_(A::div(w2pi, c.rot_period))), dz);
    const float esw = A::mul(c.ir_abs, es);  // IR_ABS * EPSSIGMA (thermal_GPU.cu:521): es when ir_abs = 1
    const float oma = A::sub(1.0f, alb);
    float T[NX + 1];
    float* tp = c.temp + (size_t)f * (NX + 1) * nsf;
#pragma unroll
    for (int i = 0; i <= NX; ++i) T[i] = act ? tp[(size_t)i * nsf + j] : 0.0f;
    bool hot = false;
    int flags = 0;
    const size_t base = (size_t)f * ntau * nsf;
    // the step's forcing and previous-revolution temperature are loaded one
    // step ahead (they are not written by the current step), so the HBM
    // latency overlaps the current step's sweep
    float nx_old = 0.0f, nx_rgh = 0.0f, nx_ri = 0.0f;
    if (act) {
        nx_old = c.stemp1[base + j];
        nx_rgh = c.RGH[base + j];
        nx_ri = c.RI[base + j];
    }
    for (int s = 0; s < ntau; ++s) {
        const size_t o = base + (size_t)s * nsf + j;
        const float old = nx_old, rgh = nx_rgh, ri = nx_ri;
        if (act && s + 1 < ntau) {
            nx_old = c.stemp1[o + nsf];
            nx_rgh = c.RGH[o + nsf];
            nx_ri = c.RI[o + nsf];
        }
        // finite_difference (GPU_code.cu:377-412)
        if (act) {
            float t0 = T[0];
#pragma unroll
            for (int i = 1; i < NX; ++i) {
                const float t1 = T[i];
                T[i] = A::add(t1, A::mul(m0f, A::add(A::sub(T[i + 1], A::mul(2.0f, t1)), t0)));
                t0 = t1;
            }
            T[NX] = T[NX - 1];
        }
        // boundary_condition (GPU_code.cu:418-490)
        if (act) {
            c.stemp0[o] = old;
            W[j] = A::mul(esw, cpow4<MODE>(p4, old, c.status));
        }
        __syncthreads();
        if (act) {
            // W is read four at a time (one broadcast 16-byte load); the
            // sum keeps the module's order in REFERENCE precision
            const float4* W4 = reinterpret_cast<const float4*>(W);
            const int n4 = nsf >> 2;
            float inc;
            if constexpr (MODE == MODE_REF) {
                inc = rgh;
                for (int q = 0; q < n4; ++q) {
                    const float4 w = W4[q];
                    const float* v = Vs + (4 * q) * nsf + j;
                    inc = A::add(inc, A::mul(w.x, v[0]));
                    inc = A::add(inc, A::mul(w.y, v[nsf]));
                    inc = A::add(inc, A::mul(w.z, v[2 * nsf]));
                    inc = A::add(inc, A::mul(w.w, v[3 * nsf]));
                }
                for (int i = 4 * n4; i < nsf; ++i) inc = A::add(inc, A::mul(W[i], Vs[i * nsf + j]));
            } else {
                // four interleaved partial sums: a quarter of the dependent chain
                float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
                for (int q = 0; q < n4; ++q) {
                    const float4 w = W4[q];
                    const float* v = Vs + (4 * q) * nsf + j;
                    a0 += w.x * v[0];
                    a1 += w.y * v[nsf];
                    a2 += w.z * v[2 * nsf];
                    a3 += w.w * v[3 * nsf];
                }
                for (int i = 4 * n4; i < nsf; ++i) a0 += W[i] * Vs[i * nsf + j];
                inc = rgh + ((a0 + a1) + (a2 + a3));
            }
            const float m2 = A::add(A::mul(oma, ri), inc);
            float TR0 = T[0], TR1 = T[0], DT = 1.0f;
            int it = 0;
            while (DT >= tacc2) {
                if (it == 200) { flags |= ST_NEWTON_CAP; break; }
                const float t3 = A::mul(A::mul(A::mul(es, TR0), TR0), TR0);
                const float sbc = A::sub(A::add(m2, A::mul(m1, A::sub(T[1], TR0))), A::mul(t3, TR0));
                const float sbcd = A::add(m1, A::mul(A::mul(A::mul(es4, TR0), TR0), TR0));
                TR1 = A::add(TR0, A::div(sbc, sbcd));
                DT = fabsf(A::sub(TR1, TR0));
                TR0 = TR1;
                ++it;
            }
            T[0] = TR1;
            c.stemp1[o] = TR1;
            hot = hot || (fabsf(A::sub(old, TR1)) >= tacc);
            if (!isfinite(TR1)) flags |= ST_NONFINITE;
        }
        __syncthreads();
    }
    if (act) {
#pragma unroll
        for (int i = 0; i <= NX; ++i) tp[(size_t)i * nsf + j] = T[i];
    }
    if (__syncthreads_or(hot) && threadIdx.x == 0) c.hot[f] = 1;
    else if (threadIdx.x == 0) c.hot[f] = 0;
    if (flags) atomicOr(c.status, flags);
}

// roughness_inst_equilibrium (GPU_code.cu:496-548)
template <int MODE>
__global__ void __launch_bounds__(128) k_crater_equilibrium(CraterDev c, PowTab p4, PowTab pq, float es) {
    using A = Ca<MODE>;
    extern __shared__ float sm[];
    const int nsf = c.nsf, ntau = c.ntau, f = blockIdx.x;
    if (c.conv[f]) return;
    float* Vs = sm;
    float* W = Vs + nsf * nsf;
    for (int k = threadIdx.x; k < nsf * nsf; k += blockDim.x) Vs[k] = c.V[k];
    const int j = threadIdx.x;
    const bool act = j < nsf;
    const float oma = A::sub(1.0f, c.albedo[f]);
    const float esw = A::mul(c.ir_abs, es);
    for (int s = 0; s < ntau; ++s) {
        const size_t o = (size_t)f * ntau * nsf + (size_t)s * nsf + j;
        if (act) {
            const float old = c.stemp1[o];
            c.stemp0[o] = old;
            W[j] = A::mul(esw, cpow4<MODE>(p4, old, c.status));
        }
        __syncthreads();
        if (act) {
            float inc = c.RGH[o];
            for (int i = 0; i != nsf; ++i) inc = A::add(inc, A::mul(W[i], Vs[i * nsf + j]));
            const float x = A::div(A::add(A::mul(oma, c.RI[o]), inc), es);
            c.stemp1[o] = (MODE == MODE_REF) ? pow_table_fix(pq, x, dev_qroot(x), c.status) : dev_qroot(x);
        }
        __syncthreads();
    }
}

// converged (GPU_code.cu:554-594)
__global__ void __launch_bounds__(128) k_crater_converged(CraterDev c, float tacc) {
    const int f = blockIdx.x;
    if (c.conv[f]) return;
    const size_t n = (size_t)c.ntau * c.nsf, base = (size_t)f * n;
    int bad = 0;
    for (size_t k = threadIdx.x; k < n; k += blockDim.x)
        if (fabsf(c.stemp0[base + k] - c.stemp1[base + k]) >= tacc) bad = 1;
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) c.conv[f] = bad ? 0 : 1;
}

// first initialisation pass: per sub-facet mean of (1-A) RI + RGH (GPU_code.cu:341-345)
__global__ void k_crater_init_mean(CraterDev c, float* out, int with_self, const float* selfh) {
    const int f = blockIdx.x, j = threadIdx.x;
    if (j >= c.nsf) return;
    const float alb = c.albedo[f];
    const float inv = __fdiv_rn(1.0f, (float)c.ntau);
    const float sh = with_self ? selfh[(size_t)f * c.nsf + j] : 0.0f;
    float t = 0.0f;
    for (int s = 0; s != c.ntau; ++s) {
        const size_t o = (size_t)f * c.ntau * c.nsf + (size_t)s * c.nsf + j;
        float x = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, alb), c.RI[o]), c.RGH[o]);
        if (with_self) x = __fadd_rn(x, sh);
        t = __fadd_rn(t, __fmul_rn(inv, x));
    }
    out[(size_t)f * c.nsf + j] = t;
}

// crater self-heating of the first initialisation temperatures (GPU_code.cu:351-354)
__global__ void k_crater_init_self(CraterDev c, PowTab p4, float es, const float* t0, float* out) {
    extern __shared__ float sm[];
    const int f = blockIdx.x, j = threadIdx.x, nsf = c.nsf;
    float* w = sm;
    if (j < nsf) w[j] = __fmul_rn(__fmul_rn(c.ir_abs, es), cpow4_exact(p4, t0[(size_t)f * nsf + j], c.status));
    __syncthreads();
    if (j >= nsf) return;
    float sh = 0.0f;
    for (int i = 0; i != nsf; ++i) sh = __fadd_rn(sh, __fmul_rn(w[i], c.V[i * nsf + j]));
    out[(size_t)f * nsf + j] = sh;
}

// t = (t / (eps sigma))^0.25 of the initialisation (GPU_code.cu:346, 362)
template <int MODE>
__global__ void k_crater_root(CraterDev c, PowTab pq, float es, float* t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.nf * c.nsf) return;
    const float x = __fdiv_rn(t[i], es);
    t[i] = (MODE == MODE_REF) ? pow_table_fix(pq, x, dev_qroot(x), c.status) : dev_qroot(x);
}

__global__ void k_crater_fill(CraterDev c, const float* t) {
    const int f = blockIdx.x, j = threadIdx.x;
    if (j >= c.nsf) return;
    const float v = t[(size_t)f * c.nsf + j];
    for (int i = 0; i <= c.nx; ++i) c.temp[((size_t)f * (c.nx + 1) + i) * c.nsf + j] = v;
    for (int s = 0; s < c.ntau; ++s) {
        const size_t o = (size_t)f * c.ntau * c.nsf + (size_t)s * c.nsf + j;
        c.stemp0[o] = v;
        c.stemp1[o] = v;
    }
}

// ------------------------------------------------------------------ launchers
#define CRATER_NX_LIST(X) X(8) X(12) X(16) X(24) X(32) X(40) X(48) X(56) X(64)

int crater_launch(int what, const CraterDev& c, const PowTab& p4, const PowTab& pq, const float* fargs, void* p0,
                  void* p1, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const size_t smv = (size_t)c.nsf * c.nsf * 4;
    const int grid_fs = 152 * 8;
    switch (what) {
        case 0:  // partial shadow
            if (c.mode == MODE_FAST) k_crater_shadow<MODE_FAST><<<grid_fs, 128, 0, st>>>(c);
            else k_crater_shadow<MODE_REF><<<grid_fs, 128, 0, st>>>(c);
            break;
        case 1: {  // scattering: fargs = {solar, acc, multiple}
            const size_t sm = smv + 2 * c.nsf * 4;
            cudaFuncSetAttribute(k_crater_scatter<MODE_REF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            cudaFuncSetAttribute(k_crater_scatter<MODE_FAST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            if (c.mode == MODE_FAST)
                k_crater_scatter<MODE_FAST><<<grid_fs, 128, sm, st>>>(c, fargs[0], fargs[1], (int)fargs[2], 10000);
            else
                k_crater_scatter<MODE_REF><<<grid_fs, 128, sm, st>>>(c, fargs[0], fargs[1], (int)fargs[2], 10000);
            break;
        }
        case 2: {  // revolution: fargs = {es, es4, m0, dz, tacc, tacc2}
            const size_t sm = (size_t)(((c.nsf * c.nsf + 3) & ~3) + c.nsf) * 4;
#define NX_CASE(n)                                                                                         \
    case n:                                                                                                \
        if (c.mode == MODE_FAST) {                                                                         \
            cudaFuncSetAttribute(k_crater_revolution<MODE_FAST, n>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm); \
            k_crater_revolution<MODE_FAST, n><<<c.nf, 128, sm, st>>>(c, p4, fargs[0], fargs[1], fargs[2], fargs[3], fargs[4], fargs[5]); \
        } else {                                                                                           \
            cudaFuncSetAttribute(k_crater_revolution<MODE_REF, n>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm); \
            k_crater_revolution<MODE_REF, n><<<c.nf, 128, sm, st>>>(c, p4, fargs[0], fargs[1], fargs[2], fargs[3], fargs[4], fargs[5]); \
        }                                                                                                  \
        break;
            switch (c.nx) {
                CRATER_NX_LIST(NX_CASE)
                default: return 1;
            }
#undef NX_CASE
            break;
        }
        case 3: {  // equilibrium: fargs = {es}
            const size_t sm = smv + c.nsf * 4;
            cudaFuncSetAttribute(k_crater_equilibrium<MODE_REF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            cudaFuncSetAttribute(k_crater_equilibrium<MODE_FAST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            if (c.mode == MODE_FAST) k_crater_equilibrium<MODE_FAST><<<c.nf, 128, sm, st>>>(c, p4, pq, fargs[0]);
            else k_crater_equilibrium<MODE_REF><<<c.nf, 128, sm, st>>>(c, p4, pq, fargs[0]);
            break;
        }
        case 4:  // converged: fargs = {tacc}
            k_crater_converged<<<c.nf, 128, 0, st>>>(c, fargs[0]);
            break;
        case 5:  // init mean (pass 1 when p1 == null, pass 2 with self-heating p1)
            k_crater_init_mean<<<c.nf, 128, 0, st>>>(c, static_cast<float*>(p0), p1 ? 1 : 0,
                                                     static_cast<const float*>(p1));
            break;
        case 6:  // init self-heating: fargs = {es}; p0 = t0, p1 = out
            k_crater_init_self<<<c.nf, 128, c.nsf * 4, st>>>(c, p4, fargs[0], static_cast<const float*>(p0),
                                                             static_cast<float*>(p1));
            break;
        case 7:  // fill
            k_crater_fill<<<c.nf, 128, 0, st>>>(c, static_cast<const float*>(p0));
            break;
        case 8: {  // fourth root in place: fargs = {es}; p0 = t
            const int g = (c.nf * c.nsf + 127) / 128;
            if (c.mode == MODE_FAST) k_crater_root<MODE_FAST><<<g, 128, 0, st>>>(c, pq, fargs[0], static_cast<float*>(p0));
            else k_crater_root<MODE_REF><<<g, 128, 0, st>>>(c, pq, fargs[0], static_cast<float*>(p0));
            break;
        }
        default:
            return 1;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

bool crater_nx_supported(int nx) {
#define NX_CASE(n) if (nx == n) return true;
    CRATER_NX_LIST(NX_CASE)
#undef NX_CASE
    return false;
}

}  // namespace atpm
