// The crater model's forcing, computed on the device from a solve's state
// instead of by the Thermal driver on the host:
//
//   k_crater_surface  surfacegeometry (3905/Thermal/NominalPole/main.cpp:
//                     873-885): each sub-facet's Sun angle from the facet's
//                     local Sun vector, and its starting shadow (0 where the
//                     facet is shadowed or the sub-facet faces away)
//   k_crater_gvf      calculate_surface_global_viewfactors (main.cpp:1053-
//                     1181): for every view-factor list entry of the facet
//                     and every sub-facet, the entry's view factor times the
//                     sub-facet's visible fraction of the 10x10 sub-points
//                     toward the dependent facet (the crater rim test of the
//                     partial-shadow kernel along the entry's direction) and
//                     its angle, over the direction's normal component
//   k_crater_gsum     load_GPU_roughness_globalillumination /
//                     _globalheating (main.cpp:2033-2103): per sub-facet and
//                     step, the list sum of those view factors times the
//                     dependent facet's scattered illumination x albedo, or
//                     eps sigma T^4 of its surface temperature
//
// REFERENCE precision follows the driver's float and double expressions
// operand by operand (round-to-nearest intrinsics, no contraction), so the
// arrays are bit-identical to the ones the driver builds on the host.
#include <cuda_runtime.h>

#include "atpm_internal.h"

namespace atpm {

namespace {

template <int MODE> struct Fa;
template <> struct Fa<MODE_REF> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }
};
template <> struct Fa<MODE_FAST> {
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
    static __device__ __forceinline__ float div(float a, float b) { return a / b; }
    static __device__ __forceinline__ float sqrt_(float a) { return sqrtf(a); }
};

constexpr int GS_STEPS = 32;    // steps per k_crater_gsum block
constexpr int GS_ENTRIES = 32;  // list entries staged per pass

}  // namespace

// one thread per (facet, step, sub-facet)
template <int MODE>
__global__ void __launch_bounds__(256) k_crater_surface(CraterDev c, float* illumangle) {
    using A = Fa<MODE>;
    const int nsf = c.nsf;
    const long long n = (long long)c.nf * c.ntau * nsf;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long fs = i / nsf;
        const int j = (int)(i % nsf);
        const float* v = c.illumvec + 3 * fs;
        const float* nj = c.cnorm + 3 * j;
        const float t = A::sqrt_(A::add(A::add(A::mul(v[0], v[0]), A::mul(v[1], v[1])), A::mul(v[2], v[2])));
        const float ia = A::div(A::add(A::add(A::mul(v[0], nj[0]), A::mul(v[1], nj[1])), A::mul(v[2], nj[2])), t);
        float sh = 1.0f;
        if (c.shadow[fs] == 0) sh = 0.0f;
        if (ia <= 0.0f) sh = 0.0f;
        illumangle[i] = ia;
        c.sfc_shadow[i] = sh;
    }
}

// one block per facet of the part, one thread per sub-facet; the facet's
// list entries in turn.  vert: the solve's body-frame vertices (double),
// vec: the entries' direction vectors (the _selfheating_vector_list.txt
// vectors) from entry k0 on, gvf: [entry - k0][nsf]
template <int MODE>
__global__ void __launch_bounds__(128) k_crater_gvf(CraterDev c, const double* vert, const int* fac,
                                                      const int* dep_ptr, const float* dep_vf, int f0,
                                                      const float* vec, float* gvf) {
    using A = Fa<MODE>;
    const int fl = blockIdx.x, f = f0 + fl, j = threadIdx.x, nsf = c.nsf;
    const int k0 = dep_ptr[f0], ka = dep_ptr[f], kb = dep_ptr[f + 1];
    if (ka == kb) return;
    // the facet's frame from its body-frame vertices (main.cpp:1065-1102)
    const double* v0 = vert + 3 * fac[3 * f];
    const double* v1 = vert + 3 * fac[3 * f + 1];
    const double* v2 = vert + 3 * fac[3 * f + 2];
    double nc0[3], nc1[3], nrm[3], y[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        nc0[k] = __dsub_rn(v1[k], v0[k]);
        nc1[k] = __dsub_rn(v2[k], v0[k]);
    }
    nrm[0] = __dsub_rn(__dmul_rn(nc0[1], nc1[2]), __dmul_rn(nc0[2], nc1[1]));
    nrm[1] = __dsub_rn(__dmul_rn(nc0[2], nc1[0]), __dmul_rn(nc0[0], nc1[2]));
    nrm[2] = __dsub_rn(__dmul_rn(nc0[0], nc1[1]), __dmul_rn(nc0[1], nc1[0]));
    const double n = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(nrm[0], nrm[0]), __dmul_rn(nrm[1], nrm[1])),
                                          __dmul_rn(nrm[2], nrm[2])));
    const double x = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(nc0[0], nc0[0]), __dmul_rn(nc0[1], nc0[1])),
                                          __dmul_rn(nc0[2], nc0[2])));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        nrm[k] = __ddiv_rn(nrm[k], n);
        nc0[k] = __ddiv_rn(nc0[k], x);
    }
    y[0] = __dsub_rn(__dmul_rn(nrm[1], nc0[2]), __dmul_rn(nrm[2], nc0[1]));
    y[1] = __dsub_rn(__dmul_rn(nrm[2], nc0[0]), __dmul_rn(nrm[0], nc0[2]));
    y[2] = __dsub_rn(__dmul_rn(nrm[0], nc0[1]), __dmul_rn(nrm[1], nc0[0]));
    const double* row[3] = {nc0, y, nrm};
    if (j >= nsf) return;
    const float* sn = c.cnorm + 3 * j;
    const float* cv = c.cverts + 3 * c.cfac[3 * j + 2];
    const float* t0 = c.ctri + 6 * j;
    const float* t1 = t0 + 3;
    const float R = 10.0f;
    for (int k = ka; k < kb; ++k) {
        const float* d = vec + 3 * (size_t)(k - k0);
        float w[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
            w[r] = (float)__dadd_rn(__dadd_rn(__dmul_rn(row[r][0], (double)d[0]), __dmul_rn(row[r][1], (double)d[1])),
                                    __dmul_rn(row[r][2], (double)d[2]));
        const float a = A::div(fabsf(w[2]), A::sqrt_(A::add(A::mul(w[0], w[0]), A::mul(w[1], w[1]))));
        float vis = 1.0f;
        const float angle = A::add(A::add(A::mul(w[0], sn[0]), A::mul(w[1], sn[1])), A::mul(w[2], sn[2]));
        if (angle < 0.0f) vis = 0.0f;
        for (int p = 0; p != 100; ++p) {
            const float m0 = c.cmult[2 * p], m1 = c.cmult[2 * p + 1];
            float mp[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) mp[q] = A::add(A::add(cv[q], A::mul(m0, t0[q])), A::mul(m1, t1[q]));
            const float tc1 = A::add(A::mul(A::mul(-1.0f, w[1]), mp[0]), A::mul(w[0], mp[1]));
            const float rad = A::sqrt_(A::sub(A::mul(R, R), A::mul(tc1, tc1)));
            const float tc0 = A::sub(A::add(A::mul(w[0], mp[0]), A::mul(w[1], mp[1])), rad);
            if (mp[2] <= A::mul(a, tc0) && vis != 0.0f) vis = A::sub(vis, A::div(1.0f, 100.0f));
            if (vis < 0.0f) vis = 0.0f;
        }
        float g = A::div(A::mul(A::mul(dep_vf[k], vis), angle), w[2]);
        if (g > 1.0f) g = 1.0f;
        // FAST: an entry whose direction is not above the facet's plane (a
        // grazing neighbour; its normal component can round to zero or
        // below) contributes nothing instead of an unbounded quotient
        if constexpr (MODE == MODE_FAST) {
            if (!(w[2] > 0.0f)) g = 0.0f;
        }
        gvf[(size_t)(k - k0) * nsf + j] = g;
    }
}

// out[fl][s][j] = sum over the facet's entries (list order) of gvf[k][j] x
// term(k, s): HEAT = 0: X[g][s] x alb (scattered illumination x albedo);
// HEAT = 1: eps sigma X[g][s]^4 (X: surface temperature).  X is facet-major
// [nf][ntau].  One block per (facet, 32-step chunk), one thread per
// sub-facet with the chunk's 32 sums in registers; entries staged 32 at a
// time with their X values.
template <int MODE, int HEAT>
__global__ void __launch_bounds__(128) k_crater_gsum(CraterDev c, const int* dep_ptr, const int* dep_idx, int f0,
                                                       const float* gvf, const float* X, int ntau_x, float alb,
                                                       float eps, float sigma, float* out) {
    using A = Fa<MODE>;
    __shared__ float xs[GS_ENTRIES][GS_STEPS];
    __shared__ float gs[GS_ENTRIES][128];
    const int nsf = c.nsf, ntau = c.ntau;
    const int fl = blockIdx.x, f = f0 + fl, s0 = blockIdx.y * GS_STEPS, j = threadIdx.x;
    const int k0 = dep_ptr[f0], ka = dep_ptr[f], kb = dep_ptr[f + 1];
    float acc[GS_STEPS];
#pragma unroll
    for (int q = 0; q < GS_STEPS; ++q) acc[q] = 0.0f;
    for (int kc = ka; kc < kb; kc += GS_ENTRIES) {
        const int ne = min(GS_ENTRIES, kb - kc);
        __syncthreads();
        for (int t = threadIdx.x; t < GS_ENTRIES * GS_STEPS; t += blockDim.x) {
            const int e = t / GS_STEPS, q = t % GS_STEPS;
            xs[e][q] = (e < ne && s0 + q < ntau) ? X[(size_t)dep_idx[kc + e] * ntau_x + s0 + q] : 0.0f;
        }
        for (int t = threadIdx.x; t < GS_ENTRIES * nsf; t += blockDim.x) {
            const int e = t / nsf, jj = t % nsf;
            gs[e][jj] = e < ne ? gvf[(size_t)(kc + e - k0) * nsf + jj] : 0.0f;
        }
        __syncthreads();
        if (j < nsf) {
            for (int e = 0; e < ne; ++e) {
                const float g = gs[e][j];
#pragma unroll
                for (int q = 0; q < GS_STEPS; ++q) {
                    const float x = xs[e][q];
                    float term;
                    if constexpr (HEAT == 0) {
                        term = A::mul(A::mul(g, x), alb);
                    } else {
                        term = A::mul(A::mul(A::mul(A::mul(A::mul(A::mul(g, eps), sigma), x), x), x), x);
                    }
                    acc[q] = A::add(acc[q], term);
                }
            }
        }
    }
    if (j >= nsf) return;
#pragma unroll
    for (int q = 0; q < GS_STEPS; ++q)
        if (s0 + q < ntau) out[((size_t)fl * ntau + s0 + q) * nsf + j] = acc[q];
}

// [ntau][nf] -> [nf][ntau]
__global__ void k_transpose_sf(const float* in, int ntau, int nf, float* out) {
    __shared__ float t[32][33];
    const int f = blockIdx.x * 32 + threadIdx.x, s = blockIdx.y * 32 + threadIdx.y;
    if (f < nf && s < ntau) t[threadIdx.y][threadIdx.x] = in[(size_t)s * nf + f];
    __syncthreads();
    const int fo = blockIdx.x * 32 + threadIdx.y, so = blockIdx.y * 32 + threadIdx.x;
    if (fo < nf && so < ntau) out[(size_t)fo * ntau + so] = t[threadIdx.x][threadIdx.y];
}

int launch_crater_surface(const CraterDev& c, float* illumangle, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const long long n = (long long)c.nf * c.ntau * c.nsf;
    const long long nb = (n + 255) / 256;
    const unsigned g = (unsigned)(nb < (1 << 20) ? nb : (1 << 20));
    if (c.mode == MODE_FAST) k_crater_surface<MODE_FAST><<<g, 256, 0, st>>>(c, illumangle);
    else k_crater_surface<MODE_REF><<<g, 256, 0, st>>>(c, illumangle);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_crater_gvf(const CraterDev& c, const double* vert, const int* fac, const int* dep_ptr,
                      const float* dep_vf, int f0, const float* vec, float* gvf, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    if (c.mode == MODE_FAST)
        k_crater_gvf<MODE_FAST><<<c.nf, 128, 0, st>>>(c, vert, fac, dep_ptr, dep_vf, f0, vec, gvf);
    else k_crater_gvf<MODE_REF><<<c.nf, 128, 0, st>>>(c, vert, fac, dep_ptr, dep_vf, f0, vec, gvf);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_crater_gsum(const CraterDev& c, const int* dep_ptr, const int* dep_idx, int f0, const float* gvf,
                       const float* X, int ntau_x, int heat, float alb, float eps, float sigma, float* out,
                       stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const dim3 g((unsigned)c.nf, (unsigned)((c.ntau + GS_STEPS - 1) / GS_STEPS));
    if (c.mode == MODE_FAST) {
        if (heat) k_crater_gsum<MODE_FAST, 1><<<g, 128, 0, st>>>(c, dep_ptr, dep_idx, f0, gvf, X, ntau_x, alb, eps, sigma, out);
        else k_crater_gsum<MODE_FAST, 0><<<g, 128, 0, st>>>(c, dep_ptr, dep_idx, f0, gvf, X, ntau_x, alb, eps, sigma, out);
    } else {
        if (heat) k_crater_gsum<MODE_REF, 1><<<g, 128, 0, st>>>(c, dep_ptr, dep_idx, f0, gvf, X, ntau_x, alb, eps, sigma, out);
        else k_crater_gsum<MODE_REF, 0><<<g, 128, 0, st>>>(c, dep_ptr, dep_idx, f0, gvf, X, ntau_x, alb, eps, sigma, out);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_transpose_sf(const float* in, int ntau, int nf, float* out, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const dim3 g((unsigned)((nf + 31) / 32), (unsigned)((ntau + 31) / 32)), b(32, 32);
    k_transpose_sf<<<g, b, 0, st>>>(in, ntau, nf, out);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // namespace atpm
