// Disk-integrated thermal flux seen by an observer, in FP64 on the device:
// the smooth-surface sum of the reference's Observe stage
// (observe, 3905/Observe/NominalPole/wise_main.cpp:662-730, geometry
// 555-645).  For every step s and wavelength l:
//
//   F[s][l] = sum over facets f visible at s of
//             B_l(T_f[s]) * eps * A_f * cos(e_f[s]) / d_f[s]^2
//
// with B the Planck radiance (the stage's constants), e the angle between
// the facet normal and the direction to the observer, d the facet's distance
// to the observer, A_f the facet area as the stage leaves it (computed at the
// last step of its geometry loop).
//
//   k_flux_partial  one thread per (facet, step): rotate the facet's three
//                   vertices (host-libm rotation table, pole matrix), build
//                   its frame, weight and Planck terms; a fixed-order
//                   shared-memory tree sums each 256-facet block
//   k_flux_sum      sums the block partials of every (step, wavelength) in
//                   block order: the result does not depend on scheduling
//
// The rough-surface sum (observe, wise_main.cpp:695-727) replaces each
// facet's own term by its crater's: the sub-facets with a visible fraction
// toward the observer > 0 add B(T_sub) eps a_sub vis cos(e_sub) / d^2, and
// the facet's total enters scaled by A_f over the crater's projected area.
#include <cuda_runtime.h>

#include "atpm_internal.h"

namespace atpm {

namespace {

constexpr int kFluxThreads = 256;

template <class R>
__device__ __forceinline__ double temp_at(const DevSolve& s, int f, int step) {
    return (double)static_cast<const R*>(s.stemp1)[(size_t)step * s.nf + f];
}

__device__ __forceinline__ void vertex_at(const DevSolve& s, const FluxArgs& a, int v, int step, double* out) {
    const double* e = s.vert + 3 * v;
    const double* rt = (v < a.vsplit) ? a.rot : a.rot2;
    const double c = rt[2 * step], sn = rt[2 * step + 1];
    double rq[3];
    rq[0] = __dsub_rn(__dmul_rn(e[0], c), __dmul_rn(e[1], sn));
    rq[1] = __dadd_rn(__dmul_rn(e[0], sn), __dmul_rn(e[1], c));
    rq[2] = e[2];
#pragma unroll
    for (int k = 0; k < 3; ++k)
        out[k] = __dadd_rn(a.car[k], __dadd_rn(__dadd_rn(__dmul_rn(a.tm[3 * k], rq[0]), __dmul_rn(a.tm[3 * k + 1], rq[1])),
                                               __dmul_rn(a.tm[3 * k + 2], rq[2])));
}

__device__ __forceinline__ void edges_at(const DevSolve& s, const FluxArgs& a, int f, int step, double* hm, double* nc0,
                                         double* nc1) {
    const int* fv = s.fac + 3 * f;
    double h0[3], h1[3], h2[3];
    vertex_at(s, a, fv[0], step, h0);
    vertex_at(s, a, fv[1], step, h1);
    vertex_at(s, a, fv[2], step, h2);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        hm[k] = __ddiv_rn(__dadd_rn(__dadd_rn(h0[k], h1[k]), h2[k]), 3.0);
        nc0[k] = __dsub_rn(h1[k], h0[k]);
        nc1[k] = __dsub_rn(h2[k], h0[k]);
    }
}

__device__ __forceinline__ void cross(const double* a, const double* b, double* n) {
    n[0] = __dsub_rn(__dmul_rn(a[1], b[2]), __dmul_rn(a[2], b[1]));
    n[1] = __dsub_rn(__dmul_rn(a[2], b[0]), __dmul_rn(a[0], b[2]));
    n[2] = __dsub_rn(__dmul_rn(a[0], b[1]), __dmul_rn(a[1], b[0]));
}

__device__ __forceinline__ double norm3(const double* v) {
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])), __dmul_rn(v[2], v[2])));
}

template <class R, bool ROUGH>
__global__ void __launch_bounds__(kFluxThreads) k_flux_partial(DevSolve s, FluxArgs a) {
    __shared__ double red[kFluxThreads];
    const int step = blockIdx.y;
    const int f = blockIdx.x * kFluxThreads + threadIdx.x;
    double term[kMaxFluxWavelengths];
#pragma unroll
    for (int l = 0; l < kMaxFluxWavelengths; ++l) term[l] = 0.0;
    if (f < s.nf && (!a.visible || a.visible[(size_t)f * s.ntau + step])) {
        double hm[3], nc0[3], nc1[3], n[3];
        // area as the stage leaves it: from the last step of its geometry loop
        edges_at(s, a, f, s.ntau - 1, hm, nc0, nc1);
        cross(nc0, nc1, n);
        const double area = __ddiv_rn(norm3(n), 2.0);
        edges_at(s, a, f, step, hm, nc0, nc1);
        cross(nc0, nc1, n);
        const double nn = norm3(n);
#pragma unroll
        for (int k = 0; k < 3; ++k) n[k] = __ddiv_rn(n[k], nn);
        const double x = norm3(nc0);
        double xh[3], y[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) xh[k] = __ddiv_rn(nc0[k], x);
        cross(n, xh, y);
        double ov[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) ov[k] = __dsub_rn(hm[k], a.obs[k]);
        const double o = norm3(ov);
        // view vector in the facet frame (rows x^, y, n)
        const double v0 = -__dadd_rn(__dadd_rn(__dmul_rn(xh[0], ov[0]), __dmul_rn(xh[1], ov[1])), __dmul_rn(xh[2], ov[2]));
        const double v1 = -__dadd_rn(__dadd_rn(__dmul_rn(y[0], ov[0]), __dmul_rn(y[1], ov[1])), __dmul_rn(y[2], ov[2]));
        const double v2 = -__dadd_rn(__dadd_rn(__dmul_rn(n[0], ov[0]), __dmul_rn(n[1], ov[1])), __dmul_rn(n[2], ov[2]));
        const double va = acos(__ddiv_rn(v2, o));
        if (!(va > (3.141592653589793 / 2.0))) {
            const double d = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(v0, v0), __dmul_rn(v1, v1)), __dmul_rn(v2, v2)));
            if constexpr (!ROUGH) {
                double mult = __ddiv_rn(__dmul_rn(__dmul_rn(a.eps, area), cos(va)), __dmul_rn(d, d));
                if (mult != mult) mult = 0.0;
                const double T = temp_at<R>(s, f, step);
                for (int l = 0; l < a.nwl; ++l) {
                    // (2hc^2 / lambda^5) * (1 / (exp(hc / (lambda k T)) - 1))
                    const double arg = __ddiv_rn(a.hc, __dmul_rn(a.lk[l], T));
                    double b = __dmul_rn(a.b1[l], __ddiv_rn(1.0, __dsub_rn(exp(arg), 1.0)));
                    if (b != b) b = 0.0;
                    term[l] = __dmul_rn(b, mult);
                }
            } else {
                // the facet's crater: every sub-facet with a visible fraction
                // > 0, its view angle from the view vector in the facet frame
                // (wise_main.cpp:515), in sub-facet order; then the facet's
                // share of the crater's projected area (wise_main.cpp:718)
                const size_t base = ((size_t)f * s.ntau + step) * (size_t)a.nsf;
                double sfc[kMaxFluxWavelengths];
#pragma unroll
                for (int l = 0; l < kMaxFluxWavelengths; ++l) sfc[l] = 0.0;
                const double dd = __dmul_rn(d, d);
                for (int j = 0; j < a.nsf; ++j) {
                    const double vis = (double)a.sub_vis[base + j];
                    if (!(vis > 0.0)) continue;
                    const double* g = a.sub_geo + 4 * j;
                    const double c = __dadd_rn(__dadd_rn(__dmul_rn(v0, g[0]), __dmul_rn(v1, g[1])), __dmul_rn(v2, g[2]));
                    const double vj = acos(__ddiv_rn(c, d));
                    double mult = __ddiv_rn(__dmul_rn(__dmul_rn(__dmul_rn(a.eps, g[3]), vis), cos(vj)), dd);
                    if (mult != mult) mult = 0.0;
                    const double T = (double)a.sub_T[base + j];
                    for (int l = 0; l < a.nwl; ++l) {
                        const double arg = __ddiv_rn(a.hc, __dmul_rn(a.lk[l], T));
                        double b = __dmul_rn(a.b1[l], __ddiv_rn(1.0, __dsub_rn(exp(arg), 1.0)));
                        if (b != b) b = 0.0;
                        sfc[l] = __dadd_rn(sfc[l], __dmul_rn(b, mult));
                    }
                }
                for (int l = 0; l < a.nwl; ++l) term[l] = __ddiv_rn(__dmul_rn(sfc[l], area), a.sub_total);
            }
        }
    }
    for (int l = 0; l < a.nwl; ++l) {
        red[threadIdx.x] = term[l];
        __syncthreads();
        for (int w = kFluxThreads / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) red[threadIdx.x] = __dadd_rn(red[threadIdx.x], red[threadIdx.x + w]);
            __syncthreads();
        }
        if (threadIdx.x == 0) a.partial[((size_t)step * gridDim.x + blockIdx.x) * a.nwl + l] = red[0];
        __syncthreads();
    }
}

__global__ void k_flux_sum(FluxArgs a, int ntau, int nblk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntau * a.nwl) return;
    const int step = i / a.nwl, l = i % a.nwl;
    double t = 0.0;
    for (int b = 0; b < nblk; ++b) t = __dadd_rn(t, a.partial[((size_t)step * nblk + b) * a.nwl + l]);
    a.out[i] = t;
}

}  // namespace

size_t flux_partial_bytes(const DevSolve& s, int nwl) {
    const size_t nblk = (size_t)(s.nf + kFluxThreads - 1) / kFluxThreads;
    return nblk * s.ntau * nwl * sizeof(double);
}

int launch_disk_flux(const DevSolve& s, const FluxArgs& a, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    if (a.nwl < 1 || a.nwl > kMaxFluxWavelengths) return 1;
    const int nblk = (s.nf + kFluxThreads - 1) / kFluxThreads;
    const dim3 grid(nblk, s.ntau);
    if (a.sub_T) {
        if (s.mode == MODE_FP64) k_flux_partial<double, true><<<grid, kFluxThreads, 0, st>>>(s, a);
        else k_flux_partial<float, true><<<grid, kFluxThreads, 0, st>>>(s, a);
    } else {
        if (s.mode == MODE_FP64) k_flux_partial<double, false><<<grid, kFluxThreads, 0, st>>>(s, a);
        else k_flux_partial<float, false><<<grid, kFluxThreads, 0, st>>>(s, a);
    }
    k_flux_sum<<<(s.ntau * a.nwl + 127) / 128, 128, 0, st>>>(a, s.ntau, nblk);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // namespace atpm
