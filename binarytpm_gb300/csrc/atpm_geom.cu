// Geometry and shadowing in heliocentric FP64 (the reference's frame).
//
//   k_geom_vertices  rotation about the body z axis, pole transform and
//                    heliocentric offset of every vertex at every step
//                    (asteroidgeometry, 3905/Thermal/NominalPole/main.cpp:938-958)
//   k_geom_facets    midpoint, unit normal, Sun angle and self-shadow of every
//                    facet at every step (main.cpp:960-1030)
//   k_shadow_dep     astshadow over the view-factor lists (main.cpp:1286-1315)
//   k_shadow_all     all-pairs astshadow of the Visibility stage
//                    (3905/Visibility/NominalPole/main.cpp:674-704)
//   dev_shadowtest   astshadowtest (main.cpp:1187-1247)
//
// Every operation uses round-to-nearest intrinsics in the reference's operand
// order, with the rotation cos/sin and the pole matrix computed on the host by
// the same libm the reference uses, so positions, normals and shadow flags
// are bit-identical to the reference's.  The Sun angle goes through the
// device's acos/cos; the float cast of cos(acos(x)) absorbs their last-bit
// differences.
//
// Layouts are facet-major over steps ([f][s][3]) so a warp that owns 32
// consecutive steps of one facet reads each neighbour's data as one
// contiguous segment.
#include <cuda_runtime.h>

#include "atpm_internal.h"

namespace atpm {

#define DADD __dadd_rn
#define DSUB __dsub_rn
#define DMUL __dmul_rn
#define DDIV __ddiv_rn

struct GeomArgs {
    DevSolve s;
    GeomWork g;
};

__global__ void __launch_bounds__(256) k_geom_vertices(GeomArgs a) {
    const int nv = a.s.nv, ntau = a.s.ntau;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nv * ntau) return;
    const int v = (int)(i / ntau), s = (int)(i % ntau);
    const double* e = a.s.vert + 3 * v;
    const double c = a.g.rot[2 * s], sn = a.g.rot[2 * s + 1];
    double rq[3];
    rq[0] = DSUB(DMUL(e[0], c), DMUL(e[1], sn));
    rq[1] = DADD(DMUL(e[0], sn), DMUL(e[1], c));
    rq[2] = e[2];
    double* hp = a.g.hp + ((size_t)v * ntau + s) * 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double ec = DADD(DADD(DMUL(a.g.tm[3 * k + 0], rq[0]), DMUL(a.g.tm[3 * k + 1], rq[1])),
                               DMUL(a.g.tm[3 * k + 2], rq[2]));
        hp[k] = DADD(a.g.car[k], ec);
    }
}

template <int MODE>
__global__ void __launch_bounds__(256) k_geom_facets(GeomArgs a) {
    const int nf = a.s.nf, ntau = a.s.ntau;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nf * ntau) return;
    const int f = (int)(i / ntau), s = (int)(i % ntau);
    const int* fv = a.s.fac + 3 * f;
    const double* h0 = a.g.hp + ((size_t)fv[0] * ntau + s) * 3;
    const double* h1 = a.g.hp + ((size_t)fv[1] * ntau + s) * 3;
    const double* h2 = a.g.hp + ((size_t)fv[2] * ntau + s) * 3;
    double hm[3], n[3], nc0[3], nc1[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        hm[k] = DDIV(DADD(DADD(h0[k], h1[k]), h2[k]), 3.0);
        nc0[k] = DSUB(h1[k], h0[k]);
        nc1[k] = DSUB(h2[k], h0[k]);
    }
    const double t = __dsqrt_rn(DADD(DADD(DMUL(hm[0], hm[0]), DMUL(hm[1], hm[1])), DMUL(hm[2], hm[2])));
    n[0] = DSUB(DMUL(nc0[1], nc1[2]), DMUL(nc0[2], nc1[1]));
    n[1] = DSUB(DMUL(nc0[2], nc1[0]), DMUL(nc0[0], nc1[2]));
    n[2] = DSUB(DMUL(nc0[0], nc1[1]), DMUL(nc0[1], nc1[0]));
    const double nn = __dsqrt_rn(DADD(DADD(DMUL(n[0], n[0]), DMUL(n[1], n[1])), DMUL(n[2], n[2])));
    n[0] = DDIV(n[0], nn);
    n[1] = DDIV(n[1], nn);
    n[2] = DDIV(n[2], nn);
    const double iv2 = -DADD(DADD(DMUL(n[0], hm[0]), DMUL(n[1], hm[1])), DMUL(n[2], hm[2]));
    const double ia = acos(DDIV(iv2, t));
    const size_t o = (size_t)f * ntau + s;
    if (MODE == MODE_FP64) static_cast<double*>(a.s.cosil)[o] = cos(ia);
    else static_cast<float*>(a.s.cosil)[o] = (float)cos(ia);
    a.s.shadow[o] = (ia > (3.141592653589793 / 2.0)) ? 0 : 1;
    double* hmo = a.g.hm + o * 3;
    double* no = a.g.nrm + o * 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) { hmo[k] = hm[k]; no[k] = n[k]; }
    a.g.dist[o] = t;
}

// astshadowtest: 0 when facet h blocks the ray from the Sun (origin) to g's midpoint
__device__ __forceinline__ int dev_shadowtest(const GeomArgs& a, int g, int h, int s) {
    const int ntau = a.s.ntau;
    const double* Gm = a.g.hm + ((size_t)g * ntau + s) * 3;
    const double* Hm = a.g.hm + ((size_t)h * ntau + s) * 3;
    const double* Hn = a.g.nrm + ((size_t)h * ntau + s) * 3;
    const int* hv = a.s.fac + 3 * h;
    const double* V0 = a.g.hp + ((size_t)hv[0] * ntau + s) * 3;
    const double* V1 = a.g.hp + ((size_t)hv[1] * ntau + s) * 3;
    const double* V2 = a.g.hp + ((size_t)hv[2] * ntau + s) * 3;
    const double tc2 = DADD(DADD(DMUL(Gm[0], Hn[0]), DMUL(Gm[1], Hn[1])), DMUL(Gm[2], Hn[2]));
    const double tc1 = DADD(DADD(DMUL(Hm[0], Hn[0]), DMUL(Hm[1], Hn[1])), DMUL(Hm[2], Hn[2]));
    const double t = DDIV(tc1, tc2);
    double x[3], n1[3], n2[3], n3[3], x1[3], x2[3], x3[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        x[k] = DMUL(t, Gm[k]);
        n1[k] = DSUB(V1[k], V0[k]);
        n2[k] = DSUB(V0[k], V2[k]);
        n3[k] = DSUB(V2[k], V1[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        x1[k] = DSUB(x[k], V0[k]);
        x3[k] = DSUB(x[k], V1[k]);
        x2[k] = DSUB(x[k], V2[k]);
    }
    double t1[3], t2[3], t3[3];
    t1[0] = DSUB(DMUL(n1[1], x1[2]), DMUL(n1[2], x1[1]));
    t1[1] = DSUB(DMUL(n1[2], x1[0]), DMUL(n1[0], x1[2]));
    t1[2] = DSUB(DMUL(n1[0], x1[1]), DMUL(n1[1], x1[0]));
    t2[0] = DSUB(DMUL(n2[1], x2[2]), DMUL(n2[2], x2[1]));
    t2[1] = DSUB(DMUL(n2[2], x2[0]), DMUL(n2[0], x2[2]));
    t2[2] = DSUB(DMUL(n2[0], x2[1]), DMUL(n2[1], x2[0]));
    t3[0] = DSUB(DMUL(n3[1], x3[2]), DMUL(n3[2], x3[1]));
    t3[1] = DSUB(DMUL(n3[2], x3[0]), DMUL(n3[0], x3[2]));
    t3[2] = DSUB(DMUL(n3[0], x3[1]), DMUL(n3[1], x3[0]));
    const double c1 = DADD(DADD(DMUL(t1[0], Hn[0]), DMUL(t1[1], Hn[1])), DMUL(t1[2], Hn[2]));
    const double c2 = DADD(DADD(DMUL(t2[0], Hn[0]), DMUL(t2[1], Hn[1])), DMUL(t2[2], Hn[2]));
    const double c3 = DADD(DADD(DMUL(t3[0], Hn[0]), DMUL(t3[1], Hn[1])), DMUL(t3[2], Hn[2]));
    return (c1 >= 0.0 && c2 >= 0.0 && c3 >= 0.0) ? 0 : 1;
}

// dependent-list shadowing; warp = 32 consecutive steps of one facet
__global__ void __launch_bounds__(256) k_shadow_dep(GeomArgs a) {
    const int nf = a.s.nf, ntau = a.s.ntau;
    const int g = blockIdx.y * blockDim.y + threadIdx.y;
    const int s = blockIdx.x * 32 + threadIdx.x;
    if (g >= nf) return;
    const int d0 = a.s.dep_ptr[g], d1 = a.s.dep_ptr[g + 1];
    if (d0 == d1) return;
    const bool valid = s < ntau;
    const size_t o = (size_t)g * ntau + (valid ? s : 0);
    bool lit = valid && a.s.shadow[o] == 1;
    const double gd = a.g.dist[o];
    for (int k = d0; k < d1; ++k) {
        if (!__any_sync(0xffffffffu, lit)) break;
        const int h = __ldg(&a.s.dep_idx[k]);
        if (lit) {
            const double hd = a.g.dist[(size_t)h * ntau + s];
            if (gd > hd && dev_shadowtest(a, g, h, s) == 0) lit = false;
        }
    }
    if (valid && !lit) a.s.shadow[o] = 0;
}

// all pairs: facet g is tested against every h with |h| < |g| (the reference
// loops g < h and tests whichever of the two is farther from the Sun; the
// outcome per facet is the same AND over occluders)
__global__ void __launch_bounds__(256) k_shadow_all(GeomArgs a) {
    const int nf = a.s.nf, ntau = a.s.ntau;
    const int g = blockIdx.y * blockDim.y + threadIdx.y;
    const int s = blockIdx.x * 32 + threadIdx.x;
    if (g >= nf) return;
    const bool valid = s < ntau;
    const size_t o = (size_t)g * ntau + (valid ? s : 0);
    bool lit = valid && a.s.shadow[o] == 1;
    const double gd = a.g.dist[o];
    for (int h = 0; h < nf; ++h) {
        if (!__any_sync(0xffffffffu, lit)) break;
        if (h == g) continue;
        if (lit) {
            const double hd = a.g.dist[(size_t)h * ntau + s];
            // pair (min,max): reference tests the farther facet when strictly
            // farther; for equal distances the higher index is tested
            const bool g_tested = (g < h) ? (gd > hd) : !(hd > gd);
            if (g_tested && dev_shadowtest(a, g, h, s) == 0) lit = false;
        }
    }
    if (valid && !lit) a.s.shadow[o] = 0;
}

int launch_geometry(const DevSolve& s, const GeomWork& g, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    GeomArgs a{s, g};
    const long long nvt = (long long)s.nv * s.ntau, nft = (long long)s.nf * s.ntau;
    k_geom_vertices<<<(unsigned)((nvt + 255) / 256), 256, 0, st>>>(a);
    if (s.mode == MODE_FP64) k_geom_facets<MODE_FP64><<<(unsigned)((nft + 255) / 256), 256, 0, st>>>(a);
    else k_geom_facets<MODE_REF><<<(unsigned)((nft + 255) / 256), 256, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_shadow_deplist(const DevSolve& s, const GeomWork& g, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    GeomArgs a{s, g};
    dim3 blk(32, 8), grd((s.ntau + 31) / 32, (s.nf + 7) / 8);
    k_shadow_dep<<<grd, blk, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_shadow_allpairs(const DevSolve& s, const GeomWork& g, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    GeomArgs a{s, g};
    dim3 blk(32, 8), grd((s.ntau + 31) / 32, (s.nf + 7) / 8);
    k_shadow_all<<<grd, blk, 0, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // namespace atpm
