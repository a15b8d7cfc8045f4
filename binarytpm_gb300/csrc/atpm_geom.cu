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
// Culled drivers (same flags, far fewer exact tests): every ray starts at the
// origin (the Sun, or the observer in the Visibility stage), so the test is
// two-dimensional in the central projection onto the plane normal to the
// body's direction.  If the exact test puts the ray's point inside facet h,
// the projection of g's midpoint lies inside h's projected triangle, hence
// inside its bounding box: a box test (FP32, padded far beyond the FP64
// test's rounding) rejects every other pair before the exact FP64 test.
//   k_proj           projected vertex coordinates of every step
//   k_window_box     each facet's box over every window of 32 steps
//   k_shadow_dep_cull the dependent-list driver with the box tests in front
//   k_grid_*         a uniform grid per step over the projected facets
//                    (one cell per facet, by its box centre; cell size the
//                    largest box), built by counting sort
//   k_shadow_grid    the all-pairs driver over the 3 x 3 cells around g
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

#include <algorithm>
#include <cstring>

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
    // a non-synchronous secondary turns at its own rate (its own table)
    const double* rt = (v < a.g.vsplit) ? a.g.rot : a.g.rot2;
    const double c = rt[2 * s], sn = rt[2 * s + 1];
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
    const double ci = DDIV(iv2, t);
    const size_t o = (size_t)f * ntau + s;
    if (MODE == MODE_FAST) {
        // FAST: the cosine itself (cos(acos(x)) is x up to its last bits,
        // and the FP64 transcendentals are most of this kernel's time on a
        // part whose FP64 rate is 1/64 of FP32); dark when it is negative
        static_cast<float*>(a.s.cosil)[o] = (float)ci;
        a.s.shadow[o] = ci < 0.0 ? 0 : 1;
    } else {
        const double ia = acos(ci);
        if (MODE == MODE_FP64) static_cast<double*>(a.s.cosil)[o] = cos(ia);
        else static_cast<float*>(a.s.cosil)[o] = (float)cos(ia);
        a.s.shadow[o] = (ia > (3.141592653589793 / 2.0)) ? 0 : 1;
    }
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

// ------------------------------------------------------------- culled drivers
struct ProjArgs {
    double c[3], e1[3], e2[3];  // projection frame: body direction and two normals
    double scale;               // |body centre|: projected coordinates in km
    float pad;                  // box padding (km)
    float2* uv;                 // [nv][ntau]
    unsigned* stats;            // [0] max |u|,|v| (float bits), [1] max box extent, [2] bad-projection flag
    float4* wbox;               // [nf][ceil(ntau/32)] union of each facet's padded boxes over 32 steps (or null)
};

__global__ void __launch_bounds__(256) k_proj(GeomArgs a, ProjArgs p) {
    const int nv = a.s.nv, ntau = a.s.ntau;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nv * ntau) return;
    const double* P = a.g.hp + (size_t)i * 3;   // [v][s][3], i = v * ntau + s
    const double d = P[0] * p.c[0] + P[1] * p.c[1] + P[2] * p.c[2];
    const double n2 = P[0] * P[0] + P[1] * P[1] + P[2] * P[2];
    if (!(d > 0.5 * sqrt(n2))) { atomicOr(&p.stats[2], 1u); return; }
    const double u = (P[0] * p.e1[0] + P[1] * p.e1[1] + P[2] * p.e1[2]) / d * p.scale;
    const double v = (P[0] * p.e2[0] + P[1] * p.e2[1] + P[2] * p.e2[2]) / d * p.scale;
    p.uv[i] = make_float2((float)u, (float)v);
    const float m = fmaxf(fabsf((float)u), fabsf((float)v));
    atomicMax(&p.stats[0], __float_as_uint(m));
}

__device__ __forceinline__ float4 facet_box(const GeomArgs& a, const ProjArgs& p, int h, int s) {
    const int* hv = a.s.fac + 3 * h;
    const int ntau = a.s.ntau;
    const float2 q0 = p.uv[(size_t)hv[0] * ntau + s], q1 = p.uv[(size_t)hv[1] * ntau + s],
                 q2 = p.uv[(size_t)hv[2] * ntau + s];
    return make_float4(fminf(q0.x, fminf(q1.x, q2.x)) - p.pad, fmaxf(q0.x, fmaxf(q1.x, q2.x)) + p.pad,
                       fminf(q0.y, fminf(q1.y, q2.y)) - p.pad, fmaxf(q0.y, fmaxf(q1.y, q2.y)) + p.pad);
}

// each facet's padded box over every window of 32 steps (the union of its
// 32 per-step boxes): a warp of the dependent-list driver covers one window,
// and an occluder whose window box misses the box around the warp's lit
// points cannot pass any lane's per-step box test
__global__ void __launch_bounds__(256) k_window_box(GeomArgs a, ProjArgs p) {
    const int ntau = a.s.ntau, nw = (ntau + 31) / 32;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)a.s.nf * nw) return;
    const int h = (int)(i / nw), w = (int)(i % nw);
    float4 u = make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
    for (int s = w * 32; s < min(ntau, w * 32 + 32); ++s) {
        const float4 b = facet_box(a, p, h, s);
        u = make_float4(fminf(u.x, b.x), fmaxf(u.y, b.y), fminf(u.z, b.z), fmaxf(u.w, b.w));
    }
    p.wbox[i] = u;
}

__device__ __forceinline__ float2 mid_uv(const GeomArgs& a, const ProjArgs& p, int g, int s) {
    const double* G = a.g.hm + ((size_t)g * a.s.ntau + s) * 3;
    const double d = G[0] * p.c[0] + G[1] * p.c[1] + G[2] * p.c[2];
    return make_float2((float)((G[0] * p.e1[0] + G[1] * p.e1[1] + G[2] * p.e1[2]) / d * p.scale),
                       (float)((G[0] * p.e2[0] + G[1] * p.e2[1] + G[2] * p.e2[2]) / d * p.scale));
}

__device__ __forceinline__ bool in_box(float2 q, float4 b) {
    return q.x >= b.x && q.x <= b.y && q.y >= b.z && q.y <= b.w;
}

// adds a thread's exact-test count to the launch's tally: one add per group
// of lanes leaving together, spread over 64 counters
__device__ __forceinline__ void count_tests(unsigned long long* ctr, unsigned n) {
    if (!ctr) return;
    const unsigned m = __activemask();
    const unsigned t = __reduce_add_sync(m, n);
    unsigned lane;
    asm("mov.u32 %0, %%laneid;" : "=r"(lane));
    if (lane == (unsigned)(__ffs(m) - 1) && t) atomicAdd(&ctr[blockIdx.x & 63], (unsigned long long)t);
}

// dependent-list shadowing with the box test in front of the exact test
__global__ void __launch_bounds__(256) k_shadow_dep_cull(GeomArgs a, ProjArgs p) {
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
    const float2 q = valid ? mid_uv(a, p, g, s) : make_float2(0.f, 0.f);
    unsigned ntest = 0;
    // the box around this warp's lit points (empty when none is lit)
    float4 qb = lit ? make_float4(q.x, q.x, q.y, q.y) : make_float4(INFINITY, -INFINITY, INFINITY, -INFINITY);
    for (int o2 = 16; o2 > 0; o2 >>= 1) {
        qb.x = fminf(qb.x, __shfl_xor_sync(0xffffffffu, qb.x, o2));
        qb.y = fmaxf(qb.y, __shfl_xor_sync(0xffffffffu, qb.y, o2));
        qb.z = fminf(qb.z, __shfl_xor_sync(0xffffffffu, qb.z, o2));
        qb.w = fmaxf(qb.w, __shfl_xor_sync(0xffffffffu, qb.w, o2));
    }
    const float4* wb = p.wbox ? p.wbox + blockIdx.x : nullptr;  // this warp's step window
    const int nw = (ntau + 31) / 32;
    for (int k = d0; k < d1; ++k) {
        if (!__any_sync(0xffffffffu, lit)) break;
        const int h = __ldg(&a.s.dep_idx[k]);
        if (wb) {  // warp-uniform: h's window box misses every lit point of the warp
            const float4 u = __ldg(wb + (size_t)h * nw);
            if (u.x > qb.y || u.y < qb.x || u.z > qb.w || u.w < qb.z) continue;
        }
        if (lit && in_box(q, facet_box(a, p, h, s))) {
            const double hd = a.g.dist[(size_t)h * ntau + s];
            if (gd > hd) {
                ++ntest;
                if (dev_shadowtest(a, g, h, s) == 0) lit = false;
            }
        }
    }
    if (valid && !lit) a.s.shadow[o] = 0;
    count_tests(a.g.tests, ntest);
}

struct GridArgs {
    int G;          // cells per side
    float cell;     // cell size (km)
    float origin;   // grid spans [origin, origin + G * cell) on both axes
    int s0, ns;     // steps of this chunk
    int* key;       // [ns][nf] cell of each facet
    int* start;     // [ns][G*G + 1] exclusive scan of the cell counts
    int* cursor;    // [ns][G*G]
    int* list;      // [ns][nf] facets by cell
};

__device__ __forceinline__ int cell_of(const GridArgs& gr, float x) {
    int c = (int)floorf((x - gr.origin) / gr.cell);
    return c < 0 ? 0 : (c >= gr.G ? gr.G - 1 : c);
}

__global__ void __launch_bounds__(256) k_grid_extent(GeomArgs a, ProjArgs p) {
    const int nf = a.s.nf, ntau = a.s.ntau;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nf * ntau) return;
    const int f = (int)(i / ntau), s = (int)(i % ntau);
    const float4 b = facet_box(a, p, f, s);
    atomicMax(&p.stats[1], __float_as_uint(fmaxf(b.y - b.x, b.w - b.z)));
}

__global__ void __launch_bounds__(256) k_grid_count(GeomArgs a, ProjArgs p, GridArgs gr) {
    const int nf = a.s.nf;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nf * gr.ns) return;
    const int k = (int)(i / nf), f = (int)(i % nf), s = gr.s0 + k;
    const float4 b = facet_box(a, p, f, s);
    const int c = cell_of(gr, 0.5f * (b.z + b.w)) * gr.G + cell_of(gr, 0.5f * (b.x + b.y));
    gr.key[i] = c;
    atomicAdd(&gr.start[(size_t)k * (gr.G * gr.G + 1) + c + 1], 1);
}

// in-place inclusive scan of start[k][1..G*G] (so start[k][c] = first slot of cell c)
__global__ void __launch_bounds__(1024) k_grid_scan(GridArgs gr) {
    __shared__ int carry;
    __shared__ int part[1024];
    const int n = gr.G * gr.G;
    int* st = gr.start + (size_t)blockIdx.x * (n + 1);
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 1; base <= n; base += 1024) {
        const int j = base + threadIdx.x;
        int v = j <= n ? st[j] : 0;
        part[threadIdx.x] = v;
        __syncthreads();
        for (int w = 1; w < 1024; w <<= 1) {
            const int t = threadIdx.x >= w ? part[threadIdx.x - w] : 0;
            __syncthreads();
            part[threadIdx.x] += t;
            __syncthreads();
        }
        if (j <= n) st[j] = part[threadIdx.x] + carry;
        __syncthreads();
        if (threadIdx.x == 1023) carry += part[1023];
        __syncthreads();
    }
    int* cu = gr.cursor + (size_t)blockIdx.x * n;
    for (int c = threadIdx.x; c < n; c += 1024) cu[c] = st[c];
}

__global__ void __launch_bounds__(256) k_grid_fill(GeomArgs a, GridArgs gr) {
    const int nf = a.s.nf;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nf * gr.ns) return;
    const int k = (int)(i / nf), f = (int)(i % nf);
    const int slot = atomicAdd(&gr.cursor[(size_t)k * gr.G * gr.G + gr.key[i]], 1);
    gr.list[(size_t)k * nf + slot] = f;
}

// all pairs over the grid: the candidates of g are the facets filed in the
// 3 x 3 cells around g's projected midpoint (a cell is as wide as the
// largest box, so every box containing the point is filed there)
__global__ void __launch_bounds__(256) k_shadow_grid(GeomArgs a, ProjArgs p, GridArgs gr) {
    const int nf = a.s.nf, ntau = a.s.ntau;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nf * gr.ns) return;
    const int k = (int)(i / nf), g = (int)(i % nf), s = gr.s0 + k;
    const size_t o = (size_t)g * ntau + s;
    if (a.s.shadow[o] != 1) return;
    const double gd = a.g.dist[o];
    const float2 q = mid_uv(a, p, g, s);
    const int cx = cell_of(gr, q.x), cy = cell_of(gr, q.y);
    const int n = gr.G * gr.G;
    const int* st = gr.start + (size_t)k * (n + 1);
    const int* li = gr.list + (size_t)k * nf;
    unsigned ntest = 0;
    for (int y = max(cy - 1, 0); y <= min(cy + 1, gr.G - 1); ++y)
        for (int x = max(cx - 1, 0); x <= min(cx + 1, gr.G - 1); ++x) {
            const int c = y * gr.G + x;
            for (int j = st[c]; j < st[c + 1]; ++j) {
                const int h = li[j];
                if (h == g || !in_box(q, facet_box(a, p, h, s))) continue;
                const double hd = a.g.dist[(size_t)h * ntau + s];
                const bool g_tested = (g < h) ? (gd > hd) : !(hd > gd);
                if (!g_tested) continue;
                ++ntest;
                if (dev_shadowtest(a, g, h, s) == 0) {
                    a.s.shadow[o] = 0;
                    count_tests(a.g.tests, ntest);
                    return;
                }
            }
        }
    count_tests(a.g.tests, ntest);
}

namespace {
// projection frame of the body direction; returns false when the body is
// too close to the origin for a central projection (the caller then runs
// the plain drivers)
bool make_frame(const GeomWork& g, ProjArgs& p) {
    const double n = sqrt(g.car[0] * g.car[0] + g.car[1] * g.car[1] + g.car[2] * g.car[2]);
    if (!(n > 0.0)) return false;
    for (int k = 0; k < 3; ++k) p.c[k] = g.car[k] / n;
    // e1: the coordinate axis least aligned with c, made orthogonal
    int ax = 0;
    for (int k = 1; k < 3; ++k)
        if (fabs(p.c[k]) < fabs(p.c[ax])) ax = k;
    double t[3] = {0, 0, 0};
    t[ax] = 1.0;
    const double dt = t[0] * p.c[0] + t[1] * p.c[1] + t[2] * p.c[2];
    for (int k = 0; k < 3; ++k) p.e1[k] = t[k] - dt * p.c[k];
    const double n1 = sqrt(p.e1[0] * p.e1[0] + p.e1[1] * p.e1[1] + p.e1[2] * p.e1[2]);
    for (int k = 0; k < 3; ++k) p.e1[k] /= n1;
    p.e2[0] = p.c[1] * p.e1[2] - p.c[2] * p.e1[1];
    p.e2[1] = p.c[2] * p.e1[0] - p.c[0] * p.e1[2];
    p.e2[2] = p.c[0] * p.e1[1] - p.c[1] * p.e1[0];
    p.scale = n;
    // 1 cm: orders of magnitude beyond the FP64 test's rounding at 1 AU
    // (3e-8 km) and the float rounding of projected km-scale coordinates
    p.pad = 1e-5f;
    return true;
}

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }
}  // namespace

// returns 0 when the culled driver ran, -1 when the caller should fall back
int launch_shadow_culled(const DevSolve& s, const GeomWork& g, bool all_pairs, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    GeomArgs a{s, g};
    ProjArgs p{};
    if (!make_frame(g, p)) return -1;
    const long long nvt = (long long)s.nv * s.ntau, nft = (long long)s.nf * s.ntau;
    void* mem = nullptr;
    const size_t b_uv = al256((size_t)nvt * sizeof(float2));
    if (cudaMallocAsync(&mem, b_uv + 256, st) != cudaSuccess) return 2;
    p.uv = static_cast<float2*>(mem);
    p.stats = reinterpret_cast<unsigned*>(static_cast<char*>(mem) + b_uv);
    cudaMemsetAsync(p.stats, 0, 16, st);
    k_proj<<<(unsigned)((nvt + 255) / 256), 256, 0, st>>>(a, p);
    if (all_pairs) k_grid_extent<<<(unsigned)((nft + 255) / 256), 256, 0, st>>>(a, p);
    unsigned stats[3] = {0, 0, 0};
    if (cudaMemcpyAsync(stats, p.stats, 12, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaFreeAsync(mem, st);
        return 2;
    }
    if (stats[2]) {  // a vertex too far off the body direction: no projection
        cudaFreeAsync(mem, st);
        return -1;
    }
    int rc = 0;
    if (!all_pairs) {
        const long long nwt = (long long)s.nf * ((s.ntau + 31) / 32);
        void* wm = nullptr;
        if (cudaMallocAsync(&wm, (size_t)nwt * sizeof(float4), st) == cudaSuccess) {
            p.wbox = static_cast<float4*>(wm);
            k_window_box<<<(unsigned)((nwt + 255) / 256), 256, 0, st>>>(a, p);
        } else {
            cudaGetLastError();  // without window boxes: the per-step tests alone (same flags)
        }
        dim3 blk(32, 8), grd((s.ntau + 31) / 32, (s.nf + 7) / 8);
        k_shadow_dep_cull<<<grd, blk, 0, st>>>(a, p);
        if (wm) cudaFreeAsync(wm, st);
    } else {
        float umax, ext;
        memcpy(&umax, &stats[0], 4);
        memcpy(&ext, &stats[1], 4);
        GridArgs gr{};
        gr.cell = ext * 1.0001f + 1e-6f;
        gr.origin = -(umax + 2.0f * p.pad) - gr.cell;
        long long G = (long long)ceilf(2.0f * -gr.origin / gr.cell) + 1;
        if (G > 2048) {  // a few huge facets: coarser cells, still correct
            G = 2048;
            gr.cell = 2.0f * -gr.origin / 2000.0f;
        }
        gr.G = (int)G;
        const size_t n = (size_t)G * G;
        // steps per chunk: at most ~64 M grid entries at once
        int sc = (int)std::max<size_t>(1, std::min<size_t>((size_t)s.ntau, (64u << 20) / (n + 1)));
        const size_t b_key = al256((size_t)sc * s.nf * 4), b_st = al256((size_t)sc * (n + 1) * 4),
                     b_cu = al256((size_t)sc * n * 4);
        void* gm = nullptr;
        if (cudaMallocAsync(&gm, 2 * b_key + b_st + b_cu, st) != cudaSuccess) {
            cudaFreeAsync(mem, st);
            return 2;
        }
        char* t = static_cast<char*>(gm);
        gr.key = reinterpret_cast<int*>(t);
        gr.list = reinterpret_cast<int*>(t + b_key);
        gr.start = reinterpret_cast<int*>(t + 2 * b_key);
        gr.cursor = reinterpret_cast<int*>(t + 2 * b_key + b_st);
        for (int s0 = 0; s0 < s.ntau && !rc; s0 += sc) {
            gr.s0 = s0;
            gr.ns = std::min(sc, s.ntau - s0);
            const long long m = (long long)s.nf * gr.ns;
            cudaMemsetAsync(gr.start, 0, (size_t)gr.ns * (n + 1) * 4, st);
            k_grid_count<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(a, p, gr);
            k_grid_scan<<<gr.ns, 1024, 0, st>>>(gr);
            k_grid_fill<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(a, gr);
            k_shadow_grid<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(a, p, gr);
            if (cudaGetLastError() != cudaSuccess) rc = 2;
        }
        cudaFreeAsync(gm, st);
    }
    cudaFreeAsync(mem, st);
    if (cudaGetLastError() != cudaSuccess) rc = 2;
    return rc;
}

// The Sun direction in every facet's local frame, the crater model's input
// (asteroidgeometry, 3905/Thermal/NominalPole/main.cpp:967-1030): frame rows
// = the first edge (unit), normal x edge, the unit normal; the vector is
// -frame . heliocentric midpoint, scaled to length 10^4 and rounded to float.
// The facet's final shadow flag (self-shadow and astshadow) goes beside it.
// Facets f0 .. f0 + nfc - 1; outputs [nfc][ntau][3] and [nfc][ntau].
__global__ void __launch_bounds__(256) k_crater_sun(GeomArgs a, int f0, int nfc, float* sun, int* shadow) {
    const int ntau = a.s.ntau;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nfc * ntau) return;
    const int fl = (int)(i / ntau), s = (int)(i % ntau), f = f0 + fl;
    const int* fv = a.s.fac + 3 * f;
    const double* h0 = a.g.hp + ((size_t)fv[0] * ntau + s) * 3;
    const double* h1 = a.g.hp + ((size_t)fv[1] * ntau + s) * 3;
    const double* h2 = a.g.hp + ((size_t)fv[2] * ntau + s) * 3;
    double hm[3], n[3], nc0[3], nc1[3], y[3];
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
    const double x = __dsqrt_rn(DADD(DADD(DMUL(nc0[0], nc0[0]), DMUL(nc0[1], nc0[1])), DMUL(nc0[2], nc0[2])));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        n[k] = DDIV(n[k], nn);
        nc0[k] = DDIV(nc0[k], x);
    }
    y[0] = DSUB(DMUL(n[1], nc0[2]), DMUL(n[2], nc0[1]));
    y[1] = DSUB(DMUL(n[2], nc0[0]), DMUL(n[0], nc0[2]));
    y[2] = DSUB(DMUL(n[0], nc0[1]), DMUL(n[1], nc0[0]));
    const double* row[3] = {nc0, y, n};
    float* out = sun + ((size_t)fl * ntau + s) * 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double iv = -DADD(DADD(DMUL(row[k][0], hm[0]), DMUL(row[k][1], hm[1])), DMUL(row[k][2], hm[2]));
        out[k] = (float)DDIV(DMUL(10000.0, iv), t);
    }
    shadow[(size_t)fl * ntau + s] = a.s.shadow[(size_t)f * ntau + s];
}

int launch_crater_sun(const DevSolve& s, const GeomWork& g, int f0, int nfc, float* sun, int* shadow, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    GeomArgs a{s, g};
    const long long nvt = (long long)s.nv * s.ntau, nct = (long long)nfc * s.ntau;
    k_geom_vertices<<<(unsigned)((nvt + 255) / 256), 256, 0, st>>>(a);
    k_crater_sun<<<(unsigned)((nct + 255) / 256), 256, 0, st>>>(a, f0, nfc, sun, shadow);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_geometry(const DevSolve& s, const GeomWork& g, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    GeomArgs a{s, g};
    const long long nvt = (long long)s.nv * s.ntau, nft = (long long)s.nf * s.ntau;
    k_geom_vertices<<<(unsigned)((nvt + 255) / 256), 256, 0, st>>>(a);
    if (s.mode == MODE_FP64) k_geom_facets<MODE_FP64><<<(unsigned)((nft + 255) / 256), 256, 0, st>>>(a);
    else if (s.mode == MODE_FAST) k_geom_facets<MODE_FAST><<<(unsigned)((nft + 255) / 256), 256, 0, st>>>(a);
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
