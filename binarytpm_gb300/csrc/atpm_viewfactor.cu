// Facet-to-facet view factors (the reference's Shape_Selfheating stage,
// 3905/Shape_Selfheating/main.cpp).  FP32 throughout, like the reference,
// with round-to-nearest intrinsics in its operand order.
//
//   k_vf_count   per facet I: number of facets J with both normals facing
//                (thetai, thetaj <= pi/2 via acos, main.cpp:653-665)
//   k_vf_fill    the same screen, writing J in index order with
//                vf = cos(ti) cos(tj) A_J / (pi d^2) and the area-weighted
//                direction (main.cpp:700-735); an ordered block compaction
//                keeps the reference's list order
//   k_vf_hidden  occlusion culling (main.cpp:187-368): candidate Z of facet G
//                is dropped when another candidate S, nearer to Z than G,
//                intersects the segment; candidates are staged through
//                shared memory in chunks
//   k_vf_refine  10x10 sub-triangle refinement of every pair with
//                vf >= 0.05 (main.cpp:374-622)
//
// The facing test and cos(theta) go through the device's acosf/cosf, so a
// pair whose cos is within ~1e-7 of zero may be classified differently from
// the reference and view factors agree to float rounding (the reference
// writes them with 6 significant digits).
#include <cuda_runtime.h>

#include <cstdint>

namespace atpm {

#define FADD __fadd_rn
#define FSUB __fsub_rn
#define FMUL __fmul_rn
#define FDIV __fdiv_rn
#define FSQRT __fsqrt_rn

struct VfGeom {
    int nv, nf;
    const float* v;      // [nv][3]
    const int* fac;      // [nf][3]
    float* mid;          // [nf][3]
    float* nrm;          // [nf][3] un-normalised (v1-v0)x(v2-v0)
    float* area;         // [nf]
    float* nlen;         // [nf] |nrm|
};

__constant__ float c_PIF = 3.14159274101257324f;  // 4.0f*atan(1.0f) (main.cpp:8)

// initialise (main.cpp:750-811)
__global__ void k_vf_init(VfGeom g) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.nf) return;
    const float* a = g.v + 3 * g.fac[3 * c];
    const float* b = g.v + 3 * g.fac[3 * c + 1];
    const float* d = g.v + 3 * g.fac[3 * c + 2];
    float n0[3], n1[3], n[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        g.mid[3 * c + k] = FDIV(FADD(FADD(a[k], b[k]), d[k]), 3.0f);
        n0[k] = FSUB(b[k], a[k]);
        n1[k] = FSUB(d[k], a[k]);
    }
    n[0] = FSUB(FMUL(n0[1], n1[2]), FMUL(n0[2], n1[1]));
    n[1] = FSUB(FMUL(n0[2], n1[0]), FMUL(n0[0], n1[2]));
    n[2] = FSUB(FMUL(n0[0], n1[1]), FMUL(n0[1], n1[0]));
    const float l = FSQRT(FADD(FADD(FMUL(n[0], n[0]), FMUL(n[1], n[1])), FMUL(n[2], n[2])));
    g.area[c] = FDIV(l, 2.0f);
    g.nlen[c] = l;
#pragma unroll
    for (int k = 0; k < 3; ++k) g.nrm[3 * c + k] = n[k];
}

struct PairEval {
    bool facing;
    float vf, dir[3];
};

// main.cpp:700-735 for one (I, J)
__device__ __forceinline__ PairEval pair_eval(const VfGeom& g, int I, int J, bool want_vf) {
    PairEval r;
    float s[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) s[k] = FSUB(g.mid[3 * J + k], g.mid[3 * I + k]);
    const float d = FSQRT(FADD(FADD(FMUL(s[0], s[0]), FMUL(s[1], s[1])), FMUL(s[2], s[2])));
    const float ni = g.nlen[I], nj = g.nlen[J];
    const float* nI = g.nrm + 3 * I;
    const float* nJ = g.nrm + 3 * J;
    const float xi = FDIV(FADD(FADD(FMUL(nI[0], s[0]), FMUL(nI[1], s[1])), FMUL(nI[2], s[2])), FMUL(ni, d));
    const float xj = FDIV(FADD(FADD(FMUL(-nJ[0], s[0]), FMUL(-nJ[1], s[1])), FMUL(-nJ[2], s[2])), FMUL(nj, d));
    const float ti = acosf(xi), tj = acosf(xj);
    const float half = FDIV(c_PIF, 2.0f);
    r.facing = (ti <= half) && (tj <= half);
    if (r.facing && want_vf) {
        float vf = FDIV(FMUL(FMUL(cosf(ti), cosf(tj)), g.area[J]), FMUL(FMUL(c_PIF, d), d));
        if (vf < 0.0f) vf = 0.0f;
        r.vf = vf;
        const float aI = g.area[I];
#pragma unroll
        for (int k = 0; k < 3; ++k) r.dir[k] = FMUL(FMUL(aI, vf), FDIV(s[k], d));
    }
    return r;
}

__global__ void __launch_bounds__(256) k_vf_count(VfGeom g, int* count) {
    const int I = blockIdx.x;
    int c = 0;
    for (int J = threadIdx.x; J < g.nf; J += blockDim.x)
        if (J != I && pair_eval(g, I, J, false).facing) ++c;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    __shared__ int ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
        count[I] = t;
    }
}

// ordered fill: 256 candidates per round, ballot + warp prefix keeps J order
__global__ void __launch_bounds__(256) k_vf_fill(VfGeom g, const long long* ptr, int* idx, float* vf, float* dir) {
    const int I = blockIdx.x;
    __shared__ int woff[9];
    long long base = ptr[I];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int J0 = 0; J0 < g.nf; J0 += blockDim.x) {
        const int J = J0 + threadIdx.x;
        PairEval p;
        p.facing = false;
        if (J < g.nf && J != I) p = pair_eval(g, I, J, true);
        const unsigned m = __ballot_sync(0xffffffffu, p.facing);
        if (lane == 0) woff[w] = __popc(m);
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int k = 0; k < 8; ++k) { const int t = woff[k]; woff[k] = acc; acc += t; }
            woff[8] = acc;
        }
        __syncthreads();
        if (p.facing) {
            const long long o = base + woff[w] + __popc(m & ((1u << lane) - 1u));
            idx[o] = J;
            vf[o] = p.vf;
            dir[3 * o] = p.dir[0];
            dir[3 * o + 1] = p.dir[1];
            dir[3 * o + 2] = p.dir[2];
        }
        base += woff[8];
        __syncthreads();
    }
}

// occlusion culling (main.cpp:187-368).  One block per facet G; thread t
// owns candidates Z = list[t], list[t+256], ...; occluders S are staged.
constexpr int HID_CHUNK = 256;
__global__ void __launch_bounds__(256) k_vf_hidden(VfGeom g, const long long* ptr, const int* idx, uint8_t* keep) {
    const int G = blockIdx.x;
    const long long p0 = ptr[G], p1 = ptr[G + 1];
    const int D = (int)(p1 - p0);
    if (D == 0) return;
    __shared__ float sm_mid[HID_CHUNK][3];
    __shared__ float sm_n[HID_CHUNK][3];
    __shared__ float sm_v[HID_CHUNK][9];
    __shared__ float sm_nc[HID_CHUNK][9];
    __shared__ int sm_id[HID_CHUNK];
    const float* Gm = g.mid + 3 * G;
    for (int z0 = 0; z0 < D; z0 += blockDim.x) {
        const int zi = z0 + threadIdx.x;
        const bool zvalid = zi < D;
        const int Z = zvalid ? idx[p0 + zi] : 0;
        float gv[3], zm[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) { zm[k] = g.mid[3 * Z + k]; gv[k] = FSUB(Gm[k], zm[k]); }
        const float gl = FSQRT(FADD(FADD(FMUL(gv[0], gv[0]), FMUL(gv[1], gv[1])), FMUL(gv[2], gv[2])));
        bool view = true;
        for (int s0 = 0; s0 < D; s0 += HID_CHUNK) {
            const int n = min(HID_CHUNK, D - s0);
            __syncthreads();
            for (int t = threadIdx.x; t < n; t += blockDim.x) {
                const int S = idx[p0 + s0 + t];
                sm_id[t] = S;
                const int* fv = g.fac + 3 * S;
                const float* V0 = g.v + 3 * fv[0];
                const float* V1 = g.v + 3 * fv[1];
                const float* V2 = g.v + 3 * fv[2];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    sm_mid[t][k] = g.mid[3 * S + k];
                    sm_n[t][k] = g.nrm[3 * S + k];
                    sm_v[t][k] = V0[k];
                    sm_v[t][3 + k] = V1[k];
                    sm_v[t][6 + k] = V2[k];
                    sm_nc[t][k] = FSUB(V1[k], V0[k]);         // normcalc1
                    sm_nc[t][3 + k] = -FSUB(V2[k], V0[k]);    // normcalc2 = -(v2-v0)
                    sm_nc[t][6 + k] = FSUB(V2[k], V1[k]);     // normcalc3
                }
            }
            __syncthreads();
            if (!zvalid || !view) continue;
            for (int j = 0; j < n; ++j) {
                const int S = sm_id[j];
                if (S == G || S == Z) continue;
                float sv[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) sv[k] = FSUB(sm_mid[j][k], zm[k]);
                const float sl = FSQRT(FADD(FADD(FMUL(sv[0], sv[0]), FMUL(sv[1], sv[1])), FMUL(sv[2], sv[2])));
                if (!(gl > sl)) continue;
                const float* nS = sm_n[j];
                const float tc1 = FADD(FADD(FMUL(sv[0], nS[0]), FMUL(sv[1], nS[1])), FMUL(sv[2], nS[2]));
                const float tc2 = FADD(FADD(FMUL(gv[0], nS[0]), FMUL(gv[1], nS[1])), FMUL(gv[2], nS[2]));
                const float t = FDIV(tc1, tc2);
                if (!(t > 0.0f)) continue;
                float x[3], x1[3], x2[3], x3[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    x[k] = FADD(FMUL(t, gv[k]), zm[k]);
                    x1[k] = FSUB(x[k], sm_v[j][k]);
                    x3[k] = FSUB(x[k], sm_v[j][3 + k]);
                    x2[k] = FSUB(x[k], sm_v[j][6 + k]);
                }
                const float* c1 = sm_nc[j];
                const float* c2 = sm_nc[j] + 3;
                const float* c3 = sm_nc[j] + 6;
                float t1[3], t2[3], t3[3];
                t1[0] = FSUB(FMUL(c1[1], x1[2]), FMUL(c1[2], x1[1]));
                t1[1] = FSUB(FMUL(c1[2], x1[0]), FMUL(c1[0], x1[2]));
                t1[2] = FSUB(FMUL(c1[0], x1[1]), FMUL(c1[1], x1[0]));
                t2[0] = FSUB(FMUL(c2[1], x2[2]), FMUL(c2[2], x2[1]));
                t2[1] = FSUB(FMUL(c2[2], x2[0]), FMUL(c2[0], x2[2]));
                t2[2] = FSUB(FMUL(c2[0], x2[1]), FMUL(c2[1], x2[0]));
                t3[0] = FSUB(FMUL(c3[1], x3[2]), FMUL(c3[2], x3[1]));
                t3[1] = FSUB(FMUL(c3[2], x3[0]), FMUL(c3[0], x3[2]));
                t3[2] = FSUB(FMUL(c3[0], x3[1]), FMUL(c3[1], x3[0]));
                const float q1 = FADD(FADD(FMUL(t1[0], nS[0]), FMUL(t1[1], nS[1])), FMUL(t1[2], nS[2]));
                const float q2 = FADD(FADD(FMUL(t2[0], nS[0]), FMUL(t2[1], nS[1])), FMUL(t2[2], nS[2]));
                const float q3 = FADD(FADD(FMUL(t3[0], nS[0]), FMUL(t3[1], nS[1])), FMUL(t3[2], nS[2]));
                if (q1 >= 0.0f && q2 >= 0.0f && q3 >= 0.0f) { view = false; break; }
            }
        }
        if (zvalid) keep[p0 + zi] = view ? 1 : 0;
    }
}

// 10x10 refinement (main.cpp:374-622) of pairs with vf >= 0.05.  One block
// per facet I; thread j < 100 owns sub-facet j of I.
__global__ void __launch_bounds__(128) k_vf_refine(VfGeom g, const long long* ptr, const int* idx, float* vf, float* dir) {
    const int I = blockIdx.x;
    const long long p0 = ptr[I], p1 = ptr[I + 1];
    constexpr int n = 10, SUBF = n * n, SUBV = (n + 1) * (n + 2) / 2;
    __shared__ float v1[SUBV][3], v2[SUBV][3];
    __shared__ int tf[SUBF][3];
    __shared__ float m1[SUBF][3], m2[SUBF][3];
    __shared__ float tot[SUBF], totv[SUBF][3];
    // sub-facet connectivity (identical for both triangles, main.cpp:486-543)
    if (threadIdx.x == 0) {
        int l = 0;
        for (int j = 1; j != n + 1; j++) {
            if (j != 1) {
                for (int k = 1; k != j; k++) {
                    tf[l][0] = ((j * (j - 1)) / 2) + k; tf[l][1] = ((j * (j - 1)) / 2) + k - 1; tf[l][2] = ((j * (j + 1)) / 2) + k - 1;
                    ++l;
                    tf[l][0] = ((j * (j + 1)) / 2) + k - 1; tf[l][1] = ((j * (j + 1)) / 2) + k; tf[l][2] = ((j * (j - 1)) / 2) + k;
                    ++l;
                }
            }
            tf[l][0] = (((j + 1) * (j + 2)) / 2) - 2; tf[l][1] = (((j + 1) * (j + 2)) / 2) - 1; tf[l][2] = ((j * (j + 1)) / 2) - 1;
            ++l;
        }
    }
    const float* nI = g.nrm + 3 * I;
    const float ni = g.nlen[I];
    const float aI = g.area[I];
    const float sub1 = FDIV(aI, (float)(n * n));
    const int* fI = g.fac + 3 * I;
    for (long long e = p0; e < p1; ++e) {
        if (!(vf[e] >= 0.05f)) continue;
        const int J = idx[e];
        const int* fJ = g.fac + 3 * J;
        const float* nJ = g.nrm + 3 * J;
        const float nj = g.nlen[J];
        const float sub2 = FDIV(g.area[J], (float)(n * n));
        __syncthreads();
        // sub-vertex tables (main.cpp:466-484)
        for (int t = threadIdx.x; t < SUBV; t += blockDim.x) {
            int l = 0, jj = 1, kk = 1;
            for (int j = 1; j != n + 2; j++)
                for (int k = 1; k != j + 1; k++) { if (l == t) { jj = j; kk = k; } ++l; }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float a1 = FDIV(FSUB(g.v[3 * fI[1] + c], g.v[3 * fI[0] + c]), (float)n);
                const float b1 = FDIV(FSUB(g.v[3 * fI[2] + c], g.v[3 * fI[0] + c]), (float)n);
                const float a2 = FDIV(FSUB(g.v[3 * fJ[1] + c], g.v[3 * fJ[0] + c]), (float)n);
                const float b2 = FDIV(FSUB(g.v[3 * fJ[2] + c], g.v[3 * fJ[0] + c]), (float)n);
                v1[t][c] = FSUB(FADD(g.v[3 * fI[2] + c], FMUL((float)(kk - 1), a1)), FMUL((float)(jj - 1), b1));
                v2[t][c] = FSUB(FADD(g.v[3 * fJ[2] + c], FMUL((float)(kk - 1), a2)), FMUL((float)(jj - 1), b2));
            }
        }
        __syncthreads();
        for (int t = threadIdx.x; t < SUBF; t += blockDim.x)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                m1[t][c] = FDIV(FADD(FADD(v1[tf[t][0]][c], v1[tf[t][1]][c]), v1[tf[t][2]][c]), 3.0f);
                m2[t][c] = FDIV(FADD(FADD(v2[tf[t][0]][c], v2[tf[t][1]][c]), v2[tf[t][2]][c]), 3.0f);
            }
        __syncthreads();
        if (threadIdx.x < SUBF) {
            const int j = threadIdx.x;
            float T = 0.0f, TV[3] = {0.0f, 0.0f, 0.0f};
            for (int k = 0; k != SUBF; k++) {
                float s[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) s[c] = FSUB(m2[k][c], m1[j][c]);
                const float d = FSQRT(FADD(FADD(FMUL(s[0], s[0]), FMUL(s[1], s[1])), FMUL(s[2], s[2])));
                const float ci = FDIV(FADD(FADD(FMUL(nI[0], s[0]), FMUL(nI[1], s[1])), FMUL(nI[2], s[2])), FMUL(ni, d));
                const float cj = FDIV(FADD(FADD(FMUL(-nJ[0], s[0]), FMUL(-nJ[1], s[1])), FMUL(-nJ[2], s[2])), FMUL(nj, d));
                float v = FDIV(FMUL(FMUL(ci, cj), sub2), FMUL(FMUL(c_PIF, d), d));
                if (v < 0.0f) v = 0.0f;
                T = FADD(T, v);
#pragma unroll
                for (int c = 0; c < 3; ++c) TV[c] = FADD(TV[c], FMUL(v, FDIV(s[c], d)));
            }
            tot[j] = T;
#pragma unroll
            for (int c = 0; c < 3; ++c) totv[j][c] = TV[c];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            float ef = 0.0f, ev[3] = {0.0f, 0.0f, 0.0f};
            for (int j = 0; j != SUBF; j++) {
                ef = FADD(ef, FMUL(FDIV(sub1, aI), tot[j]));
#pragma unroll
                for (int c = 0; c < 3; ++c) ev[c] = FADD(ev[c], FMUL(sub1, totv[j][c]));
            }
            vf[e] = ef;
#pragma unroll
            for (int c = 0; c < 3; ++c) dir[3 * e + c] = ev[c];
        }
    }
}

// ------------------------------------------------------------------ launchers
struct VfBuffers {
    VfGeom g;
};

int vf_init(const VfGeom& g, cudaStream_t st) {
    k_vf_init<<<(g.nf + 127) / 128, 128, 0, st>>>(g);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}
int vf_count(const VfGeom& g, int* count, cudaStream_t st) {
    k_vf_count<<<g.nf, 256, 0, st>>>(g, count);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}
int vf_fill(const VfGeom& g, const long long* ptr, int* idx, float* vf, float* dir, cudaStream_t st) {
    k_vf_fill<<<g.nf, 256, 0, st>>>(g, ptr, idx, vf, dir);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}
int vf_hidden(const VfGeom& g, const long long* ptr, const int* idx, uint8_t* keep, cudaStream_t st) {
    k_vf_hidden<<<g.nf, 256, 0, st>>>(g, ptr, idx, keep);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}
int vf_refine(const VfGeom& g, const long long* ptr, const int* idx, float* vf, float* dir, cudaStream_t st) {
    k_vf_refine<<<g.nf, 128, 0, st>>>(g, ptr, idx, vf, dir);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // namespace atpm
