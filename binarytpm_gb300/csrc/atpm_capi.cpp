// Host runtime of libatpm: the C ABI of include/atpm.h.
//
// It plays the part of the reference Thermal driver's single_model
// (3905/Thermal/NominalPole/main.cpp:2417-2590) for a smooth shape: one solve
// handle holds the shape, its view-factor lists and the whole thermal state
// resident in device memory; the per-revolution work is one captured CUDA
// graph (self-heating gather, conduction sweep, convergence, advance) that is
// replayed in chunks with a single host synchronisation per chunk.
//
// Scalars that the reference computes in float are computed here in float in
// the same operand order (this file is built with -ffp-contract=off).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/atpm.h"
#include "atpm_host.h"
#include "atpm_internal.h"

using namespace atpm;

namespace {

thread_local std::string g_err;

atpm_status fail(atpm_status s, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
atpm_status fail(atpm_status s, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return s;
}

#define CK(call)                                                                      \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return fail(ATPM_E_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                        __FILE__, __LINE__);                                          \
    } while (0)

const double kPI = 4.0 * std::atan(1.0);   // main.cpp:12
const double kAU = 149.6e6;                // main.cpp:13
const float kSIGMA = 5.67e-8f;             // main.cpp:15

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

namespace {

atpm_status ensure_tables(atpm_context* c) {
    std::lock_guard<std::mutex> lk(c->mu);
    if (c->tables) return ATPM_OK;
    char err[256];
    CK(cudaSetDevice(c->device));
    if (build_pow_table(4, &c->p4, err, sizeof err)) return fail(ATPM_E_CUDA, "%s", err);
    if (build_pow_table(3, &c->p3, err, sizeof err)) return fail(ATPM_E_CUDA, "%s", err);
    c->tables = true;
    return ATPM_OK;
}

// x^0.25 exceptions (about 1 s of host powf calls): only REFERENCE solves
// that initialise temperatures or run at TI 0 need them
atpm_status ensure_qroot_table(atpm_context* c) {
    std::lock_guard<std::mutex> lk(c->mu);
    if (c->pq.slots_dev) return ATPM_OK;
    char err[256];
    CK(cudaSetDevice(c->device));
    if (build_pow_table(-4, &c->pq, err, sizeof err)) return fail(ATPM_E_CUDA, "%s", err);
    return ATPM_OK;
}

// pole transformation matrix, heliocentric body centre and rotation table of
// the reference's asteroidgeometry (main.cpp:894-958), with this host's libm
// (rotation angle 2 pi step revs / NTAU: revs = 1 for a synchronous body,
// each body's own number of turns per model period for a non-synchronous
// binary, 175706/Run-04/thermal.cpp:1347, 1365)
void geometry_tables(const atpm_params& P, double* tm9, double* car, std::vector<double>& rot, int revs = 1) {
    const double r0 = P.pole[0], r1 = P.pole[1];
    const double gamma = std::acos(std::cos(r0) * std::sin(std::fabs(r1)));
    double tm[3][3];
    tm[0][0] = std::sin(r0) / std::sin(gamma);
    tm[0][1] = -1.0 * std::cos(r0) * std::cos(r0) * std::sin(r1) * std::cos(r1) / std::sin(gamma);
    tm[0][2] = std::cos(r0) * std::cos(r1);
    tm[1][0] = 0.0;
    tm[1][1] = ((std::sin(r0) * std::sin(r0)) + (std::cos(r0) * std::cos(r0) * std::cos(r1) * std::cos(r1))) /
               std::sin(gamma);
    tm[1][2] = std::cos(r0) * std::sin(r1);
    tm[2][0] = -1.0 * std::cos(r0) * std::cos(r1) / std::sin(gamma);
    tm[2][1] = -1.0 * std::sin(r0) * std::cos(r0) * std::sin(r1) / std::sin(gamma);
    tm[2][2] = std::sin(r0);
    for (int i = 0; i < 9; ++i) tm9[i] = tm[i / 3][i % 3];
    car[0] = kAU * P.polar[0] * std::cos(P.polar[1]) * std::cos(P.polar[2]);
    car[1] = kAU * P.polar[0] * std::cos(P.polar[1]) * std::sin(P.polar[2]);
    car[2] = kAU * P.polar[0] * std::sin(P.polar[1]);
    const int ntau = P.ntau;
    rot.assign(2 * (size_t)ntau, 0.0);
    for (int step = 0; step < ntau; ++step) {
        const double ang = 2.0 * kPI * step * revs / ntau;
        rot[2 * step] = std::cos(ang);
        rot[2 * step + 1] = std::sin(ang);
    }
}

PowTab view(const HostPowTab& h) {
    PowTab t;
    t.slots = h.slots_dev;
    t.log2slots = h.log2slots;
    t.lo_bits = h.lo_bits;
    t.hi_bits = h.hi_bits;
    return t;
}

struct Layout {
    size_t off[24];
    size_t total;
};

enum {
    B_VERT, B_FAC, B_DPTR, B_DIDX, B_DVF, B_SHADOW, B_COS, B_EFM, B_E, B_S0, B_S1, B_TEMP, B_Q, B_W,
    B_CONV, B_HOT, B_COUNTS, B_STATUS, B_CTL, B_DIAG, B_ACT, B_MEAN, B_RBACT, B_N
};

Layout layout(int nv, int nf, int nnz, const atpm_params& P) {
    const size_t rs = (P.precision == ATPM_FP64) ? 8 : 4;
    const size_t nt = (size_t)nf * P.ntau;
    size_t sz[B_N];
    sz[B_VERT] = (size_t)nv * 3 * 8;
    sz[B_FAC] = (size_t)nf * 3 * 4;
    sz[B_DPTR] = (size_t)(nf + 1) * 4;
    sz[B_DIDX] = (size_t)std::max(nnz, 1) * 4;
    sz[B_DVF] = (size_t)std::max(nnz, 1) * 4;
    sz[B_SHADOW] = nt;
    sz[B_COS] = nt * rs;
    sz[B_EFM] = nt * rs;
    sz[B_E] = nt * rs;
    sz[B_S0] = nt * rs;
    sz[B_S1] = nt * rs;
    sz[B_TEMP] = (size_t)(P.nx + 1) * nf * rs;
    sz[B_Q] = nt * rs;
    sz[B_W] = nt * rs;
    sz[B_CONV] = nf;
    sz[B_HOT] = nf;
    sz[B_COUNTS] = (size_t)std::max(P.revcap, 1) * 4;
    sz[B_STATUS] = 4;
    sz[B_CTL] = sizeof(Ctl);
    sz[B_DIAG] = 4 * 8;
    sz[B_ACT] = ((size_t)2 * nf + 5) * 4;
    sz[B_MEAN] = (size_t)nf * rs;
    sz[B_RBACT] = (size_t)(nf + 127) / 128;
    Layout L;
    size_t o = 0;
    for (int i = 0; i < B_N; ++i) {
        L.off[i] = o;
        o += align256(sz[i]);
    }
    L.total = o;
    return L;
}

atpm_status check_shape(const atpm_shape* sh, const atpm_params* P) {
    if (!sh || !P) return fail(ATPM_E_INVALID, "null shape or params");
    if (sh->nv < 3 || sh->nf < 1 || !sh->vertices || !sh->facets || !sh->dep_ptr)
        return fail(ATPM_E_INVALID, "shape needs nv>=3, nf>=1, vertices, facets, dep_ptr");
    if (P->ntau < 1 || P->nx < 2 || P->revcap < 1)
        return fail(ATPM_E_INVALID, "ntau>=1, nx>=2, revcap>=1 required");
    if (P->precision < 0 || P->precision > 2) return fail(ATPM_E_INVALID, "unknown precision %d", P->precision);
    if (!conduction_nx_supported(P->nx))
        return fail(ATPM_E_UNSUPPORTED, "nx=%d not built (supported: 8,12,16,24,32,40,48,56,64)", P->nx);
    if (sh->dep_ptr[0] != 0) return fail(ATPM_E_INVALID, "dep_ptr[0] must be 0");
    for (int f = 0; f < sh->nf; ++f)
        if (sh->dep_ptr[f + 1] < sh->dep_ptr[f]) return fail(ATPM_E_INVALID, "dep_ptr not monotone at %d", f);
    const int nnz = sh->dep_ptr[sh->nf];
    if (nnz > 0 && (!sh->dep_idx || !sh->dep_vf)) return fail(ATPM_E_INVALID, "dep_idx/dep_vf missing");
    for (int k = 0; k < nnz; ++k)
        if (sh->dep_idx[k] < 0 || sh->dep_idx[k] >= sh->nf)
            return fail(ATPM_E_INVALID, "dep_idx[%d]=%d out of range", k, sh->dep_idx[k]);
    for (int i = 0; i < 3 * sh->nf; ++i)
        if (sh->facets[i] < 0 || sh->facets[i] >= sh->nv)
            return fail(ATPM_E_INVALID, "facet vertex index %d out of range", sh->facets[i]);
    for (int i = 0; i < 3 * sh->nv; ++i)
        if (!std::isfinite(sh->vertices[i])) return fail(ATPM_E_NONFINITE, "vertex coordinate %d is not finite", i);
    for (int k = 0; k < nnz; ++k)
        if (!std::isfinite(sh->dep_vf[k])) return fail(ATPM_E_NONFINITE, "view factor %d is not finite", k);
    const double scal[] = {P->polar[0], P->polar[1], P->polar[2], P->pole[0], P->pole[1], P->rotation_period_s,
                           P->albedo, P->emissivity, P->tacc, P->scattering_accuracy};
    for (double x : scal)
        if (!std::isfinite(x)) return fail(ATPM_E_INVALID, "a parameter is not finite");
    if (!(P->rotation_period_s > 0.0f) || !(P->tacc > 0.0f))
        return fail(ATPM_E_INVALID, "rotation period and TACC must be positive");
    return ATPM_OK;
}

// Scalars of the reference in its float operand order (main.cpp:1477-1541).
int newton_cap();

void set_scalars(atpm_solve* s, float ti) {
    const atpm_params& P = s->P;
    DevSolve& d = s->ds;
    const float PIf = (float)kPI;
    const float DZ = 8.0f / P.nx;
    // per-body rotations per model period (non-synchronous binaries,
    // 175706/Run-04/thermal.cpp:1925, 1966-1967); 1 for a synchronous body
    const float nr = (float)s->revs_p, nr2 = (float)s->revs_s;
    const float DTAU = 2.0f * PIf * nr / (float)P.ntau;
    const float DTAU2 = 2.0f * PIf * nr2 / (float)P.ntau;
    d.ti = ti;
    d.r = DTAU / (DZ * DZ);
    d.m1 = ti * std::sqrt(2.0f * PIf * nr / P.rotation_period_s) / DZ;
    d.r2 = DTAU2 / (DZ * DZ);
    d.m1_2 = ti * std::sqrt(2.0f * PIf * nr2 / P.rotation_period_s) / DZ;
    d.fsplit = s->sec_facet >= 0 ? s->sec_facet : s->nf;
    d.es_w = s->ir_abs * P.emissivity * kSIGMA;
    d.es = P.emissivity * kSIGMA;
    d.es4 = 4.0f * P.emissivity * kSIGMA;
    d.oma = 1.0f - P.albedo;
    d.tacc = P.tacc;
    const double t10 = (double)P.tacc / 10.0;
    float c = (float)t10;
    if ((double)c < t10) c = std::nextafter(c, 1e30f);
    d.tacc10 = c;  // DT >= c  <=>  (double)DT >= TACC/10.0 for every float DT
    d.alb = P.albedo;
    d.solar = (float)(1367.0 / (P.polar[0] * P.polar[0]));
    d.sacc = P.scattering_accuracy;
    // FP64 state: the same expressions with double operands
    const double PId = (double)PIf;
    const double DZd = 8.0 / P.nx;
    const double DTAUd = 2.0 * PId * (double)nr / P.ntau;
    const double DTAU2d = 2.0 * PId * (double)nr2 / P.ntau;
    d.ti_d = ti;
    d.r_d = DTAUd / (DZd * DZd);
    d.m1_d = (double)ti * std::sqrt(2.0 * PId * (double)nr / (double)P.rotation_period_s) / DZd;
    d.r2_d = DTAU2d / (DZd * DZd);
    d.m1_2_d = (double)ti * std::sqrt(2.0 * PId * (double)nr2 / (double)P.rotation_period_s) / DZd;
    d.es_w_d = (double)s->ir_abs * (double)P.emissivity * (double)kSIGMA;
    d.es_d = (double)P.emissivity * (double)kSIGMA;
    d.es4_d = 4.0 * (double)P.emissivity * (double)kSIGMA;
    d.oma_d = 1.0 - (double)P.albedo;
    d.tacc_d = (double)P.tacc;
    d.tacc10_d = t10;
    d.alb_d = (double)P.albedo;
    d.solar_d = (double)d.solar;
    d.sacc_d = (double)P.scattering_accuracy;
    d.newton_cap = newton_cap();
}

atpm_status upload_table(atpm_solve* s) {
    CK(cudaMemcpyAsync(s->ds_dev, &s->ds, sizeof(DevSolve), cudaMemcpyHostToDevice, s->st));
    return ATPM_OK;
}

void build_maps(int nf, int ntau, int solve, std::vector<int4>& w, std::vector<int2>& fm) {
    for (int f0 = 0; f0 < nf; f0 += 32)
        for (int s0 = 0; s0 < ntau; s0 += 32) w.push_back(make_int4(solve, f0, s0, 0));
    for (int f0 = 0; f0 < nf; f0 += 128) fm.push_back(make_int2(solve, f0));
}

// FAST conduction variant: ATPM_COND_VARIANT in {1,2,3} (minimum resident
// blocks per SM given to the register allocator; 3 was the fastest of them
// on GB300 for NX = 56: 2.09 -> 1.52 ms per batched revolution) or 4 (the
// facet-range sweep as pairs of facets on the packed FP32 instructions, the
// list and warp forms as in 3: 18.1 -> 16.8 ms per 6-revolution step of the
// 8-inertia binary batch).  All four give bit-identical results.  Default 4.
int cond_variant() {
    const char* e = std::getenv("ATPM_COND_VARIANT");
    if (e && e[0] >= '1' && e[0] <= '4' && e[1] == 0) return e[0] - '0';
    return 4;
}

// Newton iteration cap of the surface boundary condition (ATPM_NEWTON_CAP,
// 1..200, default 200); a solve that reaches it stops with ATPM_E_ITERATION.
// Read when a solve is created and when its thermal inertia is set.
int newton_cap() {
    const char* e = std::getenv("ATPM_NEWTON_CAP");
    const int v = e ? std::atoi(e) : 0;
    return v >= 1 && v <= 200 ? v : 200;
}

bool autotune_enabled() {
    const char* e = std::getenv("ATPM_AUTOTUNE");
    return !(e && e[0] == '0');
}

bool shadow_cull_enabled() {
    const char* e = std::getenv("ATPM_SHADOW_CULL");
    return !(e && e[0] == '0');
}

bool warp_tail_enabled() {
    const char* e = std::getenv("ATPM_WARP_TAIL");
    return !(e && e[0] == '0');
}

// active facets per SM up to which a revolution runs warp per facet
// (ATPM_WARP_TAIL_PER_SM, 1..64; both forms give identical results)
int warp_tail_per_sm() {
    const char* e = std::getenv("ATPM_WARP_TAIL_PER_SM");
    const int v = e ? std::atoi(e) : 0;
    return v >= 1 && v <= 64 ? v : 12;
}

// Device memory of solves and batches comes from the device's
// stream-ordered pool (cudaMallocAsync), which the context sets to keep
// released memory for reuse: a job that creates and destroys solves then
// allocates from what the previous job released instead of mapping new
// pages.  The stream is synchronised, so the memory is usable from any
// stream when this returns.
cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t st) {
    cudaError_t e = cudaMallocAsync(p, bytes, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

// Fewest list entries a (128-row, 64-column) cell needs to become a
// tensor-core tile (ATPM_TC_MIN_ENTRIES, 1..8192, default 32).  The entries of
// sparser cells form the per-row remainder, summed in FP32 against W32 by
// k_spmm_rem after the tiles' product.  On the 21,760-facet binary the 4,173
// cells with at least 32 entries hold 99.0 % of the 5.8 M entries and the
// other 8,784 cells (68 % of all cells, mostly facets of one body seeing
// each other across its surface relief) 1.0 %; per 8-solve revolution the
// product took 1.76 / 1.71 / 1.73 / 1.82 ms at thresholds 16 / 32 / 64 / 128
// against 2.12 ms with every cell a tile.  The split changes rounding (the
// remainder is FP32 instead of BF16 hi/lo), not the result beyond it.
int tc_min_entries() {
    const char* e = std::getenv("ATPM_TC_MIN_ENTRIES");
    const int v = e ? std::atoi(e) : 0;
    return v >= 1 && v <= 128 * 64 ? v : 32;
}

bool tc_enabled() {
    const char* e = std::getenv("ATPM_TC");
    return !(e && e[0] == '0');
}

// step chunking of the tensor-core product: equal chunks of N <= tc_max_chunk()
// steps, N a multiple of 16 (720 steps -> 5 chunks of 144)
void tc_chunks(int ntau, int* n, int* nch) {
    const int cap = tc_max_chunk();
    const int c = (ntau + cap - 1) / cap;
    int nn = (ntau + c - 1) / c;
    nn = (nn + 15) / 16 * 16;
    *n = nn;
    *nch = c;
}

// work items of the tensor-core product {solve, row block, step chunk, 0}
// for the solves of a batch that have tiles, solve by solve and row block by
// row block: one solve's W tiles stay in L2 while its items run, and
// neighbouring row blocks read largely the same W column blocks.  (Putting
// the same row block of all solves together, to share V tiles in L2, made
// the batch's W working set exceed L2: 25 % slower.)
void build_tc_items(atpm_solve* const* solves, int n, std::vector<int4>& q) {
    for (int i = 0; i < n; ++i) {
        const atpm_solve* s = solves[i];
        if (!s->tc) continue;
        int N, nch;
        tc_chunks(s->P.ntau, &N, &nch);
        for (int mb = 0; mb < (int)s->tc->rb_tiles.size(); ++mb)
            for (int c = 0; c < nch; ++c) q.push_back(make_int4(i, mb, c, 0));
    }
}

// device layout of a batch's tensor-core map: the nq items, then room for the
// per-launch list of active items (nq), then the two work counters
size_t tc_map_entries(size_t nq) { return nq ? 2 * nq + 1 : 0; }
void tc_map_extend(std::vector<int4>& q) {
    const size_t nq = q.size();
    if (nq) q.resize(tc_map_entries(nq), make_int4(0, 0, 0, 0));
}
void set_tc_map(Batch& b, const int4* dev_map, size_t entries) {
    b.qmap = dev_map;
    b.nq = entries ? (int)((entries - 1) / 2) : 0;
    int4* w = const_cast<int4*>(dev_map);
    b.tc_list = b.nq ? w + b.nq : nullptr;
    b.tc_work = b.nq ? reinterpret_cast<int*>(w + 2 * (size_t)b.nq) : nullptr;
}

// block-sparse BF16 tiles of the view-factor matrix (128 x 64, swizzled)
atpm_status build_tc(atpm_solve* s, const atpm_shape* sh) {
    // tile structure: which 64-facet column blocks each 128-facet row block
    // touches, the largest view factor and K-slice mask of each tile (one
    // device pass over the uploaded lists, k_tc_cells); the tile tables are
    // laid out on the host from those cells, the BF16 values filled on the
    // device (k_tc_fill)
    const int nf = s->nf, ntau = s->P.ntau;
    const int nmb = (nf + 127) / 128, nkb = (nf + 63) / 64;
    int N, nch;
    tc_chunks(ntau, &N, &nch);
    const size_t ncell = (size_t)nmb * nkb;
    if (nkb >= (1 << 24)) return fail(ATPM_E_UNSUPPORTED, "tensor-core tiles: %d facets exceed the column-block index", nf);
    std::vector<float> vm(ncell, -1.0f);
    std::vector<uint8_t> km(ncell, 0);  // which 16-wide K slices of the tile hold an entry
    std::vector<unsigned> need(ncell, 0);  // the tile needs its residual for some row's flux
    const unsigned min_entries = (unsigned)tc_min_entries();
    {
        std::vector<unsigned> cmax(ncell), cmask(ncell), cnt(ncell);
        unsigned* dc = nullptr;
        CK(cudaMallocAsync((void**)&dc, ncell * 4 * sizeof(unsigned), s->st));
        cudaError_t e = cudaMemsetAsync(dc, 0, ncell * 4 * sizeof(unsigned), s->st);
        if (e == cudaSuccess && launch_tc_cells(s->ds, nkb, dc, dc + ncell, dc + 3 * ncell, s->st))
            e = cudaGetLastError();
        if (e == cudaSuccess && launch_tc_rowneed(s->ds, nkb, dc + 2 * ncell, s->st) == 2) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(cmax.data(), dc, ncell * sizeof(unsigned), cudaMemcpyDeviceToHost, s->st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(cmask.data(), dc + ncell, ncell * sizeof(unsigned), cudaMemcpyDeviceToHost, s->st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(need.data(), dc + 2 * ncell, ncell * sizeof(unsigned), cudaMemcpyDeviceToHost, s->st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(cnt.data(), dc + 3 * ncell, ncell * sizeof(unsigned), cudaMemcpyDeviceToHost, s->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
        cudaFreeAsync(dc, s->st);
        if (e != cudaSuccess) return fail(ATPM_E_CUDA, "tile structure: %s", cudaGetErrorString(e));
        for (size_t c = 0; c < ncell; ++c) {
            if (!cmax[c] || cnt[c] < min_entries) continue;  // empty, or left to the remainder
            uint32_t bits = cmax[c] - 1u;
            float v;
            std::memcpy(&v, &bits, 4);
            vm[c] = v;
            km[c] = (uint8_t)cmask[c];
        }
    }
    std::vector<int> tptr(nmb + 1, 0), tcol, slot(ncell, -1), lo_of;
    int nlo = 0;
    for (int mb = 0; mb < nmb; ++mb) {
        for (int kb = 0; kb < nkb; ++kb) {
            const float v = vm[(size_t)mb * nkb + kb];
            if (v < 0.0f) continue;
            slot[(size_t)mb * nkb + kb] = (int)tcol.size();
            // column block in the low 24 bits, K-slice mask in bits 24-27
            tcol.push_back(kb | ((int)km[(size_t)mb * nkb + kb] << 24));
            // residual tile V - bf16(V) where the tile holds a view factor >= 1e-4
            // or carries a noticeable share of some row's mass (k_tc_rowneed)
            lo_of.push_back(v >= 1e-4f || need[(size_t)mb * nkb + kb] ? nlo++ : -1);
        }
        tptr[mb + 1] = (int)tcol.size();
    }
    const size_t ntiles = tcol.size();
    const size_t tile_el = 128 * 64;
    // W32 row stride: the steps rounded up to the remainder kernel's 32-step
    // chunks (every lane's load stays inside its row; the pad stays zero)
    const int w32_ld = (ntau + 31) & ~31;
    if (lo_of.empty()) lo_of.push_back(-1);
    const size_t b_tiles = align256(std::max<size_t>(ntiles, 1) * tile_el * 2);
    const size_t b_ptr = align256((nmb + 1) * 4), b_col = align256(std::max<size_t>(ntiles, 1) * 4);
    const size_t b_w = align256((size_t)nkb * nch * N * 64 * 2 * 2);
    const size_t b_lo = align256((size_t)std::max(nlo, 1) * tile_el * 2), b_loi = align256(lo_of.size() * 4);
    const size_t b_slot = align256(ncell * 4);
    auto* tc = new TcShared();
    s->tc = tc;
    tc->bytes = b_tiles + b_ptr + b_col + b_lo + b_loi + b_slot;
    tc->tiles = ntiles;
    tc->rb_tiles.resize(nmb);
    for (int mb = 0; mb < nmb; ++mb) tc->rb_tiles[mb] = tptr[mb + 1] - tptr[mb];
    CK(pool_alloc(&tc->mem, tc->bytes, s->st));
    CK(pool_alloc(&s->wb_mem, b_w, s->st));
    s->wb_bytes = b_w;
    char* m = static_cast<char*>(tc->mem);
    char* p_lo = m + b_tiles + b_ptr + b_col;
    int* d_slot = reinterpret_cast<int*>(p_lo + b_lo + b_loi);
    CK(cudaMemsetAsync(m, 0, b_tiles, s->st));
    CK(cudaMemcpyAsync(m + b_tiles, tptr.data(), (nmb + 1) * 4, cudaMemcpyHostToDevice, s->st));
    if (ntiles) CK(cudaMemcpyAsync(m + b_tiles + b_ptr, tcol.data(), ntiles * 4, cudaMemcpyHostToDevice, s->st));
    CK(cudaMemsetAsync(s->wb_mem, 0, b_w, s->st));
    CK(cudaMemsetAsync(p_lo, 0, b_lo, s->st));
    CK(cudaMemcpyAsync(p_lo + b_lo, lo_of.data(), lo_of.size() * 4, cudaMemcpyHostToDevice, s->st));
    CK(cudaMemcpyAsync(d_slot, slot.data(), ncell * 4, cudaMemcpyHostToDevice, s->st));
    // the sparse remainder: entries of cells without a tile, per row in list
    // order (counted and gathered on the device from the uploaded lists)
    size_t rnnz = 0;
    const size_t b_rptr = align256((size_t)(nf + 1) * 4);
    {
        int* cnt_d = nullptr;
        CK(cudaMallocAsync((void**)&cnt_d, (size_t)nf * 4, s->st));
        std::vector<int> rptr(nf + 1, 0);
        int rc = launch_rem_count(s->ds, nkb, d_slot, cnt_d, s->st);
        cudaError_t e = rc ? cudaGetLastError() : cudaMemcpyAsync(rptr.data() + 1, cnt_d, (size_t)nf * 4,
                                                                   cudaMemcpyDeviceToHost, s->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
        cudaFreeAsync(cnt_d, s->st);
        if (e != cudaSuccess) return fail(ATPM_E_CUDA, "remainder count: %s", cudaGetErrorString(e));
        for (int f = 0; f < nf; ++f) rptr[f + 1] += rptr[f];
        rnnz = (size_t)rptr[nf];
        if (rnnz) {
            const size_t b_ridx = align256(rnnz * 4), b_rrow = align256(rnnz);
            CK(pool_alloc(&tc->rem_mem, b_rptr + 2 * b_ridx + b_rrow, s->st));
            char* p = static_cast<char*>(tc->rem_mem);
            CK(cudaMemcpyAsync(p, rptr.data(), (size_t)(nf + 1) * 4, cudaMemcpyHostToDevice, s->st));
            if (launch_rem_fill(s->ds, nkb, d_slot, reinterpret_cast<int*>(p), reinterpret_cast<int*>(p + b_rptr),
                                reinterpret_cast<float*>(p + b_rptr + b_ridx),
                                reinterpret_cast<uint8_t*>(p + b_rptr + 2 * b_ridx), s->st))
                return fail(ATPM_E_CUDA, "remainder fill: %s", cudaGetErrorString(cudaGetLastError()));
            s->ds.rem_ptr = reinterpret_cast<const int*>(p);
            s->ds.rem_idx = reinterpret_cast<const int*>(p + b_rptr);
            s->ds.rem_vf = reinterpret_cast<const float*>(p + b_rptr + b_ridx);
            s->ds.rem_row = reinterpret_cast<const uint8_t*>(p + b_rptr + 2 * b_ridx);
            s->w32_bytes = align256((size_t)nf * w32_ld * 4);
            CK(pool_alloc(&s->w32_mem, s->w32_bytes, s->st));
            CK(cudaMemsetAsync(s->w32_mem, 0, s->w32_bytes, s->st));
            CK(cudaStreamSynchronize(s->st));  // rptr must outlive its copy
        }
    }
    tc->remainder = rnnz;
    if (launch_tc_fill(s->ds, nkb, d_slot, reinterpret_cast<const int*>(p_lo + b_lo), m, p_lo, s->st))
        return fail(ATPM_E_CUDA, "tile fill launch: %s", cudaGetErrorString(cudaGetLastError()));
    CK(cudaStreamSynchronize(s->st));  // the host tables must outlive their copies
    DevSolve& d = s->ds;
    d.tc_tiles = m;
    d.tc_ptr = reinterpret_cast<const int*>(m + b_tiles);
    d.tc_col = reinterpret_cast<const int*>(m + b_tiles + b_ptr);
    d.Wb = s->wb_mem;
    d.tc_lo_tiles = p_lo;
    d.tc_lo = reinterpret_cast<const int*>(p_lo + b_lo);
    d.tc_n = N;
    d.tc_nchunks = nch;
    d.tc_nmb = nmb;
    d.tc_nkb = nkb;
    d.W32 = static_cast<float*>(s->w32_mem);
    d.w32_ld = w32_ld;
    std::vector<int4> q;
    atpm_solve* one[1] = {s};
    build_tc_items(one, 1, q);
    tc_map_extend(q);
    CK(pool_alloc(reinterpret_cast<void**>(&s->qmap), q.size() * sizeof(int4), s->st));
    CK(cudaMemcpy(s->qmap, q.data(), q.size() * sizeof(int4), cudaMemcpyHostToDevice));
    s->nq = (int)q.size();  // map entries (items, list, counters)
    return ATPM_OK;
}

Batch make_batch(atpm_context* ctx, const DevSolve* tab, int n, const int4* wm, int nw, const int2* fm,
                 int nfb, int mode, int nx) {
    Batch b;
    b.tab = tab;
    b.n = n;
    b.wmap = wm;
    b.nw = nw;
    b.fmap = fm;
    b.nfb = nfb;
    b.mode = mode;
    b.nx = nx;
    b.p4 = view(ctx->p4);
    b.p3 = view(ctx->p3);
    b.pq = view(ctx->pq);
    b.qmap = nullptr;
    b.nq = 0;
    b.tc_list = nullptr;
    b.tc_work = nullptr;
    b.tc_nmax = 0;
    b.cond_variant = cond_variant();
    b.tc_stages = 0;
    b.warp_tail = warp_tail_enabled() ? 1 : 0;
    // active facets of the whole batch up to which a revolution runs warp per
    // facet: about a dozen warps per SM, where one warp per facet still beats
    // the thread-per-facet sweep's latency-bound last warps
    b.tail_limit = warp_tail_per_sm() * ctx->sm_count;
    b.sms = ctx->sm_count;
    b.rem_nmb = 0;
    b.rem_ntau = 0;
    b.side = b.ev_fork = b.ev_join = nullptr;
    return b;
}

// the remainder kernel's grid: the largest row-block count and step count of
// the solves that have a sparse remainder
void set_remainder_grid(Batch& b, atpm_solve* const* solves, int n) {
    for (int i = 0; i < n; ++i) {
        const DevSolve& d = solves[i]->ds;
        if (!d.rem_ptr) continue;
        b.rem_nmb = std::max(b.rem_nmb, (d.nf + 127) / 128);
        b.rem_ntau = std::max(b.rem_ntau, d.ntau);
    }
    // the leader's side stream and events, so the remainder can run beside
    // the product (without them it runs after it: same sums)
    atpm_solve* s0 = solves[0];
    if (b.rem_nmb > 0 && !s0->side_st) {
        if (cudaStreamCreateWithFlags(&s0->side_st, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&s0->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&s0->ev_join, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            if (s0->side_st) cudaStreamDestroy(s0->side_st);
            if (s0->ev_fork) cudaEventDestroy(s0->ev_fork);
            if (s0->ev_join) cudaEventDestroy(s0->ev_join);
            s0->side_st = nullptr;
            s0->ev_fork = s0->ev_join = nullptr;
        }
    }
    if (b.rem_nmb > 0 && s0->side_st) {
        b.side = s0->side_st;
        b.ev_fork = s0->ev_fork;
        b.ev_join = s0->ev_join;
    }
}


// device table + tile maps for a set of solves (single solves reuse theirs)
atpm_status make_batch_for(atpm_solve* const* solves, int n, Batch* out, void** tmp) {
    atpm_solve* s0 = solves[0];
    *tmp = nullptr;
    if (n == 1) {
        *out = make_batch(s0->ctx, s0->ds_dev, 1, s0->wmap, s0->nw, s0->fmap, s0->nfb, s0->P.precision, s0->P.nx);
        set_tc_map(*out, s0->qmap, (size_t)s0->nq);
        out->tc_nmax = s0->ds.tc_n;
        set_remainder_grid(*out, solves, n);
        return ATPM_OK;
    }
    std::vector<DevSolve> tab(n);
    std::vector<int4> wm, qm;
    std::vector<int2> fm;
    int nmax = 0;
    for (int i = 0; i < n; ++i) {
        tab[i] = solves[i]->ds;
        std::vector<int4> w1;
        build_maps(solves[i]->nf, solves[i]->P.ntau, i, w1, fm);
        if (solves[i]->nnz > 0) wm.insert(wm.end(), w1.begin(), w1.end());
        if (solves[i]->nq > 0) nmax = std::max(nmax, solves[i]->ds.tc_n);
    }
    build_tc_items(solves, n, qm);
    const size_t bt = align256(n * sizeof(DevSolve)), bw = align256(std::max<size_t>(wm.size(), 1) * sizeof(int4));
    const size_t bf = align256(fm.size() * sizeof(int2));
    tc_map_extend(qm);
    const size_t bq = align256(std::max<size_t>(qm.size(), 1) * sizeof(int4));
    CK(pool_alloc(tmp, bt + bw + bf + bq, s0->st));
    char* t = static_cast<char*>(*tmp);
    CK(cudaMemcpy(t, tab.data(), n * sizeof(DevSolve), cudaMemcpyHostToDevice));
    if (!wm.empty()) CK(cudaMemcpy(t + bt, wm.data(), wm.size() * sizeof(int4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(t + bt + bw, fm.data(), fm.size() * sizeof(int2), cudaMemcpyHostToDevice));
    if (!qm.empty()) CK(cudaMemcpy(t + bt + bw + bf, qm.data(), qm.size() * sizeof(int4), cudaMemcpyHostToDevice));
    *out = make_batch(s0->ctx, reinterpret_cast<DevSolve*>(t), n, reinterpret_cast<int4*>(t + bt), (int)wm.size(),
                      reinterpret_cast<int2*>(t + bt + bw), (int)fm.size(), s0->P.precision, s0->P.nx);
    set_tc_map(*out, reinterpret_cast<int4*>(t + bt + bw + bf), qm.size());
    out->tc_nmax = nmax;
    set_remainder_grid(*out, solves, n);
    return ATPM_OK;
}

atpm_status capture_graph(atpm_solve* s, const Batch& b, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
    int rc = launch_revolution(b, s->st);
    cudaError_t e = cudaStreamEndCapture(s->st, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return fail(ATPM_E_CUDA, "revolution launch failed during capture (rc=%d)", rc);
    }
    if (e != cudaSuccess) return fail(ATPM_E_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(ATPM_E_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    return ATPM_OK;
}

// Autotuner for FAST batches.  Its knobs change launch configurations only,
// never results: the conduction variant (k_conduction<FAST, NX, 1|2|3>: one
// source, three register budgets; 4: the paired-facet sweep) and the
// tensor-core pipeline depth.  The first time a kind of batch (precision,
// NX, step chunk, size class, number of groups) runs, its first kTuneRevs
// revolutions -- real revolutions of the solves, each with one candidate --
// are launched for every group together, each group on its own stream as
// the revolution loop launches them, and each revolution is timed whole,
// from a common start to the end of the last group.  A variant that leaves
// issue slots to the other group's product therefore shows up as the faster
// revolution, which the sweep's own duration does not show.  The fastest
// candidates are kept in the context for every later batch of that kind.
uint64_t tune_key(const Batch& b, int groups) {
    int cls = 0;
    while ((1 << cls) < b.nfb && cls < 40) ++cls;  // facet blocks, power-of-two class
    return (uint64_t)b.mode | ((uint64_t)b.nx << 4) | ((uint64_t)b.tc_nmax << 12) | ((uint64_t)cls << 24) |
           ((uint64_t)(b.nq > 0) << 32) | ((uint64_t)(groups > 1) << 33);
}

// revolutions the autotuner times: conduction variants 1-4 at the deepest
// tensor-core pipeline, then variant 4 one stage shallower
constexpr int kTuneRevs = 5;

bool tune_log() {
    const char* e = std::getenv("ATPM_TUNE_LOG");
    return e && e[0] == '1';
}

atpm_status autotune(const std::vector<atpm_solve*>& leads, std::vector<Batch>& bs, const std::vector<int>& maxcap,
                     std::vector<int>& done, int64_t* launches, int* tuned) {
    atpm_solve* s0 = leads[0];
    atpm_context* c = s0->ctx;
    const int ng = (int)bs.size();
    const uint64_t key = tune_key(bs[0], ng);
    auto apply = [&](int v, int d) {
        for (Batch& b : bs) {
            b.cond_variant = v;
            b.tc_stages = d;
        }
    };
    {
        std::lock_guard<std::mutex> lk(c->mu);
        auto it = c->tune.find(key);
        if (it != c->tune.end()) {
            apply(it->second.cond_variant, it->second.tc_stages);
            return ATPM_OK;
        }
    }
    int mincap = maxcap[0];
    for (int g = 1; g < ng; ++g) mincap = std::min(mincap, maxcap[g]);
    if (mincap < kTuneRevs) {  // too short to time: defaults
        apply(cond_variant(), 0);
        return ATPM_OK;
    }
    const int smax = bs[0].nq > 0 ? tc_max_stages(bs[0].tc_nmax) : 0;
    const int cand_v[kTuneRevs] = {1, 2, 3, 4, 4};
    const int cand_d[kTuneRevs] = {smax, smax, smax, smax, smax > 2 ? smax - 1 : smax};
    // per revolution: start and end on the leader's stream, the end of every other group
    const int nev = kTuneRevs * (1 + ng);
    std::vector<cudaEvent_t> ev(nev, nullptr);
    for (int i = 0; i < nev; ++i) CK(cudaEventCreate(&ev[i]));
    auto ev_start = [&](int r) { return ev[r * (1 + ng)]; };
    auto ev_end = [&](int r, int g) { return ev[r * (1 + ng) + 1 + g]; };  // g = 0: all groups done
    int rc = 0;
    cudaError_t e = cudaSuccess;
    int64_t nlaunch = 0;
    for (int r = 0; r < kTuneRevs && !rc && e == cudaSuccess; ++r) {
        apply(cand_v[r], cand_d[r]);
        e = cudaEventRecord(ev_start(r), s0->st);
        for (int g = 1; g < ng && e == cudaSuccess; ++g) e = cudaStreamWaitEvent(leads[g]->st, ev_start(r), 0);
        for (int g = 0; g < ng && e == cudaSuccess && !rc; ++g) {
            rc |= launch_revolution(bs[g], leads[g]->st);
            nlaunch += kernels_per_revolution(bs[g]);
        }
        for (int g = 1; g < ng && e == cudaSuccess; ++g) {
            e = cudaEventRecord(ev_end(r, g), leads[g]->st);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(s0->st, ev_end(r, g), 0);
        }
        if (e == cudaSuccess) e = cudaEventRecord(ev_end(r, 0), s0->st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s0->st);
    float rv[kTuneRevs] = {};
    for (int r = 0; r < kTuneRevs && e == cudaSuccess && !rc; ++r)
        e = cudaEventElapsedTime(&rv[r], ev_start(r), ev_end(r, 0));
    for (int i = 0; i < nev; ++i) cudaEventDestroy(ev[i]);
    if (rc) return fail(ATPM_E_CUDA, "revolution launch (autotune): %s", cudaGetErrorString(cudaGetLastError()));
    if (e != cudaSuccess) return fail(ATPM_E_CUDA, "autotune: %s", cudaGetErrorString(e));
    // variant 4 unless another revolution was faster; ties keep it
    int best = 3;
    for (int r = 0; r < 3; ++r)
        if (rv[r] < rv[best]) best = r;
    atpm_tune_choice ch;
    ch.cond_variant = cand_v[best];
    ch.tc_stages = (smax > 2 && rv[4] < rv[3]) ? smax - 1 : 0;
    for (int r = 0; r < kTuneRevs; ++r) ch.rev_ms[r] = rv[r];
    if (tune_log())
        std::fprintf(stderr,
                     "atpm autotune: %d group(s), revolution ms v1 %.4f v2 %.4f v3 %.4f v4 %.4f v4/depth-1 %.4f "
                     "-> variant %d depth %d\n",
                     ng, rv[0], rv[1], rv[2], rv[3], rv[4], ch.cond_variant, ch.tc_stages);
    {
        std::lock_guard<std::mutex> lk(c->mu);
        c->tune[key] = ch;
    }
    apply(ch.cond_variant, ch.tc_stages);
    for (int g = 0; g < ng; ++g) done[g] = kTuneRevs;
    *launches += nlaunch;
    *tuned = 1;
    return ATPM_OK;
}

int64_t facet_steps_from_counts(const int32_t* counts, int nrev, int nf, int ntau, bool inst) {
    int64_t fs = 0;
    for (int r = 0; r < nrev; ++r) {
        int active = nf;
        if (!inst && r - 1 > 5) active = nf - counts[r - 1];
        fs += (int64_t)active * ntau;
    }
    return fs;
}

atpm_status check_status(atpm_solve* s, int st) {
    if (st & ST_NONFINITE) return fail(ATPM_E_NONFINITE, "a surface temperature became non-finite");
    if (st & ST_NEWTON_CAP) return fail(ATPM_E_ITERATION, "Newton iteration cap reached");
    if (st & ST_SCATTER_CAP) return fail(ATPM_E_ITERATION, "scattering iteration cap reached");
    if (st & ST_TC_TIMEOUT) return fail(ATPM_E_ITERATION, "tensor-core pipeline wait timed out");
    (void)s;
    return ATPM_OK;
}

}  // namespace

namespace {
template <class R>
atpm_status get_transposed(atpm_solve* s, const void* dev, size_t rows, size_t cols, float* out, double* out64) {
    // dev is [rows][cols]; out is [cols][rows]: transposed (and converted) on
    // the device, one copy into the caller's buffer
    void* host = out ? static_cast<void*>(out) : static_cast<void*>(out64);
    const int ob = out ? 4 : 8;
    void* tmp = nullptr;
    CK(cudaMallocAsync(&tmp, rows * cols * ob, s->st));
    cudaError_t e = cudaSuccess;
    if (launch_transpose(dev, (int)sizeof(R), tmp, ob, rows, cols, s->st)) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, tmp, rows * cols * ob, cudaMemcpyDeviceToHost, s->st);
    cudaFreeAsync(tmp, s->st);
    cudaError_t e2 = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) return fail(ATPM_E_CUDA, "transpose/copy: %s", cudaGetErrorString(e));
    if (e2 != cudaSuccess) return fail(ATPM_E_CUDA, "transpose/copy: %s", cudaGetErrorString(e2));
    return ATPM_OK;
}
}  // namespace

// device pointers of a solve into its arena (defined with the C ABI below)
extern "C" void wire_arena(atpm_solve* s, const Layout& L);

namespace atpm {
void set_last_error(const char* msg) { g_err = msg; }
atpm_status fail_status(atpm_status s, const char* msg) {
    g_err = msg;
    return s;
}
atpm_status ensure_pow_tables(atpm_context* c) { return ensure_tables(c); }
atpm_status ensure_pow_tables_qroot(atpm_context* c) { return ensure_qroot_table(c); }

namespace {
struct HostTable {
    std::vector<DevSolve> tab;
    std::vector<int4> wm, qm;
    std::vector<int2> fm;
    int nmax = 0;
    size_t bt = 0, bw = 0, bf = 0, bq = 0;
};
void host_table(atpm_solve* const* solves, int n, HostTable& h) {
    h.tab.resize(n);
    for (int i = 0; i < n; ++i) {
        h.tab[i] = solves[i]->ds;
        std::vector<int4> w1;
        build_maps(solves[i]->nf, solves[i]->P.ntau, i, w1, h.fm);
        if (solves[i]->nnz > 0) h.wm.insert(h.wm.end(), w1.begin(), w1.end());
        if (solves[i]->nq > 0) h.nmax = std::max(h.nmax, solves[i]->ds.tc_n);
    }
    build_tc_items(solves, n, h.qm);
    h.bt = align256(n * sizeof(DevSolve));
    h.bw = align256(std::max<size_t>(h.wm.size(), 1) * sizeof(int4));
    h.bf = align256(h.fm.size() * sizeof(int2));
    tc_map_extend(h.qm);
    h.bq = align256(std::max<size_t>(h.qm.size(), 1) * sizeof(int4));
}
}  // namespace

size_t batch_table_bytes(atpm_solve* const* solves, int n) {
    HostTable h;
    host_table(solves, n, h);
    return h.bt + h.bw + h.bf + h.bq;
}

atpm_status batch_plan(atpm_solve* const* solves, int n, BatchPlan& plan, cudaStream_t st) {
    HostTable h;
    host_table(solves, n, h);
    const size_t need = h.bt + h.bw + h.bf + h.bq;
    if (need > plan.bytes) {
        if (plan.table) cudaFree(plan.table);
        plan.table = nullptr;
        plan.bytes = 0;
        CK(cudaMalloc(&plan.table, need * 2));  // headroom: a grown batch reuses it
        plan.bytes = need * 2;
    }
    char* t = static_cast<char*>(plan.table);
    CK(cudaMemcpyAsync(t, h.tab.data(), n * sizeof(DevSolve), cudaMemcpyHostToDevice, st));
    if (!h.wm.empty()) CK(cudaMemcpyAsync(t + h.bt, h.wm.data(), h.wm.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(t + h.bt + h.bw, h.fm.data(), h.fm.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
    if (!h.qm.empty())
        CK(cudaMemcpyAsync(t + h.bt + h.bw + h.bf, h.qm.data(), h.qm.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));  // host staging above is released on return
    atpm_solve* s0 = solves[0];
    plan.b = make_batch(s0->ctx, reinterpret_cast<DevSolve*>(t), n, reinterpret_cast<int4*>(t + h.bt), (int)h.wm.size(),
                        reinterpret_cast<int2*>(t + h.bt + h.bw), (int)h.fm.size(), s0->P.precision, s0->P.nx);
    set_tc_map(plan.b, reinterpret_cast<int4*>(t + h.bt + h.bw + h.bf), h.qm.size());
    plan.b.tc_nmax = h.nmax;
    set_remainder_grid(plan.b, solves, n);
    plan.solves.assign(solves, solves + n);
    return ATPM_OK;
}

atpm_status batch_plan_step(const BatchPlan& plan, int k, cudaStream_t st) {
    for (int r = 0; r < k; ++r)
        if (launch_revolution(plan.b, st)) return fail(ATPM_E_CUDA, "batched revolution launch");
    return ATPM_OK;
}

void batch_plan_free(BatchPlan& plan) {
    if (plan.table) cudaFree(plan.table);
    plan.table = nullptr;
    plan.bytes = 0;
    plan.solves.clear();
}

atpm_status solve_refresh(atpm_solve* dst, atpm_solve* src) {
    if (dst->nf != src->nf || dst->nv != src->nv || dst->nnz != src->nnz || dst->tc != src->tc ||
        dst->arena_bytes != src->arena_bytes || dst->wb_bytes != src->wb_bytes || dst->w32_bytes != src->w32_bytes)
        return fail(ATPM_E_INVALID, "solve refresh: different shapes");
    CK(cudaSetDevice(src->ctx->device));
    CK(cudaStreamSynchronize(src->st));
    dst->P = src->P;
    dst->have_forcing = src->have_forcing;
    dst->have_temps = src->have_temps;
    dst->has_position = src->has_position;
    std::memcpy(dst->position, src->position, sizeof dst->position);
    dst->sec_vertex = src->sec_vertex;
    dst->sec_facet = src->sec_facet;
    dst->revs_p = src->revs_p;
    dst->revs_s = src->revs_s;
    dst->ir_abs = src->ir_abs;
    dst->ti = src->ti;
    dst->ds = src->ds;  // scalars; device pointers rebased below
    wire_arena(dst, layout(dst->nv, dst->nf, dst->nnz, dst->P));
    dst->ds.Wb = dst->wb_mem;
    dst->ds.W32 = static_cast<float*>(dst->w32_mem);
    CK(cudaMemcpyAsync(dst->arena, src->arena, dst->arena_bytes, cudaMemcpyDeviceToDevice, dst->st));
    if (dst->wb_mem) CK(cudaMemcpyAsync(dst->wb_mem, src->wb_mem, dst->wb_bytes, cudaMemcpyDeviceToDevice, dst->st));
    if (dst->w32_mem) CK(cudaMemcpyAsync(dst->w32_mem, src->w32_mem, dst->w32_bytes, cudaMemcpyDeviceToDevice, dst->st));
    CK(cudaStreamSynchronize(dst->st));
    return upload_table(dst);
}

atpm_status batch_step(atpm_solve* const* solves, int n, int k, void* table, cudaStream_t st) {
    HostTable h;
    host_table(solves, n, h);
    char* t = static_cast<char*>(table);
    CK(cudaMemcpyAsync(t, h.tab.data(), n * sizeof(DevSolve), cudaMemcpyHostToDevice, st));
    if (!h.wm.empty()) CK(cudaMemcpyAsync(t + h.bt, h.wm.data(), h.wm.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(t + h.bt + h.bw, h.fm.data(), h.fm.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
    if (!h.qm.empty())
        CK(cudaMemcpyAsync(t + h.bt + h.bw + h.bf, h.qm.data(), h.qm.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));  // host staging above is released on return
    atpm_solve* s0 = solves[0];
    Batch b = make_batch(s0->ctx, reinterpret_cast<DevSolve*>(t), n, reinterpret_cast<int4*>(t + h.bt), (int)h.wm.size(),
                         reinterpret_cast<int2*>(t + h.bt + h.bw), (int)h.fm.size(), s0->P.precision, s0->P.nx);
    set_tc_map(b, reinterpret_cast<int4*>(t + h.bt + h.bw + h.bf), h.qm.size());
    b.tc_nmax = h.nmax;
    set_remainder_grid(b, solves, n);
    for (int r = 0; r < k; ++r)
        if (launch_revolution(b, st)) return fail(ATPM_E_CUDA, "batched revolution launch");
    return ATPM_OK;
}

}  // namespace atpm

// =================================================================== C ABI
extern "C" {

ATPM_API const char* atpm_status_string(atpm_status s) {
    switch (s) {
        case ATPM_OK: return "ok";
        case ATPM_E_INVALID: return "invalid argument";
        case ATPM_E_CUDA: return "CUDA error";
        case ATPM_E_NOMEM: return "out of memory";
        case ATPM_E_UNSUPPORTED: return "unsupported";
        case ATPM_E_STATE: return "call out of order";
        case ATPM_E_NONFINITE: return "non-finite temperature";
        case ATPM_E_ITERATION: return "iteration cap reached";
        case ATPM_E_BUDGET: return "over HBM budget";
        case ATPM_E_CANCELLED: return "cancelled";
    }
    return "unknown status";
}

ATPM_API const char* atpm_last_error(void) { return g_err.c_str(); }
ATPM_API int32_t atpm_version(void) { return 100; }

ATPM_API atpm_status atpm_context_create(int32_t device, atpm_context** out) {
    if (!out) return fail(ATPM_E_INVALID, "null out");
    int n = 0;
    CK(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(ATPM_E_INVALID, "device %d of %d", device, n);
    CK(cudaSetDevice(device));
    int sms = 1;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    // the stream-ordered pool the solves allocate from keeps what they
    // release for the next ones (a per-process allocator setting)
    cudaMemPool_t pool = nullptr;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    auto* c = new atpm_context();
    c->device = device;
    c->sm_count = sms;
    *out = c;
    return ATPM_OK;
}

extern "C++" void atpm_context_retain(atpm_context* c) {
    if (c) c->refs.fetch_add(1, std::memory_order_relaxed);
}

extern "C++" void atpm_context_release(atpm_context* c) {
    if (!c || c->refs.fetch_sub(1, std::memory_order_acq_rel) != 1) return;
    cudaSetDevice(c->device);
    if (c->p4.slots_dev) cudaFree(c->p4.slots_dev);
    if (c->p3.slots_dev) cudaFree(c->p3.slots_dev);
    if (c->pq.slots_dev) cudaFree(c->pq.slots_dev);
    delete c;
}

ATPM_API atpm_status atpm_context_destroy(atpm_context* c) {
    atpm_context_release(c);  // freed now, or when its last solve, server or crater goes
    return ATPM_OK;
}

ATPM_API atpm_status atpm_solve_footprint(const atpm_shape* sh, const atpm_params* P, uint64_t* bytes) {
    atpm_status r = check_shape(sh, P);
    if (r) return r;
    Layout L = layout(sh->nv, sh->nf, sh->dep_ptr[sh->nf], *P);
    const size_t nt = (size_t)sh->nf * P->ntau;
    const size_t rs = (P->precision == ATPM_FP64) ? 8 : 4;
    // transient peak: geometry (hp, hm, nrm, dist) or scattering work
    const size_t geo = (size_t)sh->nv * P->ntau * 24 + nt * 56 + (size_t)P->ntau * 16;
    const size_t sct = 3 * nt * rs;
    // FAST with self-heating: this solve's BF16 W tiles (hi + lo; the view-
    // factor tiles are shared with the solve it is cloned from)
    size_t wb = 0;
    if (P->precision == ATPM_FAST && sh->dep_ptr[sh->nf] > 0 && tc_enabled()) {
        int N, nch;
        tc_chunks(P->ntau, &N, &nch);
        wb = align256((size_t)((sh->nf + 63) / 64) * nch * N * 64 * 2 * 2);
        wb += align256((size_t)sh->nf * ((P->ntau + 31) & ~31) * 4);  // W32 of the sparse remainder (when it has one)
    }
    *bytes = (uint64_t)(L.total + wb + std::max(geo, sct) + 64 * 1024);
    return ATPM_OK;
}

// device pointers of a solve into its arena (layout L)
void wire_arena(atpm_solve* s, const Layout& L) {
    char* a = static_cast<char*>(s->arena);
    DevSolve& d = s->ds;
    d.vert = reinterpret_cast<double*>(a + L.off[B_VERT]);
    d.fac = reinterpret_cast<int*>(a + L.off[B_FAC]);
    d.dep_ptr = reinterpret_cast<int*>(a + L.off[B_DPTR]);
    d.dep_idx = reinterpret_cast<int*>(a + L.off[B_DIDX]);
    d.dep_vf = reinterpret_cast<float*>(a + L.off[B_DVF]);
    d.shadow = reinterpret_cast<uint8_t*>(a + L.off[B_SHADOW]);
    d.cosil = a + L.off[B_COS];
    d.Efm = a + L.off[B_EFM];
    d.E = a + L.off[B_E];
    d.stemp0 = a + L.off[B_S0];
    d.stemp1 = a + L.off[B_S1];
    d.temp = a + L.off[B_TEMP];
    d.Q = a + L.off[B_Q];
    d.W = a + L.off[B_W];
    d.conv = reinterpret_cast<uint8_t*>(a + L.off[B_CONV]);
    d.hot = reinterpret_cast<uint8_t*>(a + L.off[B_HOT]);
    d.counts = reinterpret_cast<int*>(a + L.off[B_COUNTS]);
    d.status = reinterpret_cast<int*>(a + L.off[B_STATUS]);
    d.ctl = reinterpret_cast<Ctl*>(a + L.off[B_CTL]);
    d.diag = reinterpret_cast<double*>(a + L.off[B_DIAG]);
    d.act_list = reinterpret_cast<int*>(a + L.off[B_ACT]);
    d.act_cnt = d.act_list + (size_t)2 * s->nf;
    d.rb_act = reinterpret_cast<uint8_t*>(a + L.off[B_RBACT]);
}

ATPM_API atpm_status atpm_solve_create(atpm_context* ctx, const atpm_shape* sh, const atpm_params* P,
                                       atpm_solve** out) {
    if (!ctx || !out) return fail(ATPM_E_INVALID, "null context or out");
    atpm_status r = check_shape(sh, P);
    if (r) return r;
    CK(cudaSetDevice(ctx->device));
    if (P->precision == ATPM_REFERENCE) {
        r = ensure_tables(ctx);
        if (r) return r;
    }
    auto* s = new atpm_solve();
    s->ctx = ctx;
    atpm_context_retain(ctx);
    s->P = *P;
    s->nf = sh->nf;
    s->nv = sh->nv;
    s->nnz = sh->dep_ptr[sh->nf];
    s->rs = (P->precision == ATPM_FP64) ? 8 : 4;
    Layout L = layout(s->nv, s->nf, s->nnz, *P);
    cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) { atpm_context_release(s->ctx); delete s; return fail(ATPM_E_CUDA, "stream: %s", cudaGetErrorString(e)); }
    e = pool_alloc(&s->arena, L.total, s->st);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s->st);
        atpm_context_release(s->ctx); delete s;
        return fail(ATPM_E_NOMEM, "cudaMalloc(%zu): %s", L.total, cudaGetErrorString(e));
    }
    s->arena_bytes = L.total;
    // every array starts at zero, as the reference's do (the pool hands out
    // memory that earlier solves used)
    e = cudaMemsetAsync(s->arena, 0, L.total, s->st);
    if (e != cudaSuccess) {
        cudaFree(s->arena);
        cudaStreamDestroy(s->st);
        atpm_context_release(s->ctx); delete s;
        return fail(ATPM_E_CUDA, "arena clear: %s", cudaGetErrorString(e));
    }
    char* a = static_cast<char*>(s->arena);
    DevSolve& d = s->ds;
    d.nf = s->nf; d.nv = s->nv; d.ntau = P->ntau; d.nx = P->nx; d.revcap = P->revcap;
    d.mode = P->precision; d.nnz = s->nnz; d.freeze = P->freeze ? 1 : 0;
    wire_arena(s, L);
    set_scalars(s, 0.0f);
    s->vert_h.assign(sh->vertices, sh->vertices + 3 * (size_t)s->nv);
    s->fac_h.assign(sh->facets, sh->facets + 3 * (size_t)s->nf);
#define UP(dst, src, bytes) \
    if (bytes) { e = cudaMemcpyAsync((void*)(dst), (src), (bytes), cudaMemcpyHostToDevice, s->st); if (e != cudaSuccess) goto cuda_fail; }
    UP(d.vert, sh->vertices, (size_t)s->nv * 24);
    UP(d.fac, sh->facets, (size_t)s->nf * 12);
    UP(d.dep_ptr, sh->dep_ptr, (size_t)(s->nf + 1) * 4);
    UP(d.dep_idx, sh->dep_idx, (size_t)s->nnz * 4);
    UP(d.dep_vf, sh->dep_vf, (size_t)s->nnz * 4);
#undef UP
    e = cudaMemsetAsync(a + L.off[B_CONV], 0, L.off[B_MEAN] - L.off[B_CONV], s->st);
    if (e != cudaSuccess) goto cuda_fail;
    e = cudaMemsetAsync(d.rb_act, 1, (size_t)(s->nf + 127) / 128, s->st);  // every row block active
    if (e != cudaSuccess) goto cuda_fail;
    e = pool_alloc(reinterpret_cast<void**>(&s->ds_dev), sizeof(DevSolve), s->st);
    if (e != cudaSuccess) goto cuda_fail;
    {
        std::vector<int4> wm;
        std::vector<int2> fm;
        build_maps(s->nf, P->ntau, 0, wm, fm);
        s->nw = s->nnz > 0 ? (int)wm.size() : 0;
        s->nfb = (int)fm.size();
        e = pool_alloc(reinterpret_cast<void**>(&s->wmap), std::max<size_t>(wm.size(), 1) * sizeof(int4), s->st);
        if (e != cudaSuccess) goto cuda_fail;
        e = pool_alloc(reinterpret_cast<void**>(&s->fmap), fm.size() * sizeof(int2), s->st);
        if (e != cudaSuccess) goto cuda_fail;
        e = cudaMemcpyAsync(s->wmap, wm.data(), wm.size() * sizeof(int4), cudaMemcpyHostToDevice, s->st);
        if (e != cudaSuccess) goto cuda_fail;
        e = cudaMemcpyAsync(s->fmap, fm.data(), fm.size() * sizeof(int2), cudaMemcpyHostToDevice, s->st);
        if (e != cudaSuccess) goto cuda_fail;
        // host staging must stay alive until the copies complete
        e = cudaStreamSynchronize(s->st);
        if (e != cudaSuccess) goto cuda_fail;
    }
    if (P->precision == ATPM_FAST && s->nnz > 0 && tc_enabled()) {
        if ((r = build_tc(s, sh)) != ATPM_OK) { atpm_solve_destroy(s); return r; }
    }
    if ((r = upload_table(s)) != ATPM_OK) { atpm_solve_destroy(s); return r; }
    e = cudaEventCreate(&s->ev0);
    if (e != cudaSuccess) goto cuda_fail;
    e = cudaEventCreate(&s->ev1);
    if (e != cudaSuccess) goto cuda_fail;
    *out = s;
    return ATPM_OK;
cuda_fail:
    atpm_solve_destroy(s);
    return fail(ATPM_E_CUDA, "solve setup: %s", cudaGetErrorString(e));
}

ATPM_API atpm_status atpm_solve_destroy(atpm_solve* s) {
    if (!s) return ATPM_OK;
    cudaSetDevice(s->ctx->device);
    if (s->st) cudaStreamSynchronize(s->st);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->side_st) {
        cudaStreamSynchronize(s->side_st);
        cudaStreamDestroy(s->side_st);
    }
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_join) cudaEventDestroy(s->ev_join);
    if (s->wmap) cudaFree(s->wmap);
    if (s->fmap) cudaFree(s->fmap);
    if (s->ds_dev) cudaFree(s->ds_dev);
    if (s->tc && --s->tc->refs == 0) {
        cudaFree(s->tc->mem);
        if (s->tc->rem_mem) cudaFree(s->tc->rem_mem);
        delete s->tc;
    }
    if (s->wb_mem) cudaFree(s->wb_mem);
    if (s->w32_mem) cudaFree(s->w32_mem);
    if (s->qmap) cudaFree(s->qmap);
    if (s->arena) cudaFree(s->arena);
    if (s->st) cudaStreamDestroy(s->st);
    atpm_context* ctx = s->ctx;
    delete s;
    atpm_context_release(ctx);
    return ATPM_OK;
}

ATPM_API atpm_status atpm_solve_clone(atpm_solve* src, atpm_solve** out) {
    if (!src || !out) return fail(ATPM_E_INVALID, "null solve or out");
    CK(cudaSetDevice(src->ctx->device));
    CK(cudaStreamSynchronize(src->st));  // the source's state is complete
    auto* s = new atpm_solve();
    s->ctx = src->ctx;
    atpm_context_retain(s->ctx);
    s->P = src->P;
    s->nf = src->nf; s->nv = src->nv; s->nnz = src->nnz; s->rs = src->rs;
    s->nw = src->nw; s->nfb = src->nfb; s->nq = src->nq;
    s->vert_h = src->vert_h;
    s->fac_h = src->fac_h;
    s->have_forcing = src->have_forcing; s->have_temps = src->have_temps;
    s->has_position = src->has_position;
    std::memcpy(s->position, src->position, sizeof s->position);
    s->sec_vertex = src->sec_vertex; s->sec_facet = src->sec_facet;
    s->revs_p = src->revs_p; s->revs_s = src->revs_s;
    s->ir_abs = src->ir_abs;
    s->ti = src->ti;
    s->ds = src->ds;  // scalars; device pointers rebased below
    cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) { atpm_context_release(s->ctx); delete s; return fail(ATPM_E_CUDA, "stream: %s", cudaGetErrorString(e)); }
    e = pool_alloc(&s->arena, src->arena_bytes, s->st);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s->st);
        atpm_context_release(s->ctx); delete s;
        return fail(ATPM_E_NOMEM, "cudaMalloc(%zu): %s", src->arena_bytes, cudaGetErrorString(e));
    }
    s->arena_bytes = src->arena_bytes;
    wire_arena(s, layout(s->nv, s->nf, s->nnz, s->P));
    e = cudaMemcpyAsync(s->arena, src->arena, s->arena_bytes, cudaMemcpyDeviceToDevice, s->st);
    if (e == cudaSuccess) e = pool_alloc(reinterpret_cast<void**>(&s->ds_dev), sizeof(DevSolve), s->st);
    if (e == cudaSuccess) e = pool_alloc(reinterpret_cast<void**>(&s->wmap), std::max<size_t>((size_t)s->nw, 1) * sizeof(int4), s->st);
    if (e == cudaSuccess) e = pool_alloc(reinterpret_cast<void**>(&s->fmap), (size_t)s->nfb * sizeof(int2), s->st);
    if (e == cudaSuccess && s->nw)
        e = cudaMemcpyAsync(s->wmap, src->wmap, (size_t)s->nw * sizeof(int4), cudaMemcpyDeviceToDevice, s->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->fmap, src->fmap, (size_t)s->nfb * sizeof(int2), cudaMemcpyDeviceToDevice, s->st);
    if (e == cudaSuccess && src->tc) {
        // the tiles are read-only: shared; W is this solve's own
        s->tc = src->tc;
        ++s->tc->refs;
        e = pool_alloc(&s->wb_mem, src->wb_bytes, s->st);
        if (e == cudaSuccess) {
            s->wb_bytes = src->wb_bytes;
            e = cudaMemcpyAsync(s->wb_mem, src->wb_mem, s->wb_bytes, cudaMemcpyDeviceToDevice, s->st);
            s->ds.Wb = s->wb_mem;
        }
        s->ds.W32 = nullptr;
        if (e == cudaSuccess && src->w32_mem) {
            e = pool_alloc(&s->w32_mem, src->w32_bytes, s->st);
            if (e == cudaSuccess) {
                s->w32_bytes = src->w32_bytes;
                e = cudaMemcpyAsync(s->w32_mem, src->w32_mem, s->w32_bytes, cudaMemcpyDeviceToDevice, s->st);
                s->ds.W32 = static_cast<float*>(s->w32_mem);
            }
        }
    }
    if (e == cudaSuccess && src->qmap) {
        e = pool_alloc(reinterpret_cast<void**>(&s->qmap), (size_t)s->nq * sizeof(int4), s->st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->qmap, src->qmap, (size_t)s->nq * sizeof(int4), cudaMemcpyDeviceToDevice, s->st);
    }
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) {
        atpm_solve_destroy(s);
        return fail(ATPM_E_CUDA, "solve clone: %s", cudaGetErrorString(e));
    }
    atpm_status r = upload_table(s);
    if (r) { atpm_solve_destroy(s); return r; }
    *out = s;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_geometry_shadow(atpm_solve* s) {
    if (!s) return fail(ATPM_E_INVALID, "null solve");
    CK(cudaSetDevice(s->ctx->device));
    const atpm_params& P = s->P;
    const int ntau = P.ntau;
    // host: pole matrix, heliocentric centre, rotation table (main.cpp:894-958)
    GeomWork g{};
    std::vector<double> rot, rot2;
    geometry_tables(P, g.tm, g.car, rot, s->revs_p);
    geometry_tables(P, g.tm, g.car, rot2, s->revs_s);
    rot.insert(rot.end(), rot2.begin(), rot2.end());  // [primary | secondary]
    g.vsplit = s->sec_vertex >= 0 ? s->sec_vertex : s->nv;
    if (s->has_position)
        for (int k = 0; k < 3; ++k) g.car[k] = s->position[k];
    const size_t nt = (size_t)s->nf * ntau;
    const size_t bytes = align256((size_t)s->nv * ntau * 24) + align256(nt * 24) * 2 + align256(nt * 8) +
                         align256((size_t)ntau * 32) + 64 * 8;
    void* tmp = nullptr;
    CK(cudaMallocAsync(&tmp, bytes, s->st));
    char* t = static_cast<char*>(tmp);
    g.tests = reinterpret_cast<unsigned long long*>(t + bytes - 64 * 8);
    CK(cudaMemsetAsync(g.tests, 0, 64 * 8, s->st));
    g.hp = reinterpret_cast<double*>(t);
    t += align256((size_t)s->nv * ntau * 24);
    g.hm = reinterpret_cast<double*>(t);
    t += align256(nt * 24);
    g.nrm = reinterpret_cast<double*>(t);
    t += align256(nt * 24);
    g.dist = reinterpret_cast<double*>(t);
    t += align256(nt * 8);
    g.rot = reinterpret_cast<double*>(t);
    g.rot2 = g.rot + 2 * (size_t)ntau;
    cudaError_t e = cudaMemcpyAsync((void*)g.rot, rot.data(), rot.size() * 8, cudaMemcpyHostToDevice, s->st);
    int rc = 0;
    if (e == cudaSuccess) rc = launch_geometry(s->ds, g, s->st);
    // shadow drivers: the projected-box cull in front of the exact test (the
    // same flags); ATPM_SHADOW_CULL=0 runs the plain drivers
    const bool shadows = (P.shadowing == 1 && s->nnz > 0) || P.shadowing == 2;
    // the shadow drivers' time (events) and exact-test count (culled drivers)
    cudaEvent_t sh0 = nullptr, sh1 = nullptr;
    unsigned long long counts[64] = {};
    bool culled = false;
    if (e == cudaSuccess && !rc && shadows) {
        if (cudaEventCreate(&sh0) == cudaSuccess && cudaEventCreate(&sh1) == cudaSuccess)
            cudaEventRecord(sh0, s->st);
        int cr = shadow_cull_enabled() ? launch_shadow_culled(s->ds, g, P.shadowing == 2, s->st) : -1;
        culled = cr != -1;
        if (cr == -1) cr = (P.shadowing == 2) ? launch_shadow_allpairs(s->ds, g, s->st)
                                              : launch_shadow_deplist(s->ds, g, s->st);
        rc = cr;
        if (sh1) cudaEventRecord(sh1, s->st);
        if (!rc) e = cudaMemcpyAsync(counts, g.tests, sizeof counts, cudaMemcpyDeviceToHost, s->st);
    }
    cudaFreeAsync(tmp, s->st);
    cudaError_t e2 = cudaStreamSynchronize(s->st);  // `rot` must outlive the copy
    s->last_shadow_ms = 0.0;
    s->last_shadow_rays = shadows ? (int64_t)nt : 0;
    s->last_shadow_tests = -1;  // not counted by the plain drivers
    if (sh0 && sh1 && e2 == cudaSuccess && !rc) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, sh0, sh1) == cudaSuccess) s->last_shadow_ms = ms;
        if (culled) {
            unsigned long long tot = 0;
            for (unsigned long long c : counts) tot += c;
            s->last_shadow_tests = (int64_t)tot;
        }
    }
    if (sh0) cudaEventDestroy(sh0);
    if (sh1) cudaEventDestroy(sh1);
    if (e != cudaSuccess) return fail(ATPM_E_CUDA, "geometry upload: %s", cudaGetErrorString(e));
    if (rc) return fail(ATPM_E_CUDA, "geometry launch: %s", cudaGetErrorString(cudaGetLastError()));
    if (e2 != cudaSuccess) return fail(ATPM_E_CUDA, "geometry: %s", cudaGetErrorString(e2));
    s->have_forcing = false;
    return ATPM_OK;
}

// The crater model's Sun vectors and facet shadow flags of facets f0 ..
// f0 + nfc - 1 into device arrays, from the solve's geometry parameters and
// shadows (asteroidgeometry, main.cpp:894-1030): the vertex positions of every
// step are recomputed, as atpm_geometry_shadow does, into a scratch buffer.
extern "C++" {
atpm_status atpm::solve_crater_sun(atpm_solve* s, int f0, int nfc, float* sun, int* shadow, cudaStream_t st) {
    const atpm_params& P = s->P;
    const int ntau = P.ntau;
    GeomWork g{};
    std::vector<double> rot, rot2;
    geometry_tables(P, g.tm, g.car, rot, s->revs_p);
    geometry_tables(P, g.tm, g.car, rot2, s->revs_s);
    rot.insert(rot.end(), rot2.begin(), rot2.end());
    g.vsplit = s->sec_vertex >= 0 ? s->sec_vertex : s->nv;
    if (s->has_position)
        for (int k = 0; k < 3; ++k) g.car[k] = s->position[k];
    const size_t hp = align256((size_t)s->nv * ntau * 24);
    void* tmp = nullptr;
    CK(cudaMallocAsync(&tmp, hp + rot.size() * 8, st));
    g.hp = static_cast<double*>(tmp);
    g.rot = reinterpret_cast<double*>(static_cast<char*>(tmp) + hp);
    g.rot2 = g.rot + 2 * (size_t)ntau;
    cudaError_t e = cudaMemcpyAsync((void*)g.rot, rot.data(), rot.size() * 8, cudaMemcpyHostToDevice, st);
    int rc = e == cudaSuccess ? launch_crater_sun(s->ds, g, f0, nfc, sun, shadow, st) : 0;
    cudaFreeAsync(tmp, st);
    cudaError_t e2 = cudaStreamSynchronize(st);  // `rot` must outlive the copy
    if (e != cudaSuccess) return fail(ATPM_E_CUDA, "crater geometry upload: %s", cudaGetErrorString(e));
    if (rc) return fail(ATPM_E_CUDA, "crater geometry launch: %s", cudaGetErrorString(cudaGetLastError()));
    if (e2 != cudaSuccess) return fail(ATPM_E_CUDA, "crater geometry: %s", cudaGetErrorString(e2));
    return ATPM_OK;
}
}  // extern "C++"

ATPM_API atpm_status atpm_solve_solar(const atpm_solve* s, float* solar) {
    if (!s || !solar) return fail(ATPM_E_INVALID, "null argument");
    *solar = s->ds.solar;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_scattering(atpm_solve* s) {
    if (!s) return fail(ATPM_E_INVALID, "null solve");
    CK(cudaSetDevice(s->ctx->device));
    if (launch_single_scattering(s->ds, s->st)) return fail(ATPM_E_CUDA, "single scattering launch");
    if (s->P.multiple_scattering) {
        void* work = nullptr;
        CK(cudaMallocAsync(&work, multiple_scattering_work_bytes(s->ds), s->st));
        int rc = launch_multiple_scattering(s->ds, work, s->st);
        cudaFreeAsync(work, s->st);
        if (rc) return fail(ATPM_E_CUDA, "multiple scattering launch");
    }
    if (launch_forcing_transpose(s->ds, s->st)) return fail(ATPM_E_CUDA, "forcing transpose launch");
    int st = 0;
    CK(cudaMemcpyAsync(&st, s->ds.status, 4, cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    atpm_status r = check_status(s, st);
    if (r) return r;
    s->have_forcing = true;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_set_forcing(atpm_solve* s, const int32_t* shadow, const float* illum) {
    if (!s || !shadow || !illum) return fail(ATPM_E_INVALID, "null argument");
    CK(cudaSetDevice(s->ctx->device));
    const size_t nt = (size_t)s->nf * s->P.ntau;
    void* tmp = nullptr;
    CK(cudaMallocAsync(&tmp, nt * 8, s->st));
    int32_t* sd = static_cast<int32_t*>(tmp);
    float* id = reinterpret_cast<float*>(sd + nt);
    cudaError_t e = cudaMemcpyAsync(sd, shadow, nt * 4, cudaMemcpyHostToDevice, s->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(id, illum, nt * 4, cudaMemcpyHostToDevice, s->st);
    int rc = (e == cudaSuccess) ? launch_set_forcing(s->ds, sd, id, s->st) : 0;
    if (e == cudaSuccess && !rc) rc = launch_forcing_transpose(s->ds, s->st);
    cudaFreeAsync(tmp, s->st);
    cudaError_t e2 = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess || rc || e2 != cudaSuccess)
        return fail(ATPM_E_CUDA, "set_forcing: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    s->have_forcing = true;
    return ATPM_OK;
}

// no active-facet list is valid (counts 0, built for revolution -1)
cudaError_t reset_active_lists(atpm_solve* s) {
    cudaError_t e = cudaMemsetAsync(s->ds.act_cnt, 0, 2 * sizeof(int), s->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->ds.act_cnt + 2, 0xff, 2 * sizeof(int), s->st);
    return e;
}

ATPM_API atpm_status atpm_set_thermal_inertia(atpm_solve* s, float ti) {
    if (!s) return fail(ATPM_E_INVALID, "null solve");
    if (!(ti >= 0.0f) || !std::isfinite(ti)) return fail(ATPM_E_INVALID, "thermal inertia %g", (double)ti);
    CK(cudaSetDevice(s->ctx->device));
    if (ti == 0.0f && s->P.precision == ATPM_REFERENCE) {
        atpm_status rq = ensure_qroot_table(s->ctx);
        if (rq) return rq;
    }
    s->ti = ti;
    set_scalars(s, ti);
    atpm_status r = upload_table(s);
    if (r) return r;
    // reset_asteroid_status (main.cpp:477-485)
    Ctl c{0, 1, 0, 0};
    CK(cudaMemcpyAsync(s->ds.ctl, &c, sizeof c, cudaMemcpyHostToDevice, s->st));
    CK(cudaMemsetAsync(s->ds.conv, 0, s->nf, s->st));
    CK(cudaMemsetAsync(s->ds.rb_act, 1, (size_t)(s->nf + 127) / 128, s->st));
    CK(cudaMemsetAsync(s->ds.hot, 0, s->nf, s->st));
    CK(cudaMemsetAsync(s->ds.counts, 0, (size_t)s->P.revcap * 4, s->st));
    CK(reset_active_lists(s));
    CK(cudaStreamSynchronize(s->st));
    return ATPM_OK;
}

ATPM_API atpm_status atpm_set_albedo(atpm_solve* s, float albedo) {
    if (!s) return fail(ATPM_E_INVALID, "null solve");
    if (!(albedo >= 0.0f && albedo < 1.0f)) return fail(ATPM_E_INVALID, "albedo %g", (double)albedo);
    CK(cudaSetDevice(s->ctx->device));
    s->P.albedo = albedo;
    set_scalars(s, s->ti);
    atpm_status r = upload_table(s);
    if (r) return r;
    // the scattered illumination depends on the albedo: scatter again
    s->have_forcing = false;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_initialise_temperatures(atpm_solve* s) {
    if (!s) return fail(ATPM_E_INVALID, "null solve");
    if (!s->have_forcing) return fail(ATPM_E_STATE, "no forcing: call atpm_scattering or atpm_set_forcing");
    CK(cudaSetDevice(s->ctx->device));
    const int nf = s->nf;
    void* mean = static_cast<char*>(s->arena) + layout(s->nv, s->nf, s->nnz, s->P).off[B_MEAN];
    if (launch_initial_mean(s->ds, mean, s->st)) return fail(ATPM_E_CUDA, "initial mean launch");
    const atpm_params& P = s->P;
    if (P.precision == ATPM_REFERENCE) {
        atpm_status r = ensure_qroot_table(s->ctx);
        if (r) return r;
    }
    if (launch_fill_initial(s->ds, mean, view(s->ctx->pq), s->st)) return fail(ATPM_E_CUDA, "fill launch");
    if (P.precision != ATPM_FP64 && launch_w_bf16_one(s->ds, s->st)) return fail(ATPM_E_CUDA, "W launch");
    CK(cudaStreamSynchronize(s->st));
    s->have_temps = true;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_revolution(atpm_solve* s, int32_t rev, int32_t* numconv, int32_t* converged) {
    if (!s) return fail(ATPM_E_INVALID, "null solve");
    if (!s->have_forcing || (!s->have_temps && s->ti != 0.0f))
        return fail(ATPM_E_STATE, "forcing and initial temperatures required");
    if (rev < 0 || rev >= s->P.revcap) return fail(ATPM_E_INVALID, "rev %d outside [0, revcap)", rev);
    CK(cudaSetDevice(s->ctx->device));
    Ctl c;
    CK(cudaMemcpyAsync(&c, s->ds.ctl, sizeof c, cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    c.rev = rev;
    c.active = 1;
    CK(cudaMemcpyAsync(s->ds.ctl, &c, sizeof c, cudaMemcpyHostToDevice, s->st));
    CK(reset_active_lists(s));  // the caller chooses the revolution: no list carries over
    // the same kernels as the revolution loop (tensor-core product and its
    // sparse remainder for FAST)
    Batch b;
    void* tmp = nullptr;
    atpm_solve* one[1] = {s};
    atpm_status rb = make_batch_for(one, 1, &b, &tmp);
    if (rb) return rb;
    if (launch_revolution(b, s->st)) return fail(ATPM_E_CUDA, "revolution launch");
    int st = 0;
    CK(cudaMemcpyAsync(&c, s->ds.ctl, sizeof c, cudaMemcpyDeviceToHost, s->st));
    CK(cudaMemcpyAsync(&st, s->ds.status, 4, cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    if (numconv) *numconv = c.numconv;
    if (converged) *converged = c.converged;
    return check_status(s, st);
}

ATPM_API atpm_status atpm_run(atpm_solve* s, int32_t* nrev, int32_t* counts) {
    atpm_solve* one[1] = {s};
    return atpm_batch_run(one, 1, nrev, counts);
}

// Solves of one atpm_batch_run are advanced in two groups (even / odd
// positions), each with its own stream and revolution graph: one group's
// small late-revolution kernels and kernel tails overlap the other's work.
// ATPM_BATCH_STREAMS=1 keeps one group.  Each solve's arithmetic does not
// depend on the group it runs in.
int batch_streams() {
    const char* e = std::getenv("ATPM_BATCH_STREAMS");
    return (e && e[0] == '1' && e[1] == 0) ? 1 : 2;
}

namespace {
struct LoopOut {
    atpm_status st = ATPM_OK;
    std::string err;
    int64_t launches = 0;
};

// the revolution loop of one group on its leader's stream: the graph of one
// revolution, replayed in chunks that double up to 32 revolutions, the
// solves' control words read back after each chunk
LoopOut revolution_loop(atpm_solve* const* solves, int n, const Batch& b, cudaGraphExec_t gx, int maxcap,
                        int done_revs, std::vector<Ctl>& ctl) {
    LoopOut o;
    atpm_solve* lead = solves[0];
    if (cudaSetDevice(lead->ctx->device) != cudaSuccess) {
        o.st = fail(ATPM_E_CUDA, "cudaSetDevice");
        o.err = g_err;
        return o;
    }
    cudaError_t e = cudaSuccess;
    int chunk = 4;
    while (e == cudaSuccess && done_revs < maxcap) {
        const int k = std::min(chunk, maxcap - done_revs);
        for (int j = 0; j < k && e == cudaSuccess; ++j) e = cudaGraphLaunch(gx, lead->st);
        o.launches += (int64_t)k * kernels_per_revolution(b);
        done_revs += k;
        if (e != cudaSuccess) break;
        e = cudaEventRecord(lead->ev1, lead->st);
        bool any = false;
        for (int i = 0; i < n && e == cudaSuccess; ++i)
            e = cudaMemcpyAsync(&ctl[i], solves[i]->ds.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, lead->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(lead->st);
        for (int i = 0; i < n; ++i) any = any || ctl[i].active;
        if (!any) break;
        chunk = std::min(chunk * 2, 32);
    }
    if (e != cudaSuccess) {
        o.st = fail(ATPM_E_CUDA, "revolution loop: %s", cudaGetErrorString(e));
        o.err = g_err;
    }
    return o;
}
}  // namespace

ATPM_API atpm_status atpm_batch_run(atpm_solve* const* solves, int32_t n, int32_t* nrev, int32_t* counts) {
    if (!solves || n < 1) return fail(ATPM_E_INVALID, "empty batch");
    atpm_solve* s0 = solves[0];
    for (int i = 0; i < n; ++i) {
        atpm_solve* s = solves[i];
        if (!s) return fail(ATPM_E_INVALID, "null solve %d", i);
        if (s->ctx != s0->ctx || s->P.precision != s0->P.precision || s->P.nx != s0->P.nx)
            return fail(ATPM_E_INVALID, "batch solves must share context, precision and nx");
        if (!s->have_forcing || (!s->have_temps && s->ti != 0.0f))
            return fail(ATPM_E_STATE, "solve %d: forcing and initial temperatures required", i);
    }
    CK(cudaSetDevice(s0->ctx->device));
    // all solves must be ready before their group's stream runs them
    for (int i = 1; i < n; ++i) CK(cudaStreamSynchronize(solves[i]->st));
    const int ng = (n >= 2 && batch_streams() >= 2) ? 2 : 1;
    std::vector<std::vector<atpm_solve*>> gs(ng);
    std::vector<std::vector<int>> gi(ng);
    for (int i = 0; i < n; ++i) {
        gs[i % ng].push_back(solves[i]);
        gi[i % ng].push_back(i);
    }
    std::vector<Batch> bs(ng);
    std::vector<void*> tmps(ng, nullptr);
    auto free_tmps = [&]() {
        for (void* t : tmps)
            if (t) cudaFree(t);
    };
    for (int g = 0; g < ng; ++g) {
        atpm_status rb = make_batch_for(gs[g].data(), (int)gs[g].size(), &bs[g], &tmps[g]);
        if (rb) { free_tmps(); return rb; }
    }
    std::vector<int> maxcap(ng, 0);
    int maxcap_all = 0;
    for (int g = 0; g < ng; ++g)
        for (atpm_solve* s : gs[g]) maxcap[g] = std::max(maxcap[g], s->P.revcap);
    for (int g = 0; g < ng; ++g) maxcap_all = std::max(maxcap_all, maxcap[g]);
    int64_t launches = 0;
    int tuned = 0;
    std::vector<int> done(ng, 0);
    // the timed region starts before any revolution, tuning ones included,
    // on every group's stream
    cudaError_t e = cudaEventRecord(s0->ev0, s0->st);
    for (int g = 1; g < ng && e == cudaSuccess; ++g) e = cudaStreamWaitEvent(gs[g][0]->st, s0->ev0, 0);
    if (e != cudaSuccess) { free_tmps(); return fail(ATPM_E_CUDA, "batch start: %s", cudaGetErrorString(e)); }
    if (bs[0].mode == MODE_FAST) {
        if (!autotune_enabled()) {
            for (Batch& b : bs) {
                b.cond_variant = cond_variant();
                b.tc_stages = 0;
            }
        } else {
            // tunes every group together if this kind of batch has not been
            std::vector<atpm_solve*> leads(ng);
            for (int g = 0; g < ng; ++g) leads[g] = gs[g][0];
            atpm_status rt = autotune(leads, bs, maxcap, done, &launches, &tuned);
            if (rt) { free_tmps(); return rt; }
        }
    }
    std::vector<std::vector<Ctl>> ctl(ng);
    for (int g = 0; g < ng; ++g) ctl[g].resize(gs[g].size());
    std::vector<LoopOut> outs(ng);
    // every group's revolution graph is captured here, on the calling
    // thread, before any group's thread launches: no capture runs beside
    // another thread's launches
    std::vector<cudaGraphExec_t> gx(ng, nullptr);
    auto free_graphs = [&]() {
        for (cudaGraphExec_t x : gx)
            if (x) cudaGraphExecDestroy(x);
    };
    for (int g = 0; g < ng; ++g) {
        atpm_status rc = capture_graph(gs[g][0], bs[g], &gx[g]);
        if (rc) { free_graphs(); free_tmps(); return rc; }
    }
    {
        std::vector<std::thread> workers;
        for (int g = 1; g < ng; ++g)
            workers.emplace_back([&, g]() {
                outs[g] = revolution_loop(gs[g].data(), (int)gs[g].size(), bs[g], gx[g], maxcap[g], done[g], ctl[g]);
            });
        outs[0] = revolution_loop(gs[0].data(), (int)gs[0].size(), bs[0], gx[0], maxcap[0], done[0], ctl[0]);
        for (auto& w : workers) w.join();
    }
    free_graphs();
    free_tmps();
    for (int g = 0; g < ng; ++g) {
        launches += outs[g].launches;
        if (outs[g].st) return fail(outs[g].st, "%s", outs[g].err.c_str());
    }
    float ms = 0.0f;
    for (int g = 0; g < ng; ++g) {
        float m = 0.0f;
        CK(cudaEventElapsedTime(&m, s0->ev0, gs[g][0]->ev1));
        ms = std::max(ms, m);
    }
    int64_t fsteps_total = 0;
    atpm_status worst = ATPM_OK;
    for (int g = 0; g < ng; ++g)
        for (size_t j = 0; j < gs[g].size(); ++j) {
            atpm_solve* s = gs[g][j];
            const int i = gi[g][j];
            std::vector<int32_t> cnt(s->P.revcap);
            int st = 0;
            CK(cudaMemcpy(cnt.data(), s->ds.counts, (size_t)s->P.revcap * 4, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(&st, s->ds.status, 4, cudaMemcpyDeviceToHost));
            const int nr = ctl[g][j].rev;
            if (nrev) nrev[i] = nr;
            if (counts) std::memcpy(counts + (size_t)i * maxcap_all, cnt.data(), (size_t)s->P.revcap * 4);
            const int64_t fs = facet_steps_from_counts(cnt.data(), nr, s->nf, s->P.ntau, s->ti == 0.0f || !s->P.freeze);
            s->last_nrev = nr;
            s->last_facet_steps = fs;
            fsteps_total += fs;
            atpm_status r2 = check_status(s, st);
            if (r2 && !worst) worst = r2;
        }
    const Batch& b = bs[0];
    s0->last_ms = ms;
    s0->last_launches = launches;
    s0->last_facet_steps = fsteps_total;
    s0->last_cond_variant = b.cond_variant;
    s0->last_tc_stages = b.nq > 0 ? (b.tc_stages > 0 ? b.tc_stages : tc_max_stages(b.tc_nmax)) : 0;
    s0->last_tuned = tuned;
    return worst;
}

ATPM_API atpm_status atpm_single_model(atpm_solve* s, const float* ti, int32_t nti, int32_t* nrev,
                                       int32_t* counts, float* stemp1_out) {
    if (!s || !ti || nti < 1) return fail(ATPM_E_INVALID, "bad arguments");
    atpm_status r = atpm_geometry_shadow(s);
    if (r) return r;
    r = atpm_scattering(s);
    if (r) return r;
    bool initialised = false;
    for (int k = 0; k < nti; ++k) {
        r = atpm_set_thermal_inertia(s, ti[k]);
        if (r) return r;
        if (ti[k] != 0.0f && !initialised) {
            r = atpm_initialise_temperatures(s);
            if (r) return r;
            initialised = true;
        }
        r = atpm_run(s, nrev ? nrev + k : nullptr, counts ? counts + (size_t)k * s->P.revcap : nullptr);
        if (r) return r;
    }
    if (stemp1_out) return atpm_get_surface_temperature(s, stemp1_out, nullptr);
    return ATPM_OK;
}

// --------------------------------------------------------------- getters

ATPM_API atpm_status atpm_get_shadow(atpm_solve* s, int32_t* out) {
    if (!s || !out) return fail(ATPM_E_INVALID, "null argument");
    CK(cudaSetDevice(s->ctx->device));
    const size_t nt = (size_t)s->nf * s->P.ntau;
    std::vector<uint8_t> h(nt);
    CK(cudaMemcpyAsync(h.data(), s->ds.shadow, nt, cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    for (size_t i = 0; i < nt; ++i) out[i] = h[i];
    return ATPM_OK;
}

ATPM_API atpm_status atpm_get_illumination(atpm_solve* s, float* out) {
    if (!s || !out) return fail(ATPM_E_INVALID, "null argument");
    CK(cudaSetDevice(s->ctx->device));
    const size_t nt = (size_t)s->nf * s->P.ntau;
    if (s->rs == 8) {
        std::vector<double> h(nt);
        CK(cudaMemcpyAsync(h.data(), s->ds.Efm, nt * 8, cudaMemcpyDeviceToHost, s->st));
        CK(cudaStreamSynchronize(s->st));
        for (size_t i = 0; i < nt; ++i) out[i] = (float)h[i];
    } else {
        CK(cudaMemcpyAsync(out, s->ds.Efm, nt * 4, cudaMemcpyDeviceToHost, s->st));
        CK(cudaStreamSynchronize(s->st));
    }
    return ATPM_OK;
}

ATPM_API atpm_status atpm_get_surface_temperatures(atpm_solve* const* solves, int32_t n, float* const* stemp1) {
    if (!solves || !stemp1 || n < 0) return fail(ATPM_E_INVALID, "null argument");
    for (int i = 0; i < n; ++i)
        if (!solves[i] || !stemp1[i]) return fail(ATPM_E_INVALID, "null solve or output %d", i);
    if (n == 0) return ATPM_OK;
    CK(cudaSetDevice(solves[0]->ctx->device));
    cudaError_t e = cudaSuccess;
    int issued = 0;
    for (; issued < n && e == cudaSuccess; ++issued) {
        atpm_solve* s = solves[issued];
        const size_t nt = s->P.ntau, nf = s->nf;
        void* tmp = nullptr;
        e = cudaMallocAsync(&tmp, nt * nf * 4, s->st);
        if (e != cudaSuccess) break;
        if (launch_transpose(s->ds.stemp1, (int)s->rs, tmp, 4, nt, nf, s->st)) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(stemp1[issued], tmp, nt * nf * 4, cudaMemcpyDeviceToHost, s->st);
        cudaFreeAsync(tmp, s->st);
    }
    cudaError_t e2 = cudaSuccess;
    for (int i = 0; i < issued; ++i) {
        const cudaError_t ei = cudaStreamSynchronize(solves[i]->st);
        if (e2 == cudaSuccess) e2 = ei;
    }
    if (e != cudaSuccess) return fail(ATPM_E_CUDA, "surface temperatures: %s", cudaGetErrorString(e));
    if (e2 != cudaSuccess) return fail(ATPM_E_CUDA, "surface temperatures: %s", cudaGetErrorString(e2));
    return ATPM_OK;
}

ATPM_API atpm_status atpm_get_surface_temperature(atpm_solve* s, float* stemp1, float* stemp0) {
    if (!s) return fail(ATPM_E_INVALID, "null solve");
    CK(cudaSetDevice(s->ctx->device));
    const size_t nt = s->P.ntau, nf = s->nf;
    atpm_status r = ATPM_OK;
    if (s->rs == 8) {
        if (stemp1) r = get_transposed<double>(s, s->ds.stemp1, nt, nf, stemp1, nullptr);
        if (!r && stemp0) r = get_transposed<double>(s, s->ds.stemp0, nt, nf, stemp0, nullptr);
    } else {
        if (stemp1) r = get_transposed<float>(s, s->ds.stemp1, nt, nf, stemp1, nullptr);
        if (!r && stemp0) r = get_transposed<float>(s, s->ds.stemp0, nt, nf, stemp0, nullptr);
    }
    return r;
}

ATPM_API atpm_status atpm_get_surface_temperature64(atpm_solve* s, double* stemp1) {
    if (!s || !stemp1) return fail(ATPM_E_INVALID, "null argument");
    CK(cudaSetDevice(s->ctx->device));
    if (s->rs == 8) return get_transposed<double>(s, s->ds.stemp1, s->P.ntau, s->nf, nullptr, stemp1);
    return get_transposed<float>(s, s->ds.stemp1, s->P.ntau, s->nf, nullptr, stemp1);
}

ATPM_API atpm_status atpm_get_converged(atpm_solve* s, uint8_t* out) {
    if (!s || !out) return fail(ATPM_E_INVALID, "null argument");
    CK(cudaSetDevice(s->ctx->device));
    CK(cudaMemcpyAsync(out, s->ds.conv, (size_t)s->nf, cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    return ATPM_OK;
}

ATPM_API atpm_status atpm_get_depth_temperature(atpm_solve* s, float* temp) {
    if (!s || !temp) return fail(ATPM_E_INVALID, "null argument");
    CK(cudaSetDevice(s->ctx->device));
    if (s->rs == 8) return get_transposed<double>(s, s->ds.temp, s->P.nx + 1, s->nf, temp, nullptr);
    return get_transposed<float>(s, s->ds.temp, s->P.nx + 1, s->nf, temp, nullptr);
}

// observe (3905/Observe/NominalPole/wise_main.cpp:662-730), smooth surface,
// FP64 on the device; constants wise_main.cpp:10-12
// orbital_position_geometry (main.cpp:800-810): heliocentric body centre
// (km) at true anomaly ta_deg of the orbit (a in AU, angles in degrees)
ATPM_API atpm_status atpm_orbital_position(double a_au, double e, double inc_deg, double node_deg, double peri_deg,
                                           double ta_deg, double* car_km) {
    if (!car_km) return fail(ATPM_E_INVALID, "null output");
    const double r = (a_au * kAU * (1.0 - (e * e))) / (1.0 + (e * std::cos(ta_deg * (kPI / 180.0))));
    car_km[0] = r * ((std::cos(node_deg * (kPI / 180.0)) * std::cos((peri_deg + ta_deg) * (kPI / 180.0))) -
                     (std::sin(node_deg * (kPI / 180.0)) * std::sin((peri_deg + ta_deg) * (kPI / 180.0)) *
                      std::cos(inc_deg * (kPI / 180.0))));
    car_km[1] = r * ((std::sin(node_deg * (kPI / 180.0)) * std::cos((peri_deg + ta_deg) * (kPI / 180.0))) +
                     (std::cos(node_deg * (kPI / 180.0)) * std::sin((peri_deg + ta_deg) * (kPI / 180.0)) *
                      std::cos(inc_deg * (kPI / 180.0))));
    car_km[2] = r * std::sin((peri_deg + ta_deg) * (kPI / 180.0)) * std::sin(inc_deg * (kPI / 180.0));
    return ATPM_OK;
}

// non-synchronous binary (175706/Run-04/thermal.cpp: asteroidgeometry
// 1347-1381, set_facet_rotation 860-869, inertiadifference 1925-1967): the
// first primary_vertices vertices / primary_facets facets are the primary,
// which turns primary_revs times per model period (params.ntau steps over
// params.rotation_period_s), the rest turn secondary_revs times
ATPM_API atpm_status atpm_set_binary_rotation(atpm_solve* s, int32_t primary_vertices, int32_t primary_facets,
                                              int32_t primary_revs, int32_t secondary_revs) {
    if (!s) return fail(ATPM_E_INVALID, "null solve");
    if (primary_vertices < 1 || primary_vertices > s->nv || primary_facets < 1 || primary_facets > s->nf ||
        primary_revs < 1 || secondary_revs < 1)
        return fail(ATPM_E_INVALID, "set_binary_rotation: bad split or revolution counts");
    CK(cudaSetDevice(s->ctx->device));
    s->sec_vertex = primary_vertices;
    s->sec_facet = primary_facets;
    s->revs_p = primary_revs;
    s->revs_s = secondary_revs;
    set_scalars(s, s->ti);
    atpm_status r = upload_table(s);
    if (r) return r;
    CK(cudaStreamSynchronize(s->st));
    s->have_forcing = false;  // the geometry changes: recompute shadows and illumination
    return ATPM_OK;
}

// IR absorptivity of the self-heating sum (IR_ABS, 175706/Run-04/thermal.cpp:
// 72, 1950-1952); 1 unless set
ATPM_API atpm_status atpm_set_ir_absorptivity(atpm_solve* s, float ir_abs) {
    if (!s || !(ir_abs >= 0.0f && ir_abs <= 1.0f)) return fail(ATPM_E_INVALID, "set_ir_absorptivity: 0 <= a <= 1");
    CK(cudaSetDevice(s->ctx->device));
    s->ir_abs = ir_abs;
    set_scalars(s, s->ti);
    atpm_status r = upload_table(s);
    if (r) return r;
    CK(cudaStreamSynchronize(s->st));
    return ATPM_OK;
}

// the body centre given directly (orbital sweeps, main.cpp:2612-2640): the
// heliocentric distance and solar constant follow from it as in
// asteroidgeometry (main.cpp:901-905)
ATPM_API atpm_status atpm_set_position(atpm_solve* s, const double* car_km) {
    if (!s || !car_km) return fail(ATPM_E_INVALID, "null argument");
    CK(cudaSetDevice(s->ctx->device));
    for (int k = 0; k < 3; ++k) s->position[k] = car_km[k];
    s->has_position = true;
    s->P.polar[0] = std::sqrt((car_km[0] * car_km[0]) + (car_km[1] * car_km[1]) + (car_km[2] * car_km[2])) / kAU;
    set_scalars(s, s->ti);
    atpm_status r = upload_table(s);
    if (r) return r;
    CK(cudaStreamSynchronize(s->st));
    s->have_forcing = false;
    return ATPM_OK;
}

namespace {
// smooth (rough == null) or rough disk-integrated flux of a solve
atpm_status disk_flux_impl(atpm_solve* s, const double* observer, const int32_t* visibility, double emissivity,
                           int32_t nwl, const double* wavelength_um, double* flux, const FluxArgs* rough) {
    if (!s || !observer || !wavelength_um || !flux || nwl < 1 || nwl > kMaxFluxWavelengths)
        return fail(ATPM_E_INVALID, "disk_flux: bad arguments (1 <= nwl <= %d)", kMaxFluxWavelengths);
    if (!rough && !s->have_temps && s->ti != 0.0f) return fail(ATPM_E_STATE, "disk_flux: no temperatures yet");
    CK(cudaSetDevice(s->ctx->device));
    const atpm_params& P = s->P;
    const int nf = s->nf, ntau = P.ntau;
    FluxArgs a{};
    if (rough) {
        a.sub_T = rough->sub_T;
        a.sub_vis = rough->sub_vis;
        a.nsf = rough->nsf;
        a.sub_total = rough->sub_total;
    }
    std::vector<double> rot, rot2;
    geometry_tables(P, a.tm, a.car, rot, s->revs_p);
    geometry_tables(P, a.tm, a.car, rot2, s->revs_s);
    rot.insert(rot.end(), rot2.begin(), rot2.end());  // [primary | secondary]
    a.vsplit = s->sec_vertex >= 0 ? s->sec_vertex : s->nv;
    // the stage places the body at AU(m) x polar and the observer at the body
    // minus its geocentric vector (wise_main.cpp:8, 530-538)
    const double AUm = 149.6e9;
    a.car[0] = AUm * P.polar[0] * std::cos(P.polar[1]) * std::cos(P.polar[2]);
    a.car[1] = AUm * P.polar[0] * std::cos(P.polar[1]) * std::sin(P.polar[2]);
    a.car[2] = AUm * P.polar[0] * std::sin(P.polar[1]);
    a.obs[0] = a.car[0] - (AUm * observer[0] * std::cos(observer[1]) * std::cos(observer[2]));
    a.obs[1] = a.car[1] - (AUm * observer[0] * std::cos(observer[1]) * std::sin(observer[2]));
    a.obs[2] = a.car[2] - (AUm * observer[0] * std::sin(observer[1]));
    a.eps = emissivity;
    const double cvel = 299792458.0, hcon = 6.626068963e-34, kcon = 1.380650424e-23;
    a.nwl = nwl;
    a.hc = hcon * cvel;
    for (int l = 0; l < nwl; ++l) {
        const double wl = wavelength_um[l] * 1.0e-6;
        a.b1[l] = (2.0 * hcon * cvel * cvel) / std::pow(wl, 5.0);
        a.lk[l] = wl * kcon;
    }
    std::vector<uint8_t> vis;
    if (visibility) {
        vis.resize((size_t)nf * ntau);
        for (size_t i = 0; i < vis.size(); ++i) vis[i] = visibility[i] ? 1 : 0;
    }
    const size_t b_rot = align256(rot.size() * 8), b_part = align256(flux_partial_bytes(s->ds, nwl)),
                 b_out = align256((size_t)ntau * nwl * 8), b_vis = align256(vis.size()),
                 b_geo = rough ? align256((size_t)rough->nsf * 4 * 8) : 0;
    void* tmp = nullptr;
    CK(cudaMallocAsync(&tmp, b_rot + b_part + b_out + b_vis + b_geo, s->st));
    char* t = static_cast<char*>(tmp);
    a.rot = reinterpret_cast<const double*>(t);
    a.rot2 = a.rot + 2 * (size_t)ntau;
    a.partial = reinterpret_cast<double*>(t + b_rot);
    a.out = reinterpret_cast<double*>(t + b_rot + b_part);
    a.visible = visibility ? reinterpret_cast<const uint8_t*>(t + b_rot + b_part + b_out) : nullptr;
    if (rough) a.sub_geo = reinterpret_cast<const double*>(t + b_rot + b_part + b_out + b_vis);
    cudaError_t e = cudaMemcpyAsync((void*)a.rot, rot.data(), rot.size() * 8, cudaMemcpyHostToDevice, s->st);
    if (e == cudaSuccess && visibility)
        e = cudaMemcpyAsync((void*)a.visible, vis.data(), vis.size(), cudaMemcpyHostToDevice, s->st);
    if (e == cudaSuccess && rough)
        e = cudaMemcpyAsync((void*)a.sub_geo, rough->sub_geo, (size_t)rough->nsf * 4 * 8, cudaMemcpyHostToDevice, s->st);
    int rc = 0;
    if (e == cudaSuccess) rc = launch_disk_flux(s->ds, a, s->st);
    if (e == cudaSuccess && !rc) e = cudaMemcpyAsync(flux, a.out, (size_t)ntau * nwl * 8, cudaMemcpyDeviceToHost, s->st);
    cudaFreeAsync(tmp, s->st);
    cudaError_t e2 = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) return fail(ATPM_E_CUDA, "disk_flux: %s", cudaGetErrorString(e));
    if (rc) return fail(ATPM_E_CUDA, "disk_flux launch: %s", cudaGetErrorString(cudaGetLastError()));
    if (e2 != cudaSuccess) return fail(ATPM_E_CUDA, "disk_flux: %s", cudaGetErrorString(e2));
    return ATPM_OK;
}
}  // namespace

ATPM_API atpm_status atpm_disk_flux(atpm_solve* s, const double* observer, const int32_t* visibility,
                                    double emissivity, int32_t nwl, const double* wavelength_um, double* flux) {
    return disk_flux_impl(s, observer, visibility, emissivity, nwl, wavelength_um, flux, nullptr);
}

ATPM_API atpm_status atpm_disk_flux_rough(atpm_solve* s, const atpm_crater* temperatures,
                                          const atpm_crater* sub_visibility, int32_t nsv, const float* crater_vertices,
                                          const int32_t* crater_facets, const double* observer,
                                          const int32_t* visibility, double emissivity, int32_t nwl,
                                          const double* wavelength_um, double* flux) {
    if (!s || !temperatures || !sub_visibility || !crater_vertices || !crater_facets || nsv < 3)
        return fail(ATPM_E_INVALID, "disk_flux_rough: bad arguments");
    const CraterDev& ct = atpm_crater_device(temperatures);
    const CraterDev& cv = atpm_crater_device(sub_visibility);
    if (!ct.stemp1) return fail(ATPM_E_STATE, "disk_flux_rough: the temperature crater holds no temperatures");
    if (!cv.sfc_shadow) return fail(ATPM_E_STATE, "disk_flux_rough: the visibility crater holds no sub-facet array");
    if (ct.nf != s->nf || cv.nf != s->nf || ct.ntau != s->P.ntau || cv.ntau != s->P.ntau || ct.nsf != cv.nsf)
        return fail(ATPM_E_INVALID, "disk_flux_rough: craters and solve differ in facets, steps or sub-facets");
    const int nsf = ct.nsf;
    for (int i = 0; i < 3 * nsf; ++i)
        if (crater_facets[i] < 0 || crater_facets[i] >= nsv)
            return fail(ATPM_E_INVALID, "disk_flux_rough: crater facet vertex %d out of range", crater_facets[i]);
    // the crater's sub-facet normals and areas in double from its float
    // vertices, as the stage computes them (wise_main.cpp:464-490)
    std::vector<double> geo(4 * (size_t)nsf);
    double total = 0.0;
    for (int j = 0; j < nsf; ++j) {
        const float* p0 = crater_vertices + 3 * crater_facets[3 * j];
        const float* p1 = crater_vertices + 3 * crater_facets[3 * j + 1];
        const float* p2 = crater_vertices + 3 * crater_facets[3 * j + 2];
        double a[3], b[3], n[3];
        for (int k = 0; k < 3; ++k) {
            a[k] = (double)p1[k] - (double)p0[k];
            b[k] = (double)p2[k] - (double)p0[k];
        }
        n[0] = (a[1] * b[2]) - (a[2] * b[1]);
        n[1] = (a[2] * b[0]) - (a[0] * b[2]);
        n[2] = (a[0] * b[1]) - (a[1] * b[0]);
        const double nn = std::sqrt((n[0] * n[0]) + (n[1] * n[1]) + (n[2] * n[2]));
        const double area = nn / 2.0;
        for (int k = 0; k < 3; ++k) geo[4 * j + k] = n[k] / nn;
        geo[4 * j + 3] = area;
        total = total + (area * geo[4 * j + 2]);
    }
    CK(atpm_crater_sync(temperatures));
    CK(atpm_crater_sync(sub_visibility));
    FluxArgs r{};
    r.sub_T = ct.stemp1;
    r.sub_vis = cv.sfc_shadow;
    r.sub_geo = geo.data();  // host copy, uploaded with the call's tables
    r.nsf = nsf;
    r.sub_total = total;
    return disk_flux_impl(s, observer, visibility, emissivity, nwl, wavelength_um, flux, &r);
}

ATPM_API atpm_status atpm_energy_balance(atpm_solve* s, double* absorbed, double* emitted, double* mean_t) {
    if (!s) return fail(ATPM_E_INVALID, "null solve");
    CK(cudaSetDevice(s->ctx->device));
    CK(cudaMemsetAsync(s->ds.diag, 0, 32, s->st));
    if (launch_energy_balance(s->ds, s->st)) return fail(ATPM_E_CUDA, "energy launch");
    double d[4];
    CK(cudaMemcpyAsync(d, s->ds.diag, 32, cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    const double n = (double)s->nf * s->P.ntau;
    if (absorbed) *absorbed = d[0];
    if (emitted) *emitted = d[1];
    if (mean_t) *mean_t = d[2] / n;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_selftest_bounded_wait(int32_t device, int64_t limit_cycles, int32_t* status_bits) {
    if (limit_cycles < 0) return fail(ATPM_E_INVALID, "negative wait limit");
    CK(cudaSetDevice(device));
    int* st = nullptr;
    CK(cudaMalloc(&st, sizeof(int)));
    int h = 0;
    cudaError_t e = cudaMemset(st, 0, sizeof(int));
    if (e == cudaSuccess && launch_wait_selftest(st, (long long)limit_cycles, nullptr)) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(&h, st, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(st);
    if (e != cudaSuccess) return fail(ATPM_E_CUDA, "wait self-test: %s", cudaGetErrorString(e));
    if (status_bits) *status_bits = h;
    if (h & ST_TC_TIMEOUT) return fail(ATPM_E_ITERATION, "bounded wait gave up after %lld cycles",
                                       (long long)limit_cycles);
    return ATPM_OK;
}

ATPM_API atpm_status atpm_last_shadow_stats(atpm_solve* s, double* shadow_ms, int64_t* rays, int64_t* exact_tests) {
    if (!s) return fail(ATPM_E_INVALID, "null solve");
    if (shadow_ms) *shadow_ms = s->last_shadow_ms;
    if (rays) *rays = s->last_shadow_rays;
    if (exact_tests) *exact_tests = s->last_shadow_tests;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_get_cosillum(atpm_solve* s, float* out) {
    if (!s || !out) return fail(ATPM_E_INVALID, "null argument");
    CK(cudaSetDevice(s->ctx->device));
    const size_t nt = (size_t)s->nf * s->P.ntau;
    if (s->rs == 8) {
        std::vector<double> h(nt);
        CK(cudaMemcpyAsync(h.data(), s->ds.cosil, nt * 8, cudaMemcpyDeviceToHost, s->st));
        CK(cudaStreamSynchronize(s->st));
        for (size_t i = 0; i < nt; ++i) out[i] = (float)h[i];
    } else {
        CK(cudaMemcpyAsync(out, s->ds.cosil, nt * 4, cudaMemcpyDeviceToHost, s->st));
        CK(cudaStreamSynchronize(s->st));
    }
    return ATPM_OK;
}

ATPM_API atpm_status atpm_profile_revolution(atpm_solve* const* solves, int32_t n, double* kernel_ms,
                                             int64_t* facet_steps, int64_t* active_facets) {
    if (!solves || n < 1 || !kernel_ms) return fail(ATPM_E_INVALID, "bad arguments");
    atpm_solve* s0 = solves[0];
    CK(cudaSetDevice(s0->ctx->device));
    int64_t fs = 0, act = 0;
    for (int i = 0; i < n; ++i) {
        atpm_solve* s = solves[i];
        CK(cudaStreamSynchronize(s->st));
        std::vector<uint8_t> conv(s->nf);
        Ctl c;
        CK(cudaMemcpy(conv.data(), s->ds.conv, s->nf, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(&c, s->ds.ctl, sizeof c, cudaMemcpyDeviceToHost));
        if (!c.active) return fail(ATPM_E_STATE, "solve %d is not active (set the thermal inertia first)", i);
        int a = 0;
        for (uint8_t v : conv) a += (v && s->P.freeze) ? 0 : 1;
        act += a;
        fs += (int64_t)a * s->P.ntau;
    }
    Batch b;
    void* tmp = nullptr;
    atpm_status rb = make_batch_for(solves, n, &b, &tmp);
    if (rb) return rb;
    cudaEvent_t ev[6];
    for (int k = 0; k < 6; ++k) CK(cudaEventCreate(&ev[k]));
    cudaError_t e = cudaEventRecord(ev[0], s0->st);
    for (int part = 0; part < 5 && e == cudaSuccess; ++part) {
        if (launch_revolution_part(b, part, s0->st)) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(ev[part + 1], s0->st);
    }
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[5]);
    for (int k = 0; k < 5 && e == cudaSuccess; ++k) {
        float ms = 0.0f;
        e = cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
        kernel_ms[k] = ms;
    }
    for (int k = 0; k < 6; ++k) cudaEventDestroy(ev[k]);
    if (tmp) cudaFree(tmp);
    if (e != cudaSuccess) return fail(ATPM_E_CUDA, "profile: %s", cudaGetErrorString(e));
    if (facet_steps) *facet_steps = fs;
    if (active_facets) *active_facets = act;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_selfheating_flux(atpm_solve* s, float* q) {
    if (!s || !q) return fail(ATPM_E_INVALID, "null argument");
    CK(cudaSetDevice(s->ctx->device));
    Ctl c, on{0, 1, 0, 0};
    CK(cudaMemcpy(&c, s->ds.ctl, sizeof c, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(s->ds.ctl, &on, sizeof on, cudaMemcpyHostToDevice));
    Batch b;
    void* tmp = nullptr;
    atpm_solve* one[1] = {s};
    atpm_status r = make_batch_for(one, 1, &b, &tmp);
    if (r) return r;
    // every row block, frozen facets included: the flux of the current
    // temperatures for every facet, not only the ones still advancing
    CK(cudaMemsetAsync(s->ds.rb_act, 1, (size_t)(s->nf + 127) / 128, s->st));
    int rc = launch_revolution_part(b, 0, s->st);
    if (!rc) rc = launch_w_bf16_one(s->ds, s->st);
    if (!rc) rc = launch_revolution_part(b, 1, s->st);
    CK(cudaStreamSynchronize(s->st));
    CK(cudaMemcpy(s->ds.ctl, &c, sizeof c, cudaMemcpyHostToDevice));
    if (rc) return fail(ATPM_E_CUDA, "self-heating launch");
    int st = 0;
    CK(cudaMemcpy(&st, s->ds.status, 4, cudaMemcpyDeviceToHost));
    if (st & ST_TC_TIMEOUT) return fail(ATPM_E_ITERATION, "tensor-core pipeline wait timed out");
    const size_t nt = (size_t)s->nf * s->P.ntau;
    if (s->rs == 8) {
        std::vector<double> h(nt);
        CK(cudaMemcpy(h.data(), s->ds.Q, nt * 8, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < nt; ++i) q[i] = (float)h[i];
    } else {
        CK(cudaMemcpy(q, s->ds.Q, nt * 4, cudaMemcpyDeviceToHost));
    }
    return ATPM_OK;
}

ATPM_API atpm_status atpm_last_run_config(atpm_solve* s, int32_t* cond_variant, int32_t* tc_stages,
                                          int32_t* tuned) {
    if (!s) return fail(ATPM_E_INVALID, "null solve");
    if (cond_variant) *cond_variant = s->last_cond_variant;
    if (tc_stages) *tc_stages = s->last_tc_stages;
    if (tuned) *tuned = s->last_tuned;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_last_run_stats(atpm_solve* s, double* ms, int64_t* launches, int64_t* fsteps) {
    if (!s) return fail(ATPM_E_INVALID, "null solve");
    if (ms) *ms = s->last_ms;
    if (launches) *launches = s->last_launches;
    if (fsteps) *fsteps = s->last_facet_steps;
    return ATPM_OK;
}

}  // extern "C"
