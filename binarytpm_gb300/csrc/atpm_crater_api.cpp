// Host side of the crater (roughness) module: runtime-sized C ABI over the
// kernels of atpm_crater.cu.  One call per function of the reference's GPU
// module (3905/Thermal/NominalPole/GPU_code.cu:600-1026); arrays are
// [facet][step][sub-facet] like the module's structs.  Built with
// -ffp-contract=off: the scalars below follow the module's float expressions.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "atpm_host.h"

using namespace atpm;

struct atpm_crater {
    atpm_context* ctx = nullptr;
    int nf = 0, ntau = 0, nx = 0, nsf = 0, precision = 0;
    cudaStream_t st = nullptr;
    void* mem = nullptr;
    float* scratch = nullptr;  // 2 x nf x nsf (initialisation)
    float* numrevs = nullptr;  // [nf] revolutions per model period (non-synchronous binaries), once set
    float PI = 0.0f, rot = 0.0f;
    bool have_model = false;
    // forcing from a solve (atpm_crater_forcing): sub-facet normals, the
    // part's list entries' sub-facet view factors and direction vectors,
    // and which solve and facet range they belong to
    float* cnorm = nullptr;    // [nsf][3]
    float* gvf = nullptr;      // [entries][nsf]
    float* vec = nullptr;      // [entries][3]
    size_t gvf_cap = 0;        // entries allocated
    const atpm_solve* fsolve = nullptr;
    int ff0 = -1;
    CraterDev d{};
};

namespace {
atpm_status cfail(atpm_status s, const char* what, cudaError_t e) {
    char b[256];
    std::snprintf(b, sizeof b, "crater %s: %s", what, cudaGetErrorString(e));
    return atpm::fail_status(s, b);
}
#define CC(call, what)                                          \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return cfail(ATPM_E_CUDA, what, e_); \
    } while (0)

size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

atpm_status launch(atpm_crater* c, int what, std::initializer_list<float> f, void* p0 = nullptr,
                   void* p1 = nullptr) {
    std::vector<float> fa(f);
    fa.resize(8, 0.0f);
    auto view = [](const HostPowTab& h) {
        PowTab t{};
        t.slots = h.slots_dev;
        t.log2slots = h.log2slots;
        t.lo_bits = h.lo_bits;
        t.hi_bits = h.hi_bits;
        return t;
    };
    if (crater_launch(what, c->d, view(c->ctx->p4), view(c->ctx->pq), fa.data(), p0, p1, c->st))
        return cfail(ATPM_E_CUDA, "launch", cudaGetLastError());
    CC(cudaStreamSynchronize(c->st), "kernel");
    int stw = 0;
    CC(cudaMemcpy(&stw, c->d.status, 4, cudaMemcpyDeviceToHost), "status");
    if (stw & ST_NONFINITE) return atpm::fail_status(ATPM_E_NONFINITE, "crater: non-finite temperature");
    if (stw & (ST_NEWTON_CAP | ST_SCATTER_CAP)) return atpm::fail_status(ATPM_E_ITERATION, "crater: iteration cap");
    return ATPM_OK;
}
}  // namespace

const CraterDev& atpm_crater_device(const atpm_crater* c) { return c->d; }
cudaError_t atpm_crater_sync(const atpm_crater* c) {
    cudaError_t e = cudaSetDevice(c->ctx->device);
    return e == cudaSuccess ? cudaStreamSynchronize(c->st) : e;
}

namespace atpm {
atpm_status ensure_pow_tables(atpm_context* c);
atpm_status ensure_pow_tables_qroot(atpm_context* c);
}

extern "C" {

ATPM_API atpm_status atpm_crater_create(atpm_context* ctx, int32_t nf, int32_t ntau, int32_t nx, int32_t nsf,
                                        int32_t precision, atpm_crater** out) {
    if (!ctx || !out || nf < 1 || ntau < 1 || nsf < 1 || nsf > 128)
        return atpm::fail_status(ATPM_E_INVALID, "crater_create: bad arguments (nsf <= 128)");
    if (precision != ATPM_REFERENCE && precision != ATPM_FAST)
        return atpm::fail_status(ATPM_E_UNSUPPORTED, "crater_create: REFERENCE or FAST precision");
    const bool thermal = nx != 0;  // nx = 0: shadow arrays only (Visibility)
    if (thermal && !crater_nx_supported(nx)) return atpm::fail_status(ATPM_E_UNSUPPORTED, "crater_create: nx not built");
    if ((size_t)nsf * nsf * 4 + nsf * 8 > 200 * 1024)
        return atpm::fail_status(ATPM_E_UNSUPPORTED, "crater_create: crater matrix too large for shared memory");
    CC(cudaSetDevice(ctx->device), "device");
    atpm_status r = atpm::ensure_pow_tables(ctx);
    if (!r && precision == ATPM_REFERENCE) r = atpm::ensure_pow_tables_qroot(ctx);
    if (r) return r;
    auto* c = new atpm_crater();
    c->ctx = ctx;
    atpm_context_retain(ctx);
    c->nf = nf;
    c->ntau = ntau;
    c->nx = nx;
    c->nsf = nsf;
    c->precision = precision;
    const size_t fs = (size_t)nf * ntau, fss = fs * nsf, th = thermal ? fss * 4 : 0;
    const size_t sz[] = {(size_t)nsf * nsf * 4, 128 * 3 * 4, (size_t)nsf * 3 * 4, (size_t)nsf * 6 * 4, 100 * 2 * 4,
                         (size_t)nf, (size_t)nf * 4, (size_t)nf * 4, (size_t)nf, fs * 4, fss * 4, fs * 12, fss * 4,
                         th, th, th, th, th, thermal ? (size_t)nf * (nx + 1) * nsf * 4 : 0, 16,
                         thermal ? (size_t)nf * nsf * 8 : 0};
    const int n = sizeof(sz) / sizeof(sz[0]);
    size_t total = 0;
    for (int i = 0; i < n; ++i) total += al(sz[i]);
    cudaError_t e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&c->mem, total);
    if (e != cudaSuccess) {
        if (c->st) cudaStreamDestroy(c->st);
        atpm_context_release(c->ctx);
        delete c;
        return cfail(ATPM_E_NOMEM, "allocation", e);
    }
    cudaMemset(c->mem, 0, total);
    char* p = static_cast<char*>(c->mem);
    void* ptr[32];
    for (int i = 0; i < n; ++i) {
        ptr[i] = sz[i] ? p : nullptr;
        p += al(sz[i]);
    }
    CraterDev& d = c->d;
    d.nf = nf; d.ntau = ntau; d.nx = nx; d.nsf = nsf; d.mode = precision == ATPM_FAST ? MODE_FAST : MODE_REF;
    d.V = (float*)ptr[0]; d.cverts = (float*)ptr[1]; d.cfac = (int*)ptr[2]; d.ctri = (float*)ptr[3];
    d.cmult = (float*)ptr[4]; d.conv = (uint8_t*)ptr[5]; d.albedo = (float*)ptr[6]; d.ti = (float*)ptr[7];
    d.hot = (uint8_t*)ptr[8]; d.shadow = (int*)ptr[9]; d.sfc_shadow = (float*)ptr[10]; d.illumvec = (float*)ptr[11];
    d.illumangle = (float*)ptr[12]; d.RI = (float*)ptr[13]; d.RGI = (float*)ptr[14]; d.RGH = (float*)ptr[15];
    d.stemp0 = (float*)ptr[16]; d.stemp1 = (float*)ptr[17]; d.temp = (float*)ptr[18]; d.status = (int*)ptr[19];
    c->scratch = (float*)ptr[20];
    // trivector multipliers of the 10x10 sub-points (GPU_code.cu:669-687)
    float mult[100][2];
    for (int k = 1; k != 11; ++k)
        for (int l = 1; l != k + 1; ++l) {
            const int q = ((k - 1) * (k - 1)) + (2 * (l - 1));
            mult[q][0] = (float)k - (1.0f / 3.0f);
            mult[q][1] = (float)l - (2.0f / 3.0f);
        }
    for (int k = 2; k != 11; ++k)
        for (int l = 1; l != k; ++l) {
            const int q = ((k - 1) * (k - 1)) + (2 * (l - 1)) + 1;
            mult[q][0] = (float)k - (2.0f / 3.0f);
            mult[q][1] = (float)l - (1.0f / 3.0f);
        }
    cudaMemcpy((void*)d.cmult, mult, sizeof mult, cudaMemcpyHostToDevice);
    c->PI = 4.0f * std::atan(1.0f);
    d.PI = c->PI;
    d.numrevs = nullptr;
    d.ir_abs = 1.0f;
    *out = c;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_crater_destroy(atpm_crater* c) {
    if (!c) return ATPM_OK;
    cudaSetDevice(c->ctx->device);
    if (c->st) cudaStreamSynchronize(c->st);
    if (c->mem) cudaFree(c->mem);
    if (c->numrevs) cudaFree(c->numrevs);
    if (c->cnorm) cudaFree(c->cnorm);
    if (c->gvf) cudaFree(c->gvf);
    if (c->vec) cudaFree(c->vec);
    if (c->st) cudaStreamDestroy(c->st);
    atpm_context* ctx = c->ctx;
    delete c;
    atpm_context_release(ctx);
    return ATPM_OK;
}

ATPM_API atpm_status atpm_crater_set_surface(atpm_crater* c, int32_t nsv, const float* vertices,
                                             const int32_t* facets, const float* viewfactors, float rot_period) {
    if (!c || nsv < 3 || nsv > 128 || !vertices || !facets || (!viewfactors && c->nx != 0))
        return atpm::fail_status(ATPM_E_INVALID, "crater_set_surface: bad arguments");
    for (int i = 0; i < 3 * c->nsf; ++i)
        if (facets[i] < 0 || facets[i] >= nsv) return atpm::fail_status(ATPM_E_INVALID, "crater_set_surface: facet index");
    // surfacegeometry (3905/Thermal/NominalPole/main.cpp:822-868), in float:
    // edge vectors, unit normal, and the sub-point grid's two vectors
    // (-edge 2 / m, edge 1 / m, m = 10)
    const int nsf = c->nsf;
    std::vector<float> tri((size_t)nsf * 6), nrm((size_t)nsf * 3);
    for (int j = 0; j < nsf; ++j) {
        const float* a = vertices + 3 * facets[3 * j];
        const float* b = vertices + 3 * facets[3 * j + 1];
        const float* e = vertices + 3 * facets[3 * j + 2];
        float n0[3], n1[3], nv[3];
        for (int k = 0; k < 3; ++k) {
            n0[k] = b[k] - a[k];
            n1[k] = e[k] - a[k];
        }
        nv[0] = (n0[1] * n1[2]) - (n0[2] * n1[1]);
        nv[1] = (n0[2] * n1[0]) - (n0[0] * n1[2]);
        nv[2] = (n0[0] * n1[1]) - (n0[1] * n1[0]);
        const float n = std::sqrt((nv[0] * nv[0]) + (nv[1] * nv[1]) + (nv[2] * nv[2]));
        for (int k = 0; k < 3; ++k) {
            nrm[3 * j + k] = nv[k] / n;
            tri[6 * j + k] = -1.0f * n1[k] / 10.0f;
            tri[6 * j + 3 + k] = n0[k] / 10.0f;
        }
    }
    atpm_status r = atpm_crater_set_model(c, nsv, vertices, facets, tri.data(), viewfactors, rot_period);
    if (r) return r;
    if (!c->cnorm) CC(cudaMalloc((void**)&c->cnorm, (size_t)nsf * 12), "allocation");
    CC(cudaMemcpy(c->cnorm, nrm.data(), (size_t)nsf * 12, cudaMemcpyHostToDevice), "copy");
    c->d.cnorm = c->cnorm;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_crater_forcing(atpm_solve* s, atpm_crater* c, int32_t f0, const float* dep_vec) {
    if (!s || !c || f0 < 0 || f0 + c->nf > s->nf || c->ntau != s->P.ntau)
        return atpm::fail_status(ATPM_E_INVALID, "crater_forcing: the crater must cover facets f0 .. f0+nf-1 of the solve");
    if (!c->cnorm) return atpm::fail_status(ATPM_E_STATE, "crater_forcing: set the crater surface first");
    if (s->rs != 4) return atpm::fail_status(ATPM_E_UNSUPPORTED, "crater_forcing: FP32 solves (REFERENCE or FAST)");
    if (!s->have_forcing) return atpm::fail_status(ATPM_E_STATE, "crater_forcing: run the solve's geometry and scattering first");
    if (s->ctx->device != c->ctx->device) return atpm::fail_status(ATPM_E_INVALID, "crater_forcing: different devices");
    CC(cudaSetDevice(c->ctx->device), "device");
    CC(cudaStreamSynchronize(s->st), "solve stream");
    CraterDev& d = c->d;
    atpm_status r = solve_crater_sun(s, f0, c->nf, const_cast<float*>(d.illumvec), const_cast<int*>(d.shadow), c->st);
    if (r) return r;
    if (launch_crater_surface(d, const_cast<float*>(d.illumangle), c->st))
        return atpm::fail_status(ATPM_E_CUDA, "crater_forcing: surface launch");
    // the part's list entries
    std::vector<int32_t> ptr(2);
    CC(cudaMemcpy(ptr.data(), s->ds.dep_ptr + f0, 4, cudaMemcpyDeviceToHost), "list bounds");
    CC(cudaMemcpy(ptr.data() + 1, s->ds.dep_ptr + f0 + c->nf, 4, cudaMemcpyDeviceToHost), "list bounds");
    const size_t ne = (size_t)(ptr[1] - ptr[0]);
    if (ne > 0 && !dep_vec) return atpm::fail_status(ATPM_E_INVALID, "crater_forcing: the list entries' vectors are needed");
    if (ne > c->gvf_cap) {
        if (c->gvf) cudaFree(c->gvf);
        if (c->vec) cudaFree(c->vec);
        c->gvf = nullptr;
        c->vec = nullptr;
        c->gvf_cap = 0;
        CC(cudaMalloc((void**)&c->gvf, ne * c->nsf * 4), "allocation");
        CC(cudaMalloc((void**)&c->vec, ne * 12), "allocation");
        c->gvf_cap = ne;
    }
    if (ne > 0) {
        CC(cudaMemcpyAsync(c->vec, dep_vec + 3 * (size_t)ptr[0], ne * 12, cudaMemcpyHostToDevice, c->st), "vectors");
        if (launch_crater_gvf(d, s->ds.vert, s->ds.fac, s->ds.dep_ptr, s->ds.dep_vf, f0, c->vec, c->gvf, c->st))
            return atpm::fail_status(ATPM_E_CUDA, "crater_forcing: view-factor launch");
    }
    // global illumination: the dependent facets' scattered illumination x
    // albedo (a shadow-only crater holds arrays 0-3 only)
    if (c->nx != 0 &&
        launch_crater_gsum(d, s->ds.dep_ptr, s->ds.dep_idx, f0, c->gvf, static_cast<const float*>(s->ds.Efm),
                           s->P.ntau, 0, s->ds.alb, 0.0f, 0.0f, const_cast<float*>(d.RGI), c->st))
        return atpm::fail_status(ATPM_E_CUDA, "crater_forcing: global illumination launch");
    CC(cudaStreamSynchronize(c->st), "forcing");
    c->fsolve = s;
    c->ff0 = f0;
    return ATPM_OK;
}

namespace {
// the crater's arrays of facets c0 .. c0 + n - 1 as a crater of n facets
CraterDev crater_view(const CraterDev& d, int c0, int n) {
    CraterDev v = d;
    v.nf = n;
    const size_t fs = (size_t)d.ntau * d.nsf;
    auto off = [](auto* p, size_t k) { return p ? p + k : p; };
    v.numrevs = off(d.numrevs, (size_t)c0);
    v.conv = off(d.conv, (size_t)c0);
    v.albedo = off(d.albedo, (size_t)c0);
    v.ti = off(d.ti, (size_t)c0);
    v.hot = off(d.hot, (size_t)c0);
    v.shadow = off(d.shadow, (size_t)c0 * d.ntau);
    v.sfc_shadow = off(d.sfc_shadow, c0 * fs);
    v.illumvec = off(d.illumvec, (size_t)c0 * d.ntau * 3);
    v.illumangle = off(d.illumangle, c0 * fs);
    v.RI = off(d.RI, c0 * fs);
    v.RGI = off(d.RGI, c0 * fs);
    v.RGH = off(d.RGH, c0 * fs);
    v.stemp0 = off(d.stemp0, c0 * fs);
    v.stemp1 = off(d.stemp1, c0 * fs);
    v.temp = off(d.temp, (size_t)c0 * (d.nx + 1) * d.nsf);
    return v;
}
}  // namespace

ATPM_API atpm_status atpm_crater_prepare_part(atpm_solve* s, atpm_crater* c, int32_t f0, int32_t c0, int32_t n,
                                              const float* dep_vec) {
    if (!s || !c || n < 1 || f0 < 0 || c0 < 0 || f0 + n > s->nf || c0 + n > c->nf || c->ntau != s->P.ntau)
        return atpm::fail_status(ATPM_E_INVALID, "crater_prepare_part: facets f0 .. f0+n-1 of the solve into "
                                                 "facets c0 .. c0+n-1 of the crater");
    if (!c->cnorm) return atpm::fail_status(ATPM_E_STATE, "crater_prepare_part: set the crater surface first");
    if (c->nx == 0) return atpm::fail_status(ATPM_E_STATE, "crater_prepare_part: shadow-only crater");
    if (s->rs != 4) return atpm::fail_status(ATPM_E_UNSUPPORTED, "crater_prepare_part: FP32 solves (REFERENCE or FAST)");
    if (!s->have_forcing)
        return atpm::fail_status(ATPM_E_STATE, "crater_prepare_part: run the solve's geometry and scattering first");
    if (s->ctx->device != c->ctx->device) return atpm::fail_status(ATPM_E_INVALID, "crater_prepare_part: different devices");
    CC(cudaSetDevice(c->ctx->device), "device");
    CC(cudaStreamSynchronize(s->st), "solve stream");
    const CraterDev v = crater_view(c->d, c0, n);
    atpm_status r = solve_crater_sun(s, f0, n, const_cast<float*>(v.illumvec), const_cast<int*>(v.shadow), c->st);
    if (r) return r;
    if (launch_crater_surface(v, const_cast<float*>(v.illumangle), c->st))
        return atpm::fail_status(ATPM_E_CUDA, "crater_prepare_part: surface launch");
    std::vector<int32_t> ptr(2);
    CC(cudaMemcpy(ptr.data(), s->ds.dep_ptr + f0, 4, cudaMemcpyDeviceToHost), "list bounds");
    CC(cudaMemcpy(ptr.data() + 1, s->ds.dep_ptr + f0 + n, 4, cudaMemcpyDeviceToHost), "list bounds");
    const size_t ne = (size_t)(ptr[1] - ptr[0]);
    if (ne > 0 && !dep_vec)
        return atpm::fail_status(ATPM_E_INVALID, "crater_prepare_part: the list entries' vectors are needed");
    if (ne > c->gvf_cap) {
        if (c->gvf) cudaFree(c->gvf);
        if (c->vec) cudaFree(c->vec);
        c->gvf = nullptr;
        c->vec = nullptr;
        c->gvf_cap = 0;
        CC(cudaMalloc((void**)&c->gvf, ne * c->nsf * 4), "allocation");
        CC(cudaMalloc((void**)&c->vec, ne * 12), "allocation");
        c->gvf_cap = ne;
    }
    if (ne > 0) {
        CC(cudaMemcpyAsync(c->vec, dep_vec + 3 * (size_t)ptr[0], ne * 12, cudaMemcpyHostToDevice, c->st), "vectors");
        if (launch_crater_gvf(v, s->ds.vert, s->ds.fac, s->ds.dep_ptr, s->ds.dep_vf, f0, c->vec, c->gvf, c->st))
            return atpm::fail_status(ATPM_E_CUDA, "crater_prepare_part: view-factor launch");
    }
    if (launch_crater_gsum(v, s->ds.dep_ptr, s->ds.dep_idx, f0, c->gvf, static_cast<const float*>(s->ds.Efm),
                           s->P.ntau, 0, s->ds.alb, 0.0f, 0.0f, const_cast<float*>(v.RGI), c->st))
        return atpm::fail_status(ATPM_E_CUDA, "crater_prepare_part: global illumination launch");
    // global heating from the solve's current surface temperatures
    const size_t nt = (size_t)s->nf * s->P.ntau;
    float* tfm = nullptr;
    CC(cudaMallocAsync((void**)&tfm, nt * 4, c->st), "allocation");
    int rc = launch_transpose_sf(static_cast<const float*>(s->ds.stemp1), s->P.ntau, s->nf, tfm, c->st);
    if (!rc)
        rc = launch_crater_gsum(v, s->ds.dep_ptr, s->ds.dep_idx, f0, c->gvf, tfm, s->P.ntau, 1, 0.0f,
                                (float)s->P.emissivity, 5.67e-8f, const_cast<float*>(v.RGH), c->st);
    cudaFreeAsync(tfm, c->st);
    CC(cudaStreamSynchronize(c->st), "prepare part");
    if (rc) return atpm::fail_status(ATPM_E_CUDA, "crater_prepare_part: global heating launch");
    c->fsolve = nullptr;  // the view factors held belong to a part, not to the whole crater
    c->ff0 = -1;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_crater_global_heating(atpm_solve* s, atpm_crater* c, int32_t f0) {
    if (!s || !c) return atpm::fail_status(ATPM_E_INVALID, "crater_global_heating: null argument");
    if (c->fsolve != s || c->ff0 != f0)
        return atpm::fail_status(ATPM_E_STATE, "crater_global_heating: run atpm_crater_forcing for this solve and f0 first");
    if (c->nx == 0) return atpm::fail_status(ATPM_E_STATE, "crater_global_heating: shadow-only crater");
    CC(cudaSetDevice(c->ctx->device), "device");
    CC(cudaStreamSynchronize(s->st), "solve stream");
    // the dependent facets' surface temperatures, facet-major
    const size_t nt = (size_t)s->nf * s->P.ntau;
    float* tfm = nullptr;
    CC(cudaMallocAsync((void**)&tfm, nt * 4, c->st), "allocation");
    int rc = launch_transpose_sf(static_cast<const float*>(s->ds.stemp1), s->P.ntau, s->nf, tfm, c->st);
    // load_GPU_roughness_globalheating (main.cpp:2072-2103): EPS x SIGMA x T^4
    if (!rc)
        rc = launch_crater_gsum(c->d, s->ds.dep_ptr, s->ds.dep_idx, f0, c->gvf, tfm, s->P.ntau, 1, 0.0f,
                                (float)s->P.emissivity, 5.67e-8f, const_cast<float*>(c->d.RGH), c->st);
    cudaFreeAsync(tfm, c->st);
    CC(cudaStreamSynchronize(c->st), "global heating");
    if (rc) return atpm::fail_status(ATPM_E_CUDA, "crater_global_heating: launch");
    return ATPM_OK;
}

ATPM_API atpm_status atpm_crater_set_revolutions(atpm_crater* c, const float* numrevs) {
    if (!c) return atpm::fail_status(ATPM_E_INVALID, "null crater");
    CC(cudaSetDevice(c->ctx->device), "device");
    if (!numrevs) {
        c->d.numrevs = nullptr;
        return ATPM_OK;
    }
    for (int f = 0; f < c->nf; ++f)
        if (!(numrevs[f] > 0.0f) || !std::isfinite(numrevs[f]))
            return atpm::fail_status(ATPM_E_INVALID, "crater_set_revolutions: revolutions must be positive");
    if (!c->numrevs) CC(cudaMalloc((void**)&c->numrevs, (size_t)c->nf * 4), "allocation");
    CC(cudaMemcpy(c->numrevs, numrevs, (size_t)c->nf * 4, cudaMemcpyHostToDevice), "copy");
    c->d.numrevs = c->numrevs;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_crater_set_ir_absorptivity(atpm_crater* c, float ir_abs) {
    if (!c || !(ir_abs >= 0.0f) || !std::isfinite(ir_abs))
        return atpm::fail_status(ATPM_E_INVALID, "crater_set_ir_absorptivity: bad arguments");
    c->d.ir_abs = ir_abs;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_crater_set_model(atpm_crater* c, int32_t nsv, const float* vertices, const int32_t* facets,
                                           const float* trivectors, const float* viewfactors, float rot_period) {
    if (!c || nsv < 3 || nsv > 128 || !vertices || !facets || !trivectors || (!viewfactors && c->nx != 0))
        return atpm::fail_status(ATPM_E_INVALID, "crater_set_model: bad arguments");
    for (int i = 0; i < 3 * c->nsf; ++i)
        if (facets[i] < 0 || facets[i] >= nsv) return atpm::fail_status(ATPM_E_INVALID, "crater_set_model: facet index");
    CC(cudaSetDevice(c->ctx->device), "device");
    if (viewfactors)
        CC(cudaMemcpy((void*)c->d.V, viewfactors, (size_t)c->nsf * c->nsf * 4, cudaMemcpyHostToDevice), "model");
    CC(cudaMemcpy((void*)c->d.cverts, vertices, (size_t)nsv * 12, cudaMemcpyHostToDevice), "model");
    CC(cudaMemcpy((void*)c->d.cfac, facets, (size_t)c->nsf * 12, cudaMemcpyHostToDevice), "model");
    CC(cudaMemcpy((void*)c->d.ctri, trivectors, (size_t)c->nsf * 24, cudaMemcpyHostToDevice), "model");
    c->rot = rot_period;
    c->d.rot_period = rot_period;
    c->have_model = true;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_crater_set_properties(atpm_crater* c, const uint8_t* converged, const float* albedo,
                                                const float* ti) {
    if (!c) return atpm::fail_status(ATPM_E_INVALID, "null crater");
    CC(cudaSetDevice(c->ctx->device), "device");
    if (converged) CC(cudaMemcpy(c->d.conv, converged, c->nf, cudaMemcpyHostToDevice), "properties");
    if (albedo) CC(cudaMemcpy((void*)c->d.albedo, albedo, (size_t)c->nf * 4, cudaMemcpyHostToDevice), "properties");
    if (ti) CC(cudaMemcpy((void*)c->d.ti, ti, (size_t)c->nf * 4, cudaMemcpyHostToDevice), "properties");
    return ATPM_OK;
}

ATPM_API atpm_status atpm_crater_get_properties(atpm_crater* c, uint8_t* converged, float* albedo, float* ti) {
    if (!c) return atpm::fail_status(ATPM_E_INVALID, "null crater");
    CC(cudaSetDevice(c->ctx->device), "device");
    if (converged) CC(cudaMemcpy(converged, c->d.conv, c->nf, cudaMemcpyDeviceToHost), "properties");
    if (albedo) CC(cudaMemcpy(albedo, c->d.albedo, (size_t)c->nf * 4, cudaMemcpyDeviceToHost), "properties");
    if (ti) CC(cudaMemcpy(ti, c->d.ti, (size_t)c->nf * 4, cudaMemcpyDeviceToHost), "properties");
    return ATPM_OK;
}

// which: 0 shadow (int [nf][ntau]), 1 sub-facet shadow, 2 Sun vector ([nf][ntau][3]), 3 sub-facet Sun angle,
// 4 illumination, 5 global illumination, 6 global heating (sub-facet arrays [nf][ntau][nsf])
ATPM_API atpm_status atpm_crater_set_array(atpm_crater* c, int32_t which, const void* data) {
    if (!c || !data || which < 0 || which > 6) return atpm::fail_status(ATPM_E_INVALID, "crater_set_array");
    if (which > 3 && c->nx == 0) return atpm::fail_status(ATPM_E_STATE, "crater_set_array: shadow-only crater");
    CC(cudaSetDevice(c->ctx->device), "device");
    const size_t fs = (size_t)c->nf * c->ntau, fss = fs * c->nsf;
    void* dst[] = {(void*)c->d.shadow, c->d.sfc_shadow, (void*)c->d.illumvec, (void*)c->d.illumangle, c->d.RI,
                   (void*)c->d.RGI, (void*)c->d.RGH};
    const size_t bytes[] = {fs * 4, fss * 4, fs * 12, fss * 4, fss * 4, fss * 4, fss * 4};
    CC(cudaMemcpy(dst[which], data, bytes[which], cudaMemcpyHostToDevice), "set_array");
    return ATPM_OK;
}

ATPM_API atpm_status atpm_crater_get_array(atpm_crater* c, int32_t which, void* data) {
    if (!c || !data || which < 0 || which > 6) return atpm::fail_status(ATPM_E_INVALID, "crater_get_array");
    if (which > 3 && c->nx == 0) return atpm::fail_status(ATPM_E_STATE, "crater_get_array: shadow-only crater");
    CC(cudaSetDevice(c->ctx->device), "device");
    const size_t fs = (size_t)c->nf * c->ntau, fss = fs * c->nsf;
    const void* src[] = {c->d.shadow, c->d.sfc_shadow, c->d.illumvec, c->d.illumangle, c->d.RI, c->d.RGI, c->d.RGH};
    const size_t bytes[] = {fs * 4, fss * 4, fs * 12, fss * 4, fss * 4, fss * 4, fss * 4};
    CC(cudaMemcpy(data, src[which], bytes[which], cudaMemcpyDeviceToHost), "get_array");
    return ATPM_OK;
}

namespace {
// device base and per-facet bytes of array `which` (0-6 as set/get_array,
// 7 stemp0, 8 stemp1, 9 depth columns)
bool array_view(atpm_crater* c, int which, void** dev, size_t* per_facet) {
    const size_t st = (size_t)c->ntau, sf = st * c->nsf;
    switch (which) {
        case 0: *dev = (void*)c->d.shadow; *per_facet = st * 4; return true;
        case 1: *dev = (void*)c->d.sfc_shadow; *per_facet = sf * 4; return true;
        case 2: *dev = (void*)c->d.illumvec; *per_facet = st * 12; return true;
        case 3: *dev = (void*)c->d.illumangle; *per_facet = sf * 4; return true;
        case 4: *dev = (void*)c->d.RI; *per_facet = sf * 4; break;
        case 5: *dev = (void*)c->d.RGI; *per_facet = sf * 4; break;
        case 6: *dev = (void*)c->d.RGH; *per_facet = sf * 4; break;
        case 7: *dev = (void*)c->d.stemp0; *per_facet = sf * 4; break;
        case 8: *dev = (void*)c->d.stemp1; *per_facet = sf * 4; break;
        case 9: *dev = (void*)c->d.temp; *per_facet = (size_t)(c->nx + 1) * c->nsf * 4; break;
        default: return false;
    }
    return c->nx != 0;  // 4-9 exist only on a thermal crater
}
}  // namespace

ATPM_API atpm_status atpm_crater_set_array_strided(atpm_crater* c, int32_t which, const void* base,
                                                   uint64_t facet_stride) {
    void* dev = nullptr;
    size_t per = 0;
    if (!c || !base || !array_view(c, which, &dev, &per) || facet_stride < per)
        return atpm::fail_status(ATPM_E_INVALID, "crater_set_array_strided: bad arguments");
    CC(cudaSetDevice(c->ctx->device), "device");
    if (facet_stride == per)
        CC(cudaMemcpy(dev, base, per * c->nf, cudaMemcpyHostToDevice), "set_array_strided");
    else
        CC(cudaMemcpy2D(dev, per, base, facet_stride, per, c->nf, cudaMemcpyHostToDevice), "set_array_strided");
    return ATPM_OK;
}

ATPM_API atpm_status atpm_crater_get_array_strided(atpm_crater* c, int32_t which, void* base, uint64_t facet_stride) {
    void* dev = nullptr;
    size_t per = 0;
    if (!c || !base || !array_view(c, which, &dev, &per) || facet_stride < per)
        return atpm::fail_status(ATPM_E_INVALID, "crater_get_array_strided: bad arguments");
    CC(cudaSetDevice(c->ctx->device), "device");
    if (facet_stride == per) {
        CC(cudaMemcpy(base, dev, per * c->nf, cudaMemcpyDeviceToHost), "get_array_strided");
        return ATPM_OK;
    }
    // a strided copy into freshly allocated (never touched) host memory is
    // slow when the copy engine meets its page faults row by row: touch the
    // destination rows first
    char* b = static_cast<char*>(base);
    for (int f = 0; f < c->nf; ++f) std::memset(b + (size_t)f * facet_stride, 0, per);
    CC(cudaMemcpy2D(base, facet_stride, dev, per, per, c->nf, cudaMemcpyDeviceToHost), "get_array_strided");
    return ATPM_OK;
}

ATPM_API atpm_status atpm_crater_partial_shadow(atpm_crater* c) {
    if (!c || !c->have_model) return atpm::fail_status(ATPM_E_STATE, "crater: model not set");
    CC(cudaSetDevice(c->ctx->device), "device");
    return launch(c, 0, {});
}

ATPM_API atpm_status atpm_crater_scattering(atpm_crater* c, float solar, float accuracy, int32_t multiple) {
    if (!c || !c->have_model || c->nx == 0)
        return atpm::fail_status(ATPM_E_STATE, "crater: model not set or shadow-only crater");
    CC(cudaSetDevice(c->ctx->device), "device");
    return launch(c, 1, {solar, accuracy, multiple ? 1.0f : 0.0f});
}

ATPM_API atpm_status atpm_crater_zero_temperatures(atpm_crater* c) {
    if (!c) return atpm::fail_status(ATPM_E_INVALID, "null crater");
    if (c->nx == 0) return atpm::fail_status(ATPM_E_STATE, "shadow-only crater");
    CC(cudaSetDevice(c->ctx->device), "device");
    const size_t fss = (size_t)c->nf * c->ntau * c->nsf;
    CC(cudaMemset(c->d.stemp0, 0, fss * 4), "zero");
    CC(cudaMemset(c->d.stemp1, 0, fss * 4), "zero");
    CC(cudaMemset(c->d.temp, 0, (size_t)c->nf * (c->nx + 1) * c->nsf * 4), "zero");
    return ATPM_OK;
}

// roughness_initialise_temperatures (GPU_code.cu:328-371): mean absorbed
// flux -> 4th root -> crater self-heating of that temperature -> second mean
// -> 4th root -> every depth and step
ATPM_API atpm_status atpm_crater_initialise_temperatures(atpm_crater* c, float eps, float sigma) {
    if (!c || !c->have_model || c->nx == 0)
        return atpm::fail_status(ATPM_E_STATE, "crater: model not set or shadow-only crater");
    CC(cudaSetDevice(c->ctx->device), "device");
    const float es = eps * sigma;
    const size_t n = (size_t)c->nf * c->nsf;
    float* mean = c->scratch;
    float* selfh = c->scratch + n;
    // a non-finite value is reported but does not stop the sequence (the
    // module's kernels run on regardless); any other failure does
    atpm_status r = ATPM_OK;
    for (int k = 0; k < 6; ++k) {
        atpm_status x = ATPM_OK;
        switch (k) {
            case 0: x = launch(c, 5, {}, mean, nullptr); break;
            case 1: x = launch(c, 8, {es}, mean); break;
            case 2: x = launch(c, 6, {es}, mean, selfh); break;
            case 3: x = launch(c, 5, {}, mean, selfh); break;
            case 4: x = launch(c, 8, {es}, mean); break;
            default: x = launch(c, 7, {}, mean, nullptr); break;
        }
        if (x != ATPM_OK) {
            if (x != ATPM_E_NONFINITE) return x;
            r = x;
        }
    }
    return r;
}

// GPU_inertia_difference (GPU_code.cu:982-998): one revolution
ATPM_API atpm_status atpm_crater_inertia_difference(atpm_crater* c, float eps, float sigma, float tacc) {
    if (!c || !c->have_model || c->nx == 0)
        return atpm::fail_status(ATPM_E_STATE, "crater: model not set or shadow-only crater");
    CC(cudaSetDevice(c->ctx->device), "device");
    const float es = eps * sigma, es4 = 4.0f * es;
    const float dz = 8.0f / c->nx;
    const float dtau = (2.0f * c->PI) / c->ntau;
    const float m0 = dtau / (dz * dz);
    const float tacc2 = tacc / 10.0f;
    return launch(c, 2, {es, es4, m0, dz, tacc, tacc2});
}

ATPM_API atpm_status atpm_crater_inst_equilibrium(atpm_crater* c, float eps, float sigma) {
    if (!c || !c->have_model || c->nx == 0)
        return atpm::fail_status(ATPM_E_STATE, "crater: model not set or shadow-only crater");
    CC(cudaSetDevice(c->ctx->device), "device");
    return launch(c, 3, {eps * sigma});
}

ATPM_API atpm_status atpm_crater_converged(atpm_crater* c, float tacc) {
    if (!c) return atpm::fail_status(ATPM_E_INVALID, "null crater");
    if (c->nx == 0) return atpm::fail_status(ATPM_E_STATE, "shadow-only crater");
    CC(cudaSetDevice(c->ctx->device), "device");
    return launch(c, 4, {tacc});
}

ATPM_API atpm_status atpm_crater_get_temperatures(atpm_crater* c, float* stemp0, float* stemp1, float* temp) {
    if (!c) return atpm::fail_status(ATPM_E_INVALID, "null crater");
    if (c->nx == 0) return atpm::fail_status(ATPM_E_STATE, "shadow-only crater");
    CC(cudaSetDevice(c->ctx->device), "device");
    const size_t fss = (size_t)c->nf * c->ntau * c->nsf;
    if (stemp0) CC(cudaMemcpy(stemp0, c->d.stemp0, fss * 4, cudaMemcpyDeviceToHost), "get");
    if (stemp1) CC(cudaMemcpy(stemp1, c->d.stemp1, fss * 4, cudaMemcpyDeviceToHost), "get");
    if (temp) CC(cudaMemcpy(temp, c->d.temp, (size_t)c->nf * (c->nx + 1) * c->nsf * 4, cudaMemcpyDeviceToHost), "get");
    return ATPM_OK;
}

}  // extern "C"
