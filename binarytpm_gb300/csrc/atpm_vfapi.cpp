// Host side of the view-factor precompute (Shape_Selfheating,
// 3905/Shape_Selfheating/main.cpp:817-889): drives the kernels of
// atpm_viewfactor.cu, compacts the occlusion-culled lists and forms the
// photon-momentum vectors of main.cpp:824-835.  Built with -ffp-contract=off.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/atpm.h"

namespace atpm {
struct VfGeom {
    int nv, nf;
    const float* v;
    const int* fac;
    float* mid;
    float* nrm;
    float* area;
    float* nlen;
};
int vf_init(const VfGeom& g, cudaStream_t st);
int vf_count(const VfGeom& g, int* count, cudaStream_t st);
int vf_fill(const VfGeom& g, const long long* ptr, int* idx, float* vf, float* dir, cudaStream_t st);
int vf_hidden(const VfGeom& g, const long long* ptr, const int* idx, uint8_t* keep, cudaStream_t st);
int vf_refine(const VfGeom& g, const long long* ptr, const int* idx, float* vf, float* dir, cudaStream_t st);
void set_last_error(const char* msg);
}  // namespace atpm

struct atpm_vf_result {
    int nf = 0;
    std::vector<int32_t> ptr, idx;
    std::vector<float> vf, dir, photo;
};

namespace {
struct DevBufs {
    std::vector<void*> p;
    ~DevBufs() { for (void* x : p) cudaFree(x); }
    template <class T> cudaError_t alloc(T** out, size_t n) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, n ? n * sizeof(T) : 1);
        if (e == cudaSuccess) { p.push_back(q); *out = static_cast<T*>(q); }
        return e;
    }
};
atpm_status vfail(atpm_status s, const char* what, cudaError_t e) {
    char buf[256];
    std::snprintf(buf, sizeof buf, "viewfactors: %s: %s", what, cudaGetErrorString(e));
    atpm::set_last_error(buf);
    return s;
}
}  // namespace

extern "C" {

ATPM_API atpm_status atpm_viewfactors_compute(atpm_context* ctx, int32_t nv, int32_t nf, const float* vertices,
                                              const int32_t* facets, int32_t refine, atpm_vf_result** out,
                                              int64_t* nnz_out) {
    (void)ctx;
    if (!vertices || !facets || !out || nv < 3 || nf < 1) {
        atpm::set_last_error("viewfactors: bad arguments");
        return ATPM_E_INVALID;
    }
    for (int i = 0; i < 3 * nf; ++i)
        if (facets[i] < 0 || facets[i] >= nv) {
            atpm::set_last_error("viewfactors: facet vertex index out of range");
            return ATPM_E_INVALID;
        }
    cudaStream_t st = 0;
    DevBufs B;
    atpm::VfGeom g{};
    g.nv = nv;
    g.nf = nf;
    float* v = nullptr;
    int* fac = nullptr;
    cudaError_t e;
#define T(x, what) if ((e = (x)) != cudaSuccess) return vfail(ATPM_E_CUDA, what, e)
    T(B.alloc(&v, (size_t)nv * 3), "alloc");
    T(B.alloc(&fac, (size_t)nf * 3), "alloc");
    T(B.alloc(&g.mid, (size_t)nf * 3), "alloc");
    T(B.alloc(&g.nrm, (size_t)nf * 3), "alloc");
    T(B.alloc(&g.area, (size_t)nf), "alloc");
    T(B.alloc(&g.nlen, (size_t)nf), "alloc");
    T(cudaMemcpy(v, vertices, (size_t)nv * 12, cudaMemcpyHostToDevice), "upload");
    T(cudaMemcpy(fac, facets, (size_t)nf * 12, cudaMemcpyHostToDevice), "upload");
    g.v = v;
    g.fac = fac;
    if (atpm::vf_init(g, st)) return vfail(ATPM_E_CUDA, "init launch", cudaGetLastError());
    int* cnt = nullptr;
    T(B.alloc(&cnt, (size_t)nf), "alloc");
    if (atpm::vf_count(g, cnt, st)) return vfail(ATPM_E_CUDA, "count launch", cudaGetLastError());
    std::vector<int> hc(nf);
    T(cudaMemcpy(hc.data(), cnt, (size_t)nf * 4, cudaMemcpyDeviceToHost), "count");
    std::vector<long long> ptr(nf + 1, 0);
    for (int i = 0; i < nf; ++i) ptr[i + 1] = ptr[i] + hc[i];
    const size_t tot = (size_t)ptr[nf];
    long long* dptr = nullptr;
    int* didx = nullptr;
    float *dvf = nullptr, *ddir = nullptr;
    uint8_t* keep = nullptr;
    T(B.alloc(&dptr, (size_t)nf + 1), "alloc");
    T(B.alloc(&didx, tot), "alloc candidates");
    T(B.alloc(&dvf, tot), "alloc candidates");
    T(B.alloc(&ddir, 3 * tot), "alloc candidates");
    T(B.alloc(&keep, tot), "alloc candidates");
    T(cudaMemcpy(dptr, ptr.data(), (size_t)(nf + 1) * 8, cudaMemcpyHostToDevice), "upload");
    if (atpm::vf_fill(g, dptr, didx, dvf, ddir, st)) return vfail(ATPM_E_CUDA, "fill launch", cudaGetLastError());
    if (atpm::vf_hidden(g, dptr, didx, keep, st)) return vfail(ATPM_E_CUDA, "hidden launch", cudaGetLastError());
    std::vector<int> hidx(tot);
    std::vector<float> hvf(tot), hdir(3 * tot);
    std::vector<uint8_t> hk(tot);
    T(cudaMemcpy(hidx.data(), didx, tot * 4, cudaMemcpyDeviceToHost), "download");
    T(cudaMemcpy(hvf.data(), dvf, tot * 4, cudaMemcpyDeviceToHost), "download");
    T(cudaMemcpy(hdir.data(), ddir, tot * 12, cudaMemcpyDeviceToHost), "download");
    T(cudaMemcpy(hk.data(), keep, tot, cudaMemcpyDeviceToHost), "download");
    auto* r = new atpm_vf_result();
    r->nf = nf;
    r->ptr.assign(nf + 1, 0);
    for (int i = 0; i < nf; ++i) {
        int c = 0;
        for (long long k = ptr[i]; k < ptr[i + 1]; ++k)
            if (hk[k]) {
                r->idx.push_back(hidx[k]);
                r->vf.push_back(hvf[k]);
                r->dir.insert(r->dir.end(), &hdir[3 * k], &hdir[3 * k] + 3);
                ++c;
            }
        r->ptr[i + 1] = r->ptr[i] + c;
    }
    const size_t n2 = r->idx.size();
    if (refine && n2 > 0) {
        std::vector<long long> p2(nf + 1);
        for (int i = 0; i <= nf; ++i) p2[i] = r->ptr[i];
        e = cudaMemcpy(dptr, p2.data(), (size_t)(nf + 1) * 8, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(didx, r->idx.data(), n2 * 4, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(dvf, r->vf.data(), n2 * 4, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(ddir, r->dir.data(), n2 * 12, cudaMemcpyHostToDevice);
        if (e == cudaSuccess && atpm::vf_refine(g, dptr, didx, dvf, ddir, st)) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpy(r->vf.data(), dvf, n2 * 4, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(r->dir.data(), ddir, n2 * 12, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) { delete r; return vfail(ATPM_E_CUDA, "refine", e); }
    }
    // photon-momentum vectors (main.cpp:824-835)
    std::vector<float> area(nf);
    T(cudaMemcpy(area.data(), g.area, (size_t)nf * 4, cudaMemcpyDeviceToHost), "download");
    r->photo.assign((size_t)nf * 3, 0.0f);
    for (int i = 0; i < nf; ++i)
        for (int k = r->ptr[i]; k < r->ptr[i + 1]; ++k)
            for (int c = 0; c < 3; ++c) r->photo[3 * i + c] = r->photo[3 * i + c] + (r->dir[3 * k + c] / area[i]);
#undef T
    *out = r;
    if (nnz_out) *nnz_out = (int64_t)n2;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_viewfactors_get(const atpm_vf_result* r, int32_t* dep_ptr, int32_t* dep_idx, float* dep_vf,
                                          float* dep_vec, float* photovectors) {
    if (!r) { atpm::set_last_error("viewfactors_get: null result"); return ATPM_E_INVALID; }
    if (dep_ptr) std::memcpy(dep_ptr, r->ptr.data(), r->ptr.size() * 4);
    if (dep_idx && !r->idx.empty()) std::memcpy(dep_idx, r->idx.data(), r->idx.size() * 4);
    if (dep_vf && !r->vf.empty()) std::memcpy(dep_vf, r->vf.data(), r->vf.size() * 4);
    if (dep_vec && !r->dir.empty()) std::memcpy(dep_vec, r->dir.data(), r->dir.size() * 4);
    if (photovectors) std::memcpy(photovectors, r->photo.data(), r->photo.size() * 4);
    return ATPM_OK;
}

ATPM_API atpm_status atpm_viewfactors_free(atpm_vf_result* r) {
    delete r;
    return ATPM_OK;
}
}
