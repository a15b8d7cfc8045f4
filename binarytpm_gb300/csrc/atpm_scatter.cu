// Scattered-sunlight kernels (reference singlescattering / multiplescattering,
// 3905/Thermal/NominalPole/main.cpp:1321-1433).
//
//   k_single_scatter  E[f][s] = S cos_f shadow_f + sum_k vf_k S A cos_g shadow_g
//                     warp = 32 steps of one facet: the list loop is uniform
//                     and every gather of cos/shadow is one coalesced segment
//   k_multi_gs        the reference's per-step Gauss-Seidel sweep in facet
//                     order (values of facets before f in this sweep, after f
//                     from the last sweep) until every |change| <= accuracy;
//                     one warp per step, lanes fetch 32 list entries at once
//                     and the two partial sums are accumulated in list order
//   k_multi_jacobi    FAST precision: Jacobi sweeps of every facet and step at
//                     once (warp = 32 steps of one facet, as the single
//                     scattering), iterated to the same accuracy; the fixed
//                     point is the reference's, the iterates are not
//   k_forcing_t       [nf][ntau] -> [ntau][nf] for the conduction sweep
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <utility>

#include "../../include/atpm.h"
#include "atpm_internal.h"

namespace atpm {

template <int MODE> struct Sa;
template <> struct Sa<MODE_REF> {
    using R = float;
    static __device__ __forceinline__ R add(R a, R b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ R sub(R a, R b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ R mul(R a, R b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ R div(R a, R b) { return __fdiv_rn(a, b); }
};
template <> struct Sa<MODE_FP64> {
    using R = double;
    static __device__ __forceinline__ R add(R a, R b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ R sub(R a, R b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ R mul(R a, R b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ R div(R a, R b) { return __ddiv_rn(a, b); }
};
template <> struct Sa<MODE_FAST> {
    using R = float;
    static __device__ __forceinline__ R add(R a, R b) { return a + b; }
    static __device__ __forceinline__ R sub(R a, R b) { return a - b; }
    static __device__ __forceinline__ R mul(R a, R b) { return a * b; }
    static __device__ __forceinline__ R div(R a, R b) { return a / b; }
};

template <int MODE>
__global__ void __launch_bounds__(256) k_single_scatter(DevSolve sv) {
    using A = Sa<MODE>;
    using R = typename A::R;
    const int nf = sv.nf, ntau = sv.ntau;
    const int f = blockIdx.y * blockDim.y + threadIdx.y;
    const int s = blockIdx.x * 32 + threadIdx.x;
    if (f >= nf) return;
    const R* cs = static_cast<const R*>(sv.cosil);
    const R solar = (MODE == MODE_FP64) ? (R)sv.solar_d : (R)sv.solar;
    const R alb = (MODE == MODE_FP64) ? (R)sv.alb_d : (R)sv.alb;
    const bool ok = s < ntau;
    const int sc = ok ? s : 0;
    R e = A::mul(A::mul(solar, cs[(size_t)f * ntau + sc]), (R)sv.shadow[(size_t)f * ntau + sc]);
    const int k1 = sv.dep_ptr[f + 1];
    for (int k = sv.dep_ptr[f]; k < k1; ++k) {
        const int g = __ldg(&sv.dep_idx[k]);
        const R v = (R)__ldg(&sv.dep_vf[k]);
        const size_t o = (size_t)g * ntau + sc;
        e = A::add(e, A::mul(A::mul(A::mul(A::mul(v, solar), alb), cs[o]), (R)sv.shadow[o]));
    }
    if (ok) static_cast<R*>(sv.Efm)[(size_t)f * ntau + s] = e;
}

// Gauss-Seidel multiple scattering, one warp per step.  `work` holds three
// [ntau][nf] arrays: solar power, previous sweep, current sweep.
template <int MODE>
__global__ void __launch_bounds__(32) k_multi_gs(DevSolve sv, void* work, int cap) {
    using A = Sa<MODE>;
    using R = typename A::R;
    const int nf = sv.nf, ntau = sv.ntau;
    const int s = blockIdx.x;
    const int lane = threadIdx.x;
    if (s >= ntau) return;
    R* sp = static_cast<R*>(work) + (size_t)s * nf;
    R* po = sp + (size_t)ntau * nf;
    R* pn = po + (size_t)ntau * nf;
    const R* cs = static_cast<const R*>(sv.cosil);
    R* Efm = static_cast<R*>(sv.Efm);
    const R solar = (MODE == MODE_FP64) ? (R)sv.solar_d : (R)sv.solar;
    const R alb = (MODE == MODE_FP64) ? (R)sv.alb_d : (R)sv.alb;
    const R acc = (MODE == MODE_FP64) ? (R)sv.sacc_d : (R)sv.sacc;
    for (int c = lane; c < nf; c += 32) {
        const size_t o = (size_t)c * ntau + s;
        sp[c] = A::mul(A::mul(solar, cs[o]), (R)sv.shadow[o]);
        po[c] = A::mul(alb, Efm[o]);
    }
    __syncwarp();
    bool more = true;
    int it = 0;
    while (more) {
        if (it == cap) {
            if (lane == 0) atomicOr(sv.status, ST_SCATTER_CAP);
            break;
        }
        for (int c = 0; c < nf; ++c) {
            const int d0 = sv.dep_ptr[c], d1 = sv.dep_ptr[c + 1];
            R val;
            if (d1 == d0) {
                val = po[c];
            } else {
                R after = R(0), before = R(0);
                for (int base = d0; base < d1; base += 32) {
                    const int k = base + lane;
                    R term = R(0);
                    int isafter = 0;
                    if (k < d1) {
                        const int g = __ldg(&sv.dep_idx[k]);
                        const R v = (R)__ldg(&sv.dep_vf[k]);
                        isafter = g > c;
                        term = A::mul(v, isafter ? po[g] : pn[g]);
                    }
                    const int n = min(32, d1 - base);
                    for (int j = 0; j < n; ++j) {
                        const R tj = __shfl_sync(0xffffffffu, term, j);
                        const int aj = __shfl_sync(0xffffffffu, isafter, j);
                        if (aj) after = A::add(after, tj);
                        else before = A::add(before, tj);
                    }
                }
                val = A::mul(alb, A::add(A::add(sp[c], after), before));
            }
            if (lane == 0) pn[c] = val;
            __syncwarp();
        }
        int test = 0;
        for (int c = lane; c < nf; c += 32) {
            const R d = A::sub(pn[c], po[c]);
            if ((d < R(0) ? -d : d) > acc) test = 1;
            po[c] = pn[c];
        }
        more = __any_sync(0xffffffffu, test) != 0;
        __syncwarp();
        ++it;
    }
    for (int c = lane; c < nf; c += 32) Efm[(size_t)c * ntau + s] = A::div(pn[c], alb);
}

// one Jacobi sweep: pn = alb (sp + sum_k v_k po[g_k]) for every (facet, step),
// [nf][ntau] arrays; *more = 1 if some |pn - po| > accuracy
__global__ void __launch_bounds__(256) k_multi_jacobi(DevSolve sv, const float* sp, const float* po, float* pn,
                                                      int* more) {
    const int nf = sv.nf, ntau = sv.ntau;
    const int f = blockIdx.y * blockDim.y + threadIdx.y;
    const int s = blockIdx.x * 32 + threadIdx.x;
    if (f >= nf) return;
    const bool ok = s < ntau;
    const int sc = ok ? s : 0;
    float a0 = 0.0f, a1 = 0.0f;
    const int k0 = sv.dep_ptr[f], k1 = sv.dep_ptr[f + 1];
    int k = k0;
    for (; k + 1 < k1; k += 2) {
        a0 += __ldg(&sv.dep_vf[k]) * po[(size_t)__ldg(&sv.dep_idx[k]) * ntau + sc];
        a1 += __ldg(&sv.dep_vf[k + 1]) * po[(size_t)__ldg(&sv.dep_idx[k + 1]) * ntau + sc];
    }
    if (k < k1) a0 += __ldg(&sv.dep_vf[k]) * po[(size_t)__ldg(&sv.dep_idx[k]) * ntau + sc];
    if (!ok) return;
    const size_t o = (size_t)f * ntau + s;
    const float v = sv.alb * (sp[o] + (a0 + a1));
    pn[o] = v;
    if (fabsf(v - po[o]) > sv.sacc) *more = 1;
}

__global__ void k_status_or(int* status, int bits) { atomicOr(status, bits); }

__global__ void __launch_bounds__(256) k_multi_jacobi_init(DevSolve sv, float* sp, float* po) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)sv.nf * sv.ntau) return;
    const float* cs = static_cast<const float*>(sv.cosil);
    sp[i] = sv.solar * cs[i] * (float)sv.shadow[i];
    po[i] = sv.alb * static_cast<const float*>(sv.Efm)[i];
}

__global__ void __launch_bounds__(256) k_multi_jacobi_out(DevSolve sv, const float* p) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)sv.nf * sv.ntau) return;
    static_cast<float*>(sv.Efm)[i] = p[i] / sv.alb;
}

// [nf][ntau] -> [ntau][nf]
template <class R>
__global__ void __launch_bounds__(256) k_forcing_t(const R* src, R* dst, int nf, int ntau) {
    __shared__ R sm[32][33];
    const int f0 = blockIdx.y * 32, s0 = blockIdx.x * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int f = f0 + j, s = s0 + threadIdx.x;
        sm[j][threadIdx.x] = (f < nf && s < ntau) ? src[(size_t)f * ntau + s] : R(0);
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int s = s0 + j, f = f0 + threadIdx.x;
        if (f < nf && s < ntau) dst[(size_t)s * nf + f] = sm[threadIdx.x][j];
    }
}

// [rows][cols] -> [cols][rows] with a type conversion, 32 x 32 tiles
template <class Ri, class Ro>
__global__ void __launch_bounds__(256) k_transpose(const Ri* src, Ro* dst, size_t rows, size_t cols) {
    __shared__ Ri sm[32][33];
    const size_t r0 = (size_t)blockIdx.y * 32, c0 = (size_t)blockIdx.x * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const size_t r = r0 + j, c = c0 + threadIdx.x;
        sm[j][threadIdx.x] = (r < rows && c < cols) ? src[r * cols + c] : Ri(0);
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const size_t c = c0 + j, r = r0 + threadIdx.x;
        if (r < rows && c < cols) dst[c * rows + r] = (Ro)sm[threadIdx.x][j];
    }
}

template <class R>
__global__ void k_set_forcing(DevSolve sv, const int32_t* shadow, const float* illum) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n = (size_t)sv.nf * sv.ntau;
    if (i >= n) return;
    sv.shadow[i] = shadow[i] ? 1 : 0;
    static_cast<R*>(sv.Efm)[i] = (R)illum[i];
}

// ------------------------------------------------------------------ launchers
int launch_single_scattering(const DevSolve& s, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    dim3 blk(32, 8), grd((s.ntau + 31) / 32, (s.nf + 7) / 8);
    switch (s.mode) {
        case MODE_REF: k_single_scatter<MODE_REF><<<grd, blk, 0, st>>>(s); break;
        case MODE_FP64: k_single_scatter<MODE_FP64><<<grd, blk, 0, st>>>(s); break;
        default: k_single_scatter<MODE_FAST><<<grd, blk, 0, st>>>(s); break;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

size_t multiple_scattering_work_bytes(const DevSolve& s) {
    const size_t rs = (s.mode == MODE_FP64) ? 8 : 4;
    return 3 * (size_t)s.ntau * s.nf * rs + 256;
}

namespace {
// FAST: Jacobi sweeps until no (facet, step) changes by more than the
// accuracy; one 4-byte read-back per sweep
int multiple_scattering_jacobi(const DevSolve& s, void* work, cudaStream_t st, int cap) {
    const size_t n = (size_t)s.nf * s.ntau;
    float* sp = static_cast<float*>(work);
    float* pa = sp + n;
    float* pb = pa + n;
    int* more = reinterpret_cast<int*>(pb + n);
    const int g1 = (int)((n + 255) / 256);
    k_multi_jacobi_init<<<g1, 256, 0, st>>>(s, sp, pa);
    dim3 blk(32, 8), grd((s.ntau + 31) / 32, (s.nf + 7) / 8);
    for (int it = 0;; ++it) {
        if (it == cap) {
            k_status_or<<<1, 1, 0, st>>>(s.status, ST_SCATTER_CAP);
            break;
        }
        cudaMemsetAsync(more, 0, 4, st);
        k_multi_jacobi<<<grd, blk, 0, st>>>(s, sp, pa, pb, more);
        int m = 0;
        if (cudaMemcpyAsync(&m, more, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess) return 2;
        if (cudaStreamSynchronize(st) != cudaSuccess) return 2;
        std::swap(pa, pb);
        if (!m) break;
    }
    k_multi_jacobi_out<<<g1, 256, 0, st>>>(s, pa);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}
}  // namespace

int launch_multiple_scattering(const DevSolve& s, void* work, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const int cap = 1000;  // the reference iterates unbounded; real cases need < 50 sweeps
    if (s.mode == MODE_FAST) return multiple_scattering_jacobi(s, work, st, cap);
    switch (s.mode) {
        case MODE_REF: k_multi_gs<MODE_REF><<<s.ntau, 32, 0, st>>>(s, work, cap); break;
        case MODE_FP64: k_multi_gs<MODE_FP64><<<s.ntau, 32, 0, st>>>(s, work, cap); break;
        default: k_multi_gs<MODE_FAST><<<s.ntau, 32, 0, st>>>(s, work, cap); break;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_forcing_transpose(const DevSolve& s, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    dim3 blk(32, 8), grd((s.ntau + 31) / 32, (s.nf + 31) / 32);
    if (s.mode == MODE_FP64)
        k_forcing_t<double><<<grd, blk, 0, st>>>(static_cast<const double*>(s.Efm), static_cast<double*>(s.E), s.nf, s.ntau);
    else
        k_forcing_t<float><<<grd, blk, 0, st>>>(static_cast<const float*>(s.Efm), static_cast<float*>(s.E), s.nf, s.ntau);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_transpose(const void* src, int src_bytes, void* dst, int dst_bytes, size_t rows, size_t cols,
                     stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    dim3 blk(32, 8), grd((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
    if (src_bytes == 4 && dst_bytes == 4)
        k_transpose<float, float><<<grd, blk, 0, st>>>(static_cast<const float*>(src), static_cast<float*>(dst), rows, cols);
    else if (src_bytes == 8 && dst_bytes == 8)
        k_transpose<double, double><<<grd, blk, 0, st>>>(static_cast<const double*>(src), static_cast<double*>(dst), rows, cols);
    else if (src_bytes == 4 && dst_bytes == 8)
        k_transpose<float, double><<<grd, blk, 0, st>>>(static_cast<const float*>(src), static_cast<double*>(dst), rows, cols);
    else if (src_bytes == 8 && dst_bytes == 4)
        k_transpose<double, float><<<grd, blk, 0, st>>>(static_cast<const double*>(src), static_cast<float*>(dst), rows, cols);
    else
        return 1;
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_set_forcing(const DevSolve& s, const int32_t* shadow_d, const float* illum_d, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const size_t n = (size_t)s.nf * s.ntau;
    const int g = (int)((n + 255) / 256);
    if (s.mode == MODE_FP64) k_set_forcing<double><<<g, 256, 0, st>>>(s, shadow_d, illum_d);
    else k_set_forcing<float><<<g, 256, 0, st>>>(s, shadow_d, illum_d);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}


// --------------------------------------------------------- no-allocation variant
// Scattered sunlight over caller-owned device buffers for callers that cannot
// allocate device memory themselves or through this library: code running
// where cudaMalloc is unavailable or forbidden (inside a framework that owns
// every device allocation through its own pool, or a host loop that must not
// trigger allocator synchronisation).  The Gauss-Seidel work arrays live in a
// fixed file-scope device array instead of a per-call allocation.
//
//  * Limit: nf * ntau <= ATPM_NOALLOC_MAX_CELLS (2^20 cells, 12 MiB of
//    scratch); larger problems are rejected with ATPM_E_UNSUPPORTED.  Every
//    GPU that loads the library reserves this array until the process exits.
//  * The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress, with that device current; make that first call
//    before any stream capture on the device.
//  * All calls share the one array: calls whose work overlaps on the GPU
//    (different streams, or different host threads) race and corrupt each
//    other's results.  Serialise them.
//  * The array keeps the previous call's contents; every cell a call reads is
//    written by that call first (the status word is cleared by each call).
namespace {
constexpr size_t kNoAllocMaxCells = size_t(1) << 20;
constexpr size_t kNoAllocStatusSlot = 3 * kNoAllocMaxCells;  // one int after the three arrays
constexpr int kNoAllocMaxFacets = 8 * 65535;  // grid.y of the single-scattering launch is nf / 8
static __device__ __align__(256) float g_noalloc_scratch[3 * kNoAllocMaxCells + 64];

std::mutex g_noalloc_mu;
void* g_noalloc_addr[256] = {};  // per-device address of g_noalloc_scratch

int noalloc_scratch(void** out, int* device, char* err, size_t errlen) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        std::snprintf(err, errlen, "cudaGetDevice: %s", cudaGetErrorString(e));
        return 1;
    }
    if (dev < 0 || dev >= 256) {
        std::snprintf(err, errlen, "device ordinal %d out of range", dev);
        return 1;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            std::snprintf(err, errlen, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
            return 1;
        }
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    *device = dev;
    return 0;
}
}  // namespace

void set_last_error(const char* msg);

}  // namespace atpm

extern "C" ATPM_API atpm_status atpm_scattering_noalloc(
    int32_t nf, int32_t ntau, const int32_t* dep_ptr, const int32_t* dep_idx, const float* dep_vf,
    const float* cosillum, const uint8_t* shadow, float solar, float albedo, float scattering_accuracy,
    int32_t multiple, float* illumination, int32_t* status, void* stream) {
    using namespace atpm;
    char err[256];
    if (nf < 1 || ntau < 1 || !dep_ptr || !dep_idx || !dep_vf || !cosillum || !shadow || !illumination) {
        set_last_error("scattering_noalloc: bad arguments (every array, dep_idx and dep_vf included, must be a "
                       "device pointer)");
        return ATPM_E_INVALID;
    }
    if (multiple && !status) {
        set_last_error("scattering_noalloc: multiple scattering needs a status word (the Gauss-Seidel cap is "
                       "reported there)");
        return ATPM_E_INVALID;
    }
    if (nf > kNoAllocMaxFacets) {
        std::snprintf(err, sizeof err, "scattering_noalloc: nf = %d exceeds %d facets (launch grid limit)", nf,
                      kNoAllocMaxFacets);
        set_last_error(err);
        return ATPM_E_UNSUPPORTED;
    }
    if ((size_t)nf * (size_t)ntau > kNoAllocMaxCells) {
        std::snprintf(err, sizeof err,
                      "scattering_noalloc: nf*ntau = %lld exceeds the fixed scratch of %lld cells; "
                      "use atpm_scattering",
                      (long long)nf * ntau, (long long)kNoAllocMaxCells);
        set_last_error(err);
        return ATPM_E_UNSUPPORTED;
    }
    void* scratch = nullptr;
    int dev = 0;
    if (noalloc_scratch(&scratch, &dev, err, sizeof err)) {
        set_last_error(err);
        return ATPM_E_CUDA;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int* st_word = status ? status : reinterpret_cast<int*>(static_cast<float*>(scratch) + kNoAllocStatusSlot);
    if (!status) {
        cudaError_t e = cudaMemsetAsync(st_word, 0, sizeof(int), st);
        if (e != cudaSuccess) {
            std::snprintf(err, sizeof err, "scattering_noalloc: %s", cudaGetErrorString(e));
            set_last_error(err);
            return ATPM_E_CUDA;
        }
    }
    DevSolve sv{};
    sv.nf = nf;
    sv.ntau = ntau;
    sv.mode = MODE_REF;
    sv.dep_ptr = dep_ptr;
    sv.dep_idx = dep_idx;
    sv.dep_vf = dep_vf;
    sv.nnz = 0;
    sv.shadow = const_cast<uint8_t*>(shadow);
    sv.cosil = const_cast<float*>(cosillum);
    sv.Efm = illumination;
    sv.status = st_word;
    sv.solar = solar;
    sv.alb = albedo;
    sv.sacc = scattering_accuracy;
    dim3 blk(32, 8), grd((ntau + 31) / 32, (nf + 7) / 8);
    k_single_scatter<MODE_REF><<<grd, blk, 0, st>>>(sv);
    if (multiple) k_multi_gs<MODE_REF><<<ntau, 32, 0, st>>>(sv, scratch, 1000);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        std::snprintf(err, sizeof err, "scattering_noalloc launch: %s", cudaGetErrorString(e));
        set_last_error(err);
        return ATPM_E_CUDA;
    }
    return ATPM_OK;
}
