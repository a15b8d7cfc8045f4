// Block-sparse self-heating flux on the 5th-generation tensor cores (FAST
// precision).  The reference sums Q_f = sum_g eps sigma T_g^4 V_fg over each
// facet's view-factor list (3905/Thermal/NominalPole/main.cpp:1519-1529); with
// previous-revolution temperatures the whole revolution is one product
//
//     Q[s][f] = sum_g V[f][g] * (W_hi[s][g] + W_lo[s][g])
//
// with W = eps sigma T^4 split into two BF16 parts (W_hi = bf16(W),
// W_lo = bf16(W - W_hi): a 16-bit significand, so the flux does not jitter
// from one revolution to the next by more than ~1e-5 relative) and V in BF16.
// Tiles holding a view factor >= 1e-4 (neighbours in concavities, where one
// entry can carry a third of a facet's flux) also keep V_lo = bf16(V - V_hi)
// and get a third product V_lo * W_hi.  Accumulation is FP32 in TMEM.
// Row blocks whose 128 facets are all frozen (reference freeze protocol)
// are skipped: their flux is not read.
//
// Only the dense part of V goes to the tensor cores: a (128-facet row block,
// 64-facet column block) cell becomes a tile when it holds at least
// ATPM_TC_MIN_ENTRIES list entries (32).  The entries of sparser cells (1 %
// of the binary's entries, in 68 % of its cells: facets of one body seeing
// each other across its relief) are the sparse remainder, summed in FP32 by
// k_spmm_rem against W32 (eps sigma T^4 facet-major, written by the
// conduction sweep beside the BF16 tiles) and added to the tiles' Q.
//
// V is stored as 128 x 64 BF16 tiles (block-sparse rows: every 128-facet row
// block keeps the 64-facet column blocks it has tiles in; one set per shape,
// shared by clones) and W as 64-facet x N-step tiles (per solve, written by
// the conduction sweep).  Both are laid out in HBM already in the
// 128-byte-swizzled K-major form the tensor core reads, so each tile moves
// with one bulk copy (cp.async.bulk) into a shared-memory stage ring.  The
// product kernel is persistent (one CTA per SM) and warp-specialised: a
// producer warp takes work items (row block x step chunk) by ticket from the
// list k_tc_compact builds before each launch and streams their tiles, an MMA
// warp issues tcgen05.mma (M = 128, N = step chunk, K = 16) into one of two
// TMEM accumulators, and four epilogue warps drain the other with
// tcgen05.ld and write Q coalesced along facets.  All-zero 16-wide K slices
// of a tile are not issued.
//
// Every mbarrier wait is bounded (about one second of clock cycles); a
// timeout sets ST_TC_TIMEOUT in the solve's status word and the roles stop,
// let their copies and products land and free TMEM instead of spinning.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <cstdint>

#include "atpm_internal.h"

namespace atpm {

namespace {

constexpr int TC_M = 128;        // facets per row block (TMEM lanes)
constexpr int TC_K = 64;         // facets per column block (one 128-byte swizzle row of BF16)
constexpr int TC_STAGES = 4;   // upper bound; the ring depth follows the stage size
constexpr long long WAIT_CYCLES = 2000000000LL;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// bounded wait: false after `limit` clock cycles
__device__ __forceinline__ bool mbar_wait_lim(uint64_t* bar, uint32_t parity, long long limit) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > limit) return false;
    }
    return true;
}

// bounded wait of the product pipeline: false after ~1 s
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    return mbar_wait_lim(bar, parity, WAIT_CYCLES);
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tc_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tc_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(accum)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (tcgen05 descriptor version 1)
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;                  // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024u >> 4) << 32;       // stride byte offset
    d |= (uint64_t)1 << 46;                  // descriptor version
    d |= (uint64_t)2 << 61;                  // SWIZZLE_128B
    return d;
}

// instruction descriptor: D f32, A/B bf16, both K-major, M = 128, N = n
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
}

// ring depth: as many stages (<= 4) as fit in 220 KB of shared memory;
// a stage holds A_hi, A_lo (16 KB each) and B_hi, B_lo (N x 128 B each)
__host__ __device__ inline int tc_stages(int N) {
    const int stage = (TC_M * TC_K * 4 + N * TC_K * 4 + 1023) & ~1023;
    const int s = (220 * 1024) / stage;
    return s < TC_STAGES ? s : TC_STAGES;
}

}  // namespace

int tc_max_chunk() { return 160; }

// float -> BF16, round to nearest even (quiet NaN for NaN), as the host's f2bf
__device__ __forceinline__ uint16_t bf16_rne(float x) {
    uint32_t u = __float_as_uint(x);
    if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

// tile structure from the uploaded lists, one warp per facet row: for every
// (128-facet row block, 64-facet column block) cell the largest |view
// factor| (its float bits + 1, so 0 marks an empty cell: max, or and add do
// not depend on the order the entries arrive in), the mask of 16-wide K
// slices holding an entry and the number of entries
__global__ void __launch_bounds__(256) k_tc_cells(DevSolve s, int nkb, unsigned* cmax, unsigned* cmask,
                                                  unsigned* count) {
    const int f = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (f >= s.nf) return;
    const size_t row = (size_t)(f >> 7) * nkb;
    for (int k = s.dep_ptr[f] + lane; k < s.dep_ptr[f + 1]; k += 32) {
        const int g = s.dep_idx[k];
        const size_t cell = row + (size_t)(g >> 6);
        atomicMax(&cmax[cell], __float_as_uint(fabsf(s.dep_vf[k])) + 1u);
        atomicOr(&cmask[cell], 1u << ((g & 63) >> 4));
        atomicAdd(&count[cell], 1u);
    }
}

int launch_tc_cells(const DevSolve& s, int nkb, unsigned* cmax, unsigned* cmask, unsigned* count, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const size_t threads = (size_t)s.nf * 32;
    k_tc_cells<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(s, nkb, cmax, cmask, count);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// Which tiles need the residual V_lo for the rows they serve.  BF16 rounding
// of V is correlated between neighbouring entries of a smooth surface, so in
// a row's flux its error can approach 2^-9 of the mass it applies to.  A warp
// per facet row sums the row's |view factor| per 64-facet column block in
// shared memory (fixed point, 2^-36 units, plus one unit per entry so a
// touched block is never zero: the sums do not depend on the order of the
// additions); a block holding at least 1 % of the row's mean per touched
// block marks its tile.  The blocks left unmarked hold less than 1 % of the
// row's view-factor mass between them.
__global__ void k_tc_rowneed(DevSolve s, int nkb, unsigned* need) {
    extern __shared__ unsigned long long mass_sm[];
    const int warps = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < warps * nkb; i += blockDim.x) mass_sm[i] = 0ull;
    __syncthreads();
    const int f = blockIdx.x * warps + warp;
    if (f >= s.nf) return;  // warp-uniform; no block barrier follows
    unsigned long long* m = mass_sm + (size_t)warp * nkb;
    const int k0 = s.dep_ptr[f], k1 = s.dep_ptr[f + 1];
    unsigned long long tot = 0;
    unsigned touched = 0;
    for (int k = k0 + lane; k < k1; k += 32) {
        const unsigned long long q = __double2ull_rn((double)fabsf(s.dep_vf[k]) * 68719476736.0) + 1ull;
        if (atomicAdd(&m[s.dep_idx[k] >> 6], q) == 0ull) ++touched;
        tot += q;
    }
    for (int o = 16; o > 0; o >>= 1) {
        tot += __shfl_xor_sync(0xffffffffu, tot, o);
        touched += __shfl_xor_sync(0xffffffffu, touched, o);
    }
    __syncwarp();
    unsigned* row = need + (size_t)(f >> 7) * nkb;
    for (int k = k0 + lane; k < k1; k += 32) {
        const int kb = s.dep_idx[k] >> 6;
        if (100ull * touched * m[kb] >= tot) atomicOr(&row[kb], 1u);
    }
}

// 0: launched; 1: the row maps do not fit shared memory (very large shapes:
// the caller keeps the absolute rule alone); 2: launch error
int launch_tc_rowneed(const DevSolve& s, int nkb, unsigned* need, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const size_t per_warp = (size_t)nkb * 8;
    constexpr size_t kMax = 200 * 1024;
    if (per_warp > kMax) return 1;
    int warps = (int)std::min<size_t>(8, kMax / per_warp);
    const size_t smem = per_warp * warps;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k_tc_rowneed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return 2;
    k_tc_rowneed<<<(unsigned)((s.nf + warps - 1) / warps), warps * 32, smem, st>>>(s, nkb, need);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// one warp per facet row: every list entry of a kept tile goes to its
// swizzled slot of its (row block, column block) tile, plus the BF16 residual
// where the tile has one; entries of cells without a tile (slot -1) belong to
// the sparse remainder
__global__ void __launch_bounds__(256) k_tc_fill(DevSolve s, int nkb, const int* slot, const int* lo_of,
                                                 uint16_t* tiles, uint16_t* lo_tiles) {
    const int f = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (f >= s.nf) return;
    const int* srow = slot + (size_t)(f >> 7) * nkb;
    const uint32_t row = (uint32_t)(f & 127);
    for (int k = s.dep_ptr[f] + lane; k < s.dep_ptr[f + 1]; k += 32) {
        const int g = s.dep_idx[k];
        const float v = s.dep_vf[k];
        const int t = srow[g >> 6];
        if (t < 0) continue;
        const uint32_t off = swz(row, (uint32_t)(g & 63));
        const uint16_t hb = bf16_rne(v);
        tiles[(size_t)t * (TC_M * TC_K) + off] = hb;
        const int l = lo_of[t];
        if (l >= 0) lo_tiles[(size_t)l * (TC_M * TC_K) + off] = bf16_rne(__fsub_rn(v, __uint_as_float((uint32_t)hb << 16)));
    }
}

int launch_tc_fill(const DevSolve& s, int nkb, const int* slot, const int* lo_of, void* tiles, void* lo_tiles,
                   stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const size_t threads = (size_t)s.nf * 32;
    k_tc_fill<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(s, nkb, slot, lo_of, static_cast<uint16_t*>(tiles),
                                                                   static_cast<uint16_t*>(lo_tiles));
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// The sparse remainder's lists from the uploaded view-factor lists and the
// tile slot table (-1: the cell has no tile), a warp per facet row: first
// the number of each row's entries in cells without a tile, then (after
// the caller's scan into rptr) the entries themselves, in list order.
__global__ void __launch_bounds__(256) k_rem_count(DevSolve s, int nkb, const int* slot, int* count) {
    const int f = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (f >= s.nf) return;
    const int* srow = slot + (size_t)(f >> 7) * nkb;
    int n = 0;
    for (int k = s.dep_ptr[f] + lane; k < s.dep_ptr[f + 1]; k += 32) n += srow[s.dep_idx[k] >> 6] < 0 ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
    if (lane == 0) count[f] = n;
}

__global__ void __launch_bounds__(256) k_rem_fill(DevSolve s, int nkb, const int* slot, const int* rptr, int* ridx,
                                                  float* rvf, uint8_t* rrow) {
    const int f = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (f >= s.nf) return;  // warp-uniform
    const int* srow = slot + (size_t)(f >> 7) * nkb;
    int out = rptr[f];
    const int k0 = s.dep_ptr[f], k1 = s.dep_ptr[f + 1];
    for (int kb = k0; kb < k1; kb += 32) {
        const int k = kb + lane;
        const bool take = k < k1 && srow[s.dep_idx[k] >> 6] < 0;
        const unsigned m = __ballot_sync(0xffffffffu, take);
        if (take) {
            const int o = out + __popc(m & ((1u << lane) - 1u));
            ridx[o] = s.dep_idx[k];
            rvf[o] = s.dep_vf[k];
            rrow[o] = (uint8_t)(f & 127);
        }
        out += __popc(m);
    }
}

int launch_rem_count(const DevSolve& s, int nkb, const int* slot, int* count, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const size_t threads = (size_t)s.nf * 32;
    k_rem_count<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(s, nkb, slot, count);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_rem_fill(const DevSolve& s, int nkb, const int* slot, const int* rptr, int* ridx, float* rvf, uint8_t* rrow,
                    stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const size_t threads = (size_t)s.nf * 32;
    k_rem_fill<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(s, nkb, slot, rptr, ridx, rvf, rrow);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// Work items whose row block has an active facet, compacted before every
// launch (in map order within each warp), so tickets are spent on work only.
__global__ void __launch_bounds__(128) k_tc_compact(Batch b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool use = false;
    int4 it = make_int4(0, 0, 0, 0);
    if (i < b.nq) {
        it = b.qmap[i];
        const DevSolve& sv = b.tab[it.x];
        const bool everyone = !sv.freeze || sv.ti == 0.0f;
        use = sv.ctl->active && sv.tc_tiles && (everyone || sv.rb_act[it.y]);
    }
    const unsigned m = __ballot_sync(0xffffffffu, use);
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(&b.tc_work[0], __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (use) b.tc_list[base + __popc(m & ((1u << lane) - 1u))] = it;
}

// Persistent, warp-specialised: one CTA per SM.  Work items are handed out
// dynamically: the producer takes the next ticket of the launch's counter
// over the compacted list and queues the item in a small shared-memory queue
// read by the other roles; a ticket past the end queues the stop item.
//   warp 0, lane 0   producer: tickets, the item queue, and bulk copies of
//                    each tile's V_hi (+ V_lo) and W chunk into the stage
//                    ring, across item boundaries
//   warp 1, lane 0   MMA issuer: per item, into TMEM accumulator buffer
//                    (item & 1), then tcgen05.commit -> tfull[buffer]
//   warps 2-5        epilogue: TMEM quadrant (warp & 3) -> Q, then arrive on
//                    tempty[buffer]; the issuer's next-but-one item waits on it
// Every item's products accumulate in the single-item order, so Q does not
// depend on which CTA computed it.
constexpr int TC_THREADS = 192;
constexpr int TC_QUEUE = 4;  // queued work items
// Tiles accumulated in TMEM before the partial sum goes to Q: the tensor
// core's FP32 accumulation of long runs of positive products drifts low
// (measured -1.9e-5 relative on rows of ~3,700 entries summed in one
// accumulator, -1.0e-5 with 64-tile segments, -4.4e-6 with 32), so a work
// item is summed in segments of this many tiles, each a fresh accumulator,
// and the epilogue adds the segments into Q in order with round-to-nearest.
constexpr int TC_SEG = 64;

__global__ void __launch_bounds__(TC_THREADS, 1) k_spmm_tc(Batch b) {
    extern __shared__ __align__(1024) unsigned char dyn[];
    __shared__ __align__(8) uint64_t full[TC_STAGES], empty[TC_STAGES], tfull[2], tempty[2], fin;
    __shared__ __align__(8) uint64_t qfull[TC_QUEUE], qempty[TC_QUEUE];
    __shared__ int4 qitem[TC_QUEUE];
    __shared__ uint32_t tmem_base;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // one stage layout for the launch, sized for the largest chunk of the batch
    const int Nmax = b.tc_nmax;
    const uint32_t a_bytes = TC_M * TC_K * 2;
    const uint32_t stage_bytes = (2 * a_bytes + (uint32_t)Nmax * TC_K * 2 * 2 + 1023) & ~1023u;
    int S = (b.tc_stages > 0 && b.tc_stages < tc_stages(Nmax)) ? b.tc_stages : tc_stages(Nmax);
    {
        uint32_t dsz;
        asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dsz));
        const int fit = (int)((dsz - 1024u) / stage_bytes);
        if (S > fit) S = fit;
    }
    unsigned char* base = dyn + ((1024u - (smem_u32(dyn) & 1023u)) & 1023u);
    constexpr uint32_t kBufCols = 256;  // TMEM columns per accumulator buffer (N <= 256)
    if (warp == 0) {
        tc_alloc(&tmem_base, 2 * kBufCols);
        tc_relinquish();
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < TC_STAGES; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&tfull[i], 1);
            mbar_init(&tempty[i], 4);  // one arrival per epilogue warp
        }
        for (int i = 0; i < TC_QUEUE; ++i) {
            mbar_init(&qfull[i], 1);
            mbar_init(&qempty[i], 5);  // the issuer and the four epilogue warps
        }
        mbar_init(&fin, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    int* status0 = b.tab[0].status;  // where a timeout is reported when no item is at hand

    if (threadIdx.x == 0) {
        // ------------------------------------------------------------ producer
        uint32_t slot = 0, ph = 0, qs = 0, qph = 0;
        int last_ph[TC_STAGES];  // parity of each stage's last fill (-1: never filled)
#pragma unroll
        for (int i = 0; i < TC_STAGES; ++i) last_ph[i] = -1;
        bool ok = true;
        const int nlist = b.tc_work[0];
        for (;;) {
            const int g = atomicAdd(&b.tc_work[1], 1);
            const bool stop = g >= nlist;
            const int4 it = stop ? make_int4(-1, 0, 0, 0) : b.tc_list[g];
            const int tall = stop ? 0 : b.tab[it.x].tc_ptr[it.y + 1] - b.tab[it.x].tc_ptr[it.y];
            const int nseg = stop ? 1 : max(1, (tall + TC_SEG - 1) / TC_SEG);
            for (int seg = 0; seg < nseg && ok; ++seg) {
                // queue the item's segment (or the stop item)
                if (!mbar_wait(&qempty[qs], qph ^ 1u)) { ok = false; break; }
                qitem[qs] = make_int4(it.x, it.y, it.z, seg);
                mbar_arrive(&qfull[qs]);
                if (++qs == TC_QUEUE) { qs = 0; qph ^= 1u; }
                if (stop) break;
                const DevSolve& sv = b.tab[it.x];
                const int N = sv.tc_n, c = it.z;
                const int t0 = sv.tc_ptr[it.y] + seg * TC_SEG, T = min(TC_SEG, tall - seg * TC_SEG);
                const uint32_t b_bytes = (uint32_t)N * TC_K * 2 * 2;
                const __nv_bfloat16* tiles = static_cast<const __nv_bfloat16*>(sv.tc_tiles);
                const __nv_bfloat16* lo_tiles = static_cast<const __nv_bfloat16*>(sv.tc_lo_tiles);
                const __nv_bfloat16* Wb = static_cast<const __nv_bfloat16*>(sv.Wb);
                for (int i = 0; i < T; ++i) {
                    if (!mbar_wait(&empty[slot], ph ^ 1u)) { ok = false; break; }
                    unsigned char* sa = base + (size_t)slot * stage_bytes;
                    const int kb = sv.tc_col[t0 + i] & 0xffffff;
                    const int lo = sv.tc_lo[t0 + i];
                    mbar_expect_tx(&full[slot], a_bytes + (lo >= 0 ? a_bytes : 0u) + b_bytes);
                    bulk_g2s(sa, tiles + (size_t)(t0 + i) * (TC_M * TC_K), a_bytes, &full[slot]);
                    if (lo >= 0) bulk_g2s(sa + a_bytes, lo_tiles + (size_t)lo * (TC_M * TC_K), a_bytes, &full[slot]);
                    bulk_g2s(sa + 2 * a_bytes, Wb + ((size_t)kb * sv.tc_nchunks + c) * (size_t)2 * N * TC_K, b_bytes,
                             &full[slot]);
                    last_ph[slot] = (int)ph;
                    if (++slot == (uint32_t)S) { slot = 0; ph ^= 1u; }
                }
            }
            if (!ok || stop) break;
        }
        if (!ok) atomicOr(status0, ST_TC_TIMEOUT);
        // copies still in flight exist only after a timeout: let them land
#pragma unroll
        for (int i = 0; i < TC_STAGES; ++i)
            if (last_ph[i] >= 0) mbar_wait(&full[i], (uint32_t)last_ph[i]);
    } else if (threadIdx.x == 32) {
        // ---------------------------------------------------------- MMA issuer
        uint32_t slot = 0, ph = 0, qs = 0, qph = 0, item_no = 0;
        bool ok = true;
        for (;;) {
            if (!mbar_wait(&qfull[qs], qph)) { ok = false; break; }
            const int4 w = qitem[qs];
            if (w.x < 0) break;
            const DevSolve& sv = b.tab[w.x];
            const int N = sv.tc_n;
            const int tall = sv.tc_ptr[w.y + 1] - sv.tc_ptr[w.y];
            const int t0 = sv.tc_ptr[w.y] + w.w * TC_SEG, T = max(0, min(TC_SEG, tall - w.w * TC_SEG));
            const uint32_t b_bytes = (uint32_t)N * TC_K * 2 * 2;
            const uint32_t ab = item_no & 1u, use_no = item_no >> 1;
            if (!mbar_wait(&tempty[ab], (use_no & 1u) ^ 1u)) { ok = false; break; }
            tc_fence_after();
            const uint32_t d = tmem + ab * kBufCols;
            const uint32_t idesc = idesc_bf16(N);
            uint32_t acc = 0u;  // the first product issued overwrites the accumulator
            for (int i = 0; i < T && ok; ++i) {
                if (!mbar_wait(&full[slot], ph)) { ok = false; break; }
                tc_fence_after();
                const uint32_t sa = smem_u32(base + (size_t)slot * stage_bytes);
                const uint64_t ad = sw128_desc(sa), al = sw128_desc(sa + a_bytes);
                const uint64_t bh = sw128_desc(sa + 2 * a_bytes), bl = sw128_desc(sa + 2 * a_bytes + b_bytes / 2);
                const bool has_lo = sv.tc_lo[t0 + i] >= 0;
                // K slices without an entry are zero in both A tiles: their
                // products would add exact zeros, so they are not issued
                const uint32_t kmask = (uint32_t)sv.tc_col[t0 + i] >> 24;
#pragma unroll
                for (int kk = 0; kk < TC_K / 16; ++kk) {
                    if (!((kmask >> kk) & 1u)) continue;
                    tc_mma(d, ad + (uint64_t)(2 * kk), bh + (uint64_t)(2 * kk), idesc, acc);
                    tc_mma(d, ad + (uint64_t)(2 * kk), bl + (uint64_t)(2 * kk), idesc, 1u);
                    if (has_lo) tc_mma(d, al + (uint64_t)(2 * kk), bh + (uint64_t)(2 * kk), idesc, 1u);
                    acc = 1u;
                }
                tc_commit(&empty[slot]);
                if (++slot == (uint32_t)S) { slot = 0; ph ^= 1u; }
            }
            if (!ok) break;
            tc_commit(&tfull[ab]);  // this item's products complete -> epilogue
            mbar_arrive(&qempty[qs]);
            if (++qs == TC_QUEUE) { qs = 0; qph ^= 1u; }
            ++item_no;
        }
        if (!ok) atomicOr(status0, ST_TC_TIMEOUT);
        tc_commit(&fin);  // every product issued by this thread has completed
        mbar_wait(&fin, 0);
    } else if (warp >= 2) {
        // ------------------------------------------------------------ epilogue
        const int q = warp & 3;  // TMEM lanes q * 32 .. q * 32 + 31
        uint32_t qs = 0, qph = 0, item_no = 0;
        for (;;) {
            if (!__all_sync(0xffffffffu, mbar_wait(&qfull[qs], qph))) {
                if (lane == 0) atomicOr(status0, ST_TC_TIMEOUT);
                break;
            }
            const int4 w = qitem[qs];
            if (w.x < 0) break;
            const DevSolve& sv = b.tab[w.x];
            const int N = sv.tc_n, nf = sv.nf, ntau = sv.ntau, nc = w.z;
            const int T = sv.tc_ptr[w.y + 1] - sv.tc_ptr[w.y];
            float* Q = static_cast<float*>(sv.Q);
            const uint32_t ab = item_no & 1u, use_no = item_no >> 1;
            if (!__all_sync(0xffffffffu, mbar_wait(&tfull[ab], use_no & 1u))) {
                if (lane == 0) atomicOr(sv.status, ST_TC_TIMEOUT);
                break;
            }
            tc_fence_after();
            const int f = w.y * TC_M + q * 32 + lane;
            if (T == 0) {  // no tile in this row block
                if (f < nf)
                    for (int n = 0; n < N; ++n) {
                        const int s = nc * N + n;
                        if (s < ntau) Q[(size_t)s * nf + f] = 0.0f;
                    }
            } else {
                // the first segment stores, later ones add to Q in order
                // (round to nearest); a batch's 16 loads all issue before
                // its stores
                const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + ab * kBufCols;
                for (int c0 = 0; c0 < N; c0 += 16) {
                    float v[16];
                    tc_ld16(tbase + (uint32_t)c0, v);
                    if (f < nf) {
                        float prev[16];
#pragma unroll
                        for (int j = 0; j < 16; ++j) {
                            const int s = nc * N + c0 + j;
                            prev[j] = (w.w > 0 && c0 + j < N && s < ntau) ? __ldcg(&Q[(size_t)s * nf + f]) : 0.0f;
                        }
#pragma unroll
                        for (int j = 0; j < 16; ++j) {
                            const int s = nc * N + c0 + j;
                            if (c0 + j < N && s < ntau) Q[(size_t)s * nf + f] = w.w == 0 ? v[j] : prev[j] + v[j];
                        }
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&tempty[ab]);
                mbar_arrive(&qempty[qs]);
            }
            if (++qs == TC_QUEUE) { qs = 0; qph ^= 1u; }
            ++item_no;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tmem, 2 * kBufCols);
}

size_t spmm_tc_smem_bytes(int N, int stages) {
    const size_t a = TC_M * TC_K * 2 * 2, bb = (size_t)N * TC_K * 2 * 2;
    const int S = (stages > 0 && stages < tc_stages(N)) ? stages : tc_stages(N);
    return (size_t)S * ((a + bb + 1023) & ~(size_t)1023) + 1024;
}

int tc_max_stages(int N) { return tc_stages(N); }

// The sparse remainder of the product: the list entries of the cells too
// sparse for a tensor-core tile, added to the tiles' Q in FP32.  One CTA per
// (solve, 128-facet row block, 32-step chunk), lane j of every warp on step
// s0 + j, so each entry is one coalesced 128-byte load of its column facet's
// W32 row.  The block's entries (rows in order, each row's in list order)
// are cut into four contiguous ranges, one per warp; a warp reads 32
// entries' column, value and row at once and keeps eight W32 loads in
// flight across row boundaries, so the gather is not a chain of dependent
// loads per row (a row holds ~3 remainder entries on average).  A row's sum
// is the multiply-add chain over its entries in list order within each
// warp's range; a row split between warps adds the warps' partial sums in
// warp order after a barrier.  The block's 128 x 32 sums go through shared
// memory into the remainder's own array (along facets, coalesced), which
// k_rem_add adds to Q once the tensor-core product is complete.  Row blocks the
// tensor-core product skips (all facets frozen) are skipped alike.
// Earlier forms, a warp per facet row (one dependent index-then-W32 chain
// per row: 1.80 ms for the product per batch revolution of the 8-inertia
// binary), the same with the block's entries staged in shared memory first
// (1.93 ms) and one CTA per row block looping over the chunks (2.43 ms),
// were latency-bound.
constexpr int REM_STEPS = 32;
constexpr int REM_WARPS = 4;
constexpr int REM_INFLIGHT = 8;

__global__ void __launch_bounds__(REM_WARPS * 32) k_spmm_rem(Batch b) {
    const DevSolve& sv = b.tab[blockIdx.z];
    const int rb = blockIdx.x, s0 = blockIdx.y * REM_STEPS;
    const int nf = sv.nf, ntau = sv.ntau;
    if (!sv.rem_ptr || rb * 128 >= nf || s0 >= ntau || !sv.ctl->active) return;
    const bool everyone = !sv.freeze || sv.ti == 0.0f;
    if (!everyone && !sv.rb_act[rb]) return;
    const int f_lo = rb * 128, f_hi = min(nf, f_lo + 128);
    const int e0 = __ldg(&sv.rem_ptr[f_lo]), e1 = __ldg(&sv.rem_ptr[f_hi]);
    if (e0 == e1) return;  // no remainder entry in this block
    __shared__ float acc[128][REM_STEPS + 1];
    __shared__ float edge[REM_WARPS][REM_STEPS];
    __shared__ int edge_row[REM_WARPS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < 128 * (REM_STEPS + 1); i += blockDim.x) (&acc[0][0])[i] = 0.0f;
    __syncthreads();
    const float* W32 = sv.W32;
    const size_t ld = (size_t)sv.w32_ld;
    const int s = s0 + lane;  // W32 rows are padded to the chunk grid: s < w32_ld
    const int n = e1 - e0;
    const int a0 = e0 + (int)(((long long)n * warp) / REM_WARPS);
    const int a1 = e0 + (int)(((long long)n * (warp + 1)) / REM_WARPS);
    // the warp's first row goes to its edge slot, every later row (which
    // starts inside this range) straight to acc
    int cur = -1;
    bool first = true;
    float a = 0.0f;
    if (lane == 0) edge_row[warp] = -1;
    for (int kb = a0; kb < a1; kb += 32) {
        const int k = kb + lane;
        const bool in = k < a1;
        const int gk = in ? __ldg(&sv.rem_idx[k]) : 0;
        const float vk = in ? __ldg(&sv.rem_vf[k]) : 0.0f;
        const int rk = in ? (int)__ldg(&sv.rem_row[k]) : 0;
        const int cnt = min(32, a1 - kb);
        for (int j0 = 0; j0 < cnt; j0 += REM_INFLIGHT) {
            float w[REM_INFLIGHT];
#pragma unroll
            for (int u = 0; u < REM_INFLIGHT; ++u) {
                const int g = __shfl_sync(0xffffffffu, gk, (j0 + u) & 31);
                w[u] = (j0 + u < cnt) ? W32[(size_t)g * ld + s] : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < REM_INFLIGHT; ++u) {
                const float v = __shfl_sync(0xffffffffu, vk, (j0 + u) & 31);
                const int r = __shfl_sync(0xffffffffu, rk, (j0 + u) & 31);
                if (j0 + u < cnt) {
                    if (r != cur) {  // warp-uniform: the entry's row is the same on every lane
                        if (cur >= 0) {
                            if (first) {
                                edge[warp][lane] = a;
                                if (lane == 0) edge_row[warp] = cur;
                                first = false;
                            } else {
                                acc[cur][lane] = a;
                            }
                        }
                        cur = r;
                        a = 0.0f;
                    }
                    a = fmaf(v, w[u], a);
                }
            }
        }
    }
    if (cur >= 0) {
        if (first) {
            edge[warp][lane] = a;
            if (lane == 0) edge_row[warp] = cur;
        } else {
            acc[cur][lane] = a;
        }
    }
    __syncthreads();
    // the edge sums, in warp order
    if (warp == 0)
        for (int w = 0; w < REM_WARPS; ++w) {
            const int r = edge_row[w];
            if (r >= 0) acc[r][lane] = acc[r][lane] + edge[w][lane];
        }
    __syncthreads();
    float* R = static_cast<float*>(sv.W);
    const int f = f_lo + threadIdx.x;
    if (f >= f_hi || __ldg(&sv.rem_ptr[f]) == __ldg(&sv.rem_ptr[f + 1])) return;
    for (int j = 0; j < REM_STEPS && s0 + j < ntau; ++j) R[(size_t)(s0 + j) * nf + f] = acc[threadIdx.x][j];
}

// Q += the remainder's sums, for the rows k_spmm_rem summed (same grid and
// the same tests): runs once both the tensor-core product and the remainder
// are complete, so the two can run side by side.
__global__ void __launch_bounds__(128) k_rem_add(Batch b) {
    const DevSolve& sv = b.tab[blockIdx.z];
    const int rb = blockIdx.x, s0 = blockIdx.y * REM_STEPS;
    const int nf = sv.nf, ntau = sv.ntau;
    if (!sv.rem_ptr || rb * 128 >= nf || s0 >= ntau || !sv.ctl->active) return;
    const bool everyone = !sv.freeze || sv.ti == 0.0f;
    if (!everyone && !sv.rb_act[rb]) return;
    const int f = rb * 128 + threadIdx.x;
    if (f >= nf || __ldg(&sv.rem_ptr[f]) == __ldg(&sv.rem_ptr[f + 1])) return;
    float* Q = static_cast<float*>(sv.Q);
    const float* R = static_cast<const float*>(sv.W);
    for (int j = 0; j < REM_STEPS && s0 + j < ntau; ++j) {
        const size_t o = (size_t)(s0 + j) * nf + f;
        Q[o] = Q[o] + R[o];
    }
}

int launch_spmm_tc(const Batch& b, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    if (b.nq == 0) return 0;
    const size_t smem = spmm_tc_smem_bytes(b.tc_nmax, b.tc_stages);
    // the shared-memory attribute is set once per device; the two batch
    // groups launch from their own threads, so the record is atomic
    static std::atomic<uint64_t> attr_set{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = dev < 64 ? uint64_t(1) << dev : 0;
    if (!bit || !(attr_set.load(std::memory_order_acquire) & bit)) {
        size_t most = 0;  // largest ring over every admissible chunk size
        for (int n = 16; n <= tc_max_chunk(); n += 16) most = spmm_tc_smem_bytes(n) > most ? spmm_tc_smem_bytes(n) : most;
        if (cudaFuncSetAttribute(k_spmm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most) != cudaSuccess)
            return 2;
        attr_set.fetch_or(bit, std::memory_order_release);
    }
    // the list length and the ticket counter start at zero for every launch
    // (a memset node when the revolution is captured in a graph)
    if (cudaMemsetAsync(b.tc_work, 0, 2 * sizeof(int), st) != cudaSuccess) return 2;
    k_tc_compact<<<(b.nq + 127) / 128, 128, 0, st>>>(b);
    const int grid = b.nq < b.sms ? b.nq : b.sms;  // one persistent CTA per SM
    // The sparse remainder (latency-bound gathers) runs beside the product
    // (latency-bound on its copy ring) on the side stream, into its own sums.
    // Submitting the remainder first was measured faster on the 8-inertia
    // binary (two batch groups): 16.1 against 17.2 ms for the 6-revolution
    // step, 255.5 against 260.5 ms solved to convergence.
    const dim3 g((unsigned)b.rem_nmb, (unsigned)((b.rem_ntau + REM_STEPS - 1) / REM_STEPS), (unsigned)b.n);
    cudaStream_t side = static_cast<cudaStream_t>(b.side);
    const bool fork = b.rem_nmb > 0 && side && b.ev_fork && b.ev_join;
    if (fork) {
        cudaEvent_t ef = static_cast<cudaEvent_t>(b.ev_fork), ej = static_cast<cudaEvent_t>(b.ev_join);
        if (cudaEventRecord(ef, st) != cudaSuccess || cudaStreamWaitEvent(side, ef, 0) != cudaSuccess) return 2;
        k_spmm_rem<<<g, REM_WARPS * 32, 0, side>>>(b);
        if (cudaEventRecord(ej, side) != cudaSuccess) return 2;
    }
    k_spmm_tc<<<grid, TC_THREADS, smem, st>>>(b);
    if (b.rem_nmb > 0) {
        if (fork) {
            if (cudaStreamWaitEvent(st, static_cast<cudaEvent_t>(b.ev_join), 0) != cudaSuccess) return 2;
        } else {
            k_spmm_rem<<<g, REM_WARPS * 32, 0, st>>>(b);
        }
        k_rem_add<<<g, 128, 0, st>>>(b);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

__global__ void __launch_bounds__(256) k_w_bf16_one(DevSolve sv) {
    const int nf = sv.nf, ntau = sv.ntau, N = sv.tc_n, nch = sv.tc_nchunks;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)nf * ntau) return;
    const int s = (int)(i / nf), f = (int)(i % nf);
    const float x = static_cast<const float*>(sv.stemp1)[i];
    const float x2 = x * x;
    const float w = sv.es_w * (x2 * x2);
    __nv_bfloat16* W = static_cast<__nv_bfloat16*>(sv.Wb);
    const size_t base = ((size_t)(f / TC_K) * nch + s / N) * (size_t)2 * N * TC_K;
    const __nv_bfloat16 hi = __float2bfloat16_rn(w);
    W[base + swz(s % N, f % TC_K)] = hi;
    W[base + (size_t)N * TC_K + swz(s % N, f % TC_K)] = __float2bfloat16_rn(w - __bfloat162float(hi));
}

// Self-test of the bounded wait: one thread waits on an mbarrier that
// nothing arrives at, gives up after `limit` cycles and reports
// ST_TC_TIMEOUT, the path every wait of k_spmm_tc takes when its copies or
// products never land.  No copy, product or TMEM allocation is involved.
__global__ void k_wait_selftest(int* status, long long limit) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0 && !mbar_wait_lim(&bar, 0u, limit)) atomicOr(status, ST_TC_TIMEOUT);
}

int launch_wait_selftest(int* status, long long limit, stream_t stv) {
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    if (limit < 0) limit = 0;
    if (limit > WAIT_CYCLES) limit = WAIT_CYCLES;
    k_wait_selftest<<<1, 32, 0, st>>>(status, limit);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// W32[f][s] = eps sigma T^4 from the current surface temperatures (FP32,
// facet-major) through 32 x 32 tiles transposed in shared memory: the
// remainder's operand, set up with the temperatures (the conduction sweeps
// keep it current after that)
__global__ void __launch_bounds__(256) k_w32_fill(DevSolve sv) {
    __shared__ float t[32][33];
    const int f0 = blockIdx.x * 32, s0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const float* S1 = static_cast<const float*>(sv.stemp1);
    for (int j = ty; j < 32; j += 8) {
        const int s = s0 + j, f = f0 + tx;
        float w = 0.0f;
        if (s < sv.ntau && f < sv.nf) {
            const float x = S1[(size_t)s * sv.nf + f];
            const float x2 = x * x;
            w = sv.es_w * (x2 * x2);
        }
        t[j][tx] = w;
    }
    __syncthreads();
    for (int j = ty; j < 32; j += 8) {
        const int f = f0 + j, s = s0 + tx;
        if (f < sv.nf && s < sv.ntau) sv.W32[(size_t)f * sv.w32_ld + s] = t[tx][j];
    }
}

int launch_w_bf16_one(const DevSolve& s, stream_t stv) {
    if (!s.tc_tiles) return 0;
    cudaStream_t st = static_cast<cudaStream_t>(stv);
    const size_t n = (size_t)s.nf * s.ntau;
    k_w_bf16_one<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s);
    if (s.W32) {
        dim3 g((unsigned)((s.nf + 31) / 32), (unsigned)((s.ntau + 31) / 32));
        k_w32_fill<<<g, 256, 0, st>>>(s);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // namespace atpm
