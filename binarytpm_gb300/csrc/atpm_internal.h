// Internal declarations shared by the CUDA kernels and the host runtime of
// libatpm.  Device layouts (all per solve, resident for the solve's life):
//
//   E, Q, stemp0, stemp1   [ntau][nf]   step-major: thread f reads step s of
//                                       consecutive facets -> coalesced
//   temp                   [nx+1][nf]   depth-major, read once per revolution
//   W                      [nf][ntau]   facet-major eps*sigma*T^4 of the
//                                       previous revolution: the self-heating
//                                       gather reads 32 consecutive steps
//   shadow, cosil          [nf][ntau]   facet-major (scattering gathers)
//   dep_ptr/idx/vf         CSR view-factor lists in file order
//
// Scalar precision: MODE 0 = reference FP32 (exact operand order), MODE 1 =
// FP64, MODE 2 = fast FP32.
#pragma once
#include <cstdint>
#include <cstddef>

namespace atpm {

enum : int { MODE_REF = 0, MODE_FP64 = 1, MODE_FAST = 2 };

// status bits written by kernels into DevSolve::status
enum : int {
    ST_NONFINITE = 1,     // a surface temperature became NaN/Inf
    ST_NEWTON_CAP = 2,    // Newton iteration cap reached
    ST_POW_RANGE = 4,     // REFERENCE mode: pow argument outside the exact table range
    ST_SCATTER_CAP = 8,   // scattering iteration cap reached
    ST_TC_TIMEOUT = 16,   // a tensor-core pipeline wait gave up
};

// exception table: glibc powf(x, e) where it differs from the device's
// double-float evaluation of x^e; open addressing on the float's bits
struct PowTab {
    const uint2* slots;   // {key bits, value bits}; key 0xFFFFFFFF = empty
    uint32_t log2slots;
    uint32_t lo_bits;     // first float (bits) covered
    uint32_t hi_bits;     // one past the last float covered
};

#ifdef __CUDACC__
// libm-exact result: table hit -> libm's value, miss -> the device value v;
// an argument outside the table's range (or no table) flags ST_POW_RANGE
__device__ __forceinline__ float pow_table_fix(const PowTab& t, float x, float v, int* status) {
    const uint32_t b = __float_as_uint(x);
    if (t.slots && b - t.lo_bits < t.hi_bits - t.lo_bits) {
        const uint32_t mask = (1u << t.log2slots) - 1u;
        uint32_t h = (b * 2654435761u) >> (32 - t.log2slots);
        for (int probe = 0; probe < 1024; ++probe) {
            const uint2 kv = __ldg(&t.slots[h]);
            if (kv.x == b) return __uint_as_float(kv.y);
            if (kv.x == 0xFFFFFFFFu) return v;
            h = (h + 1u) & mask;
        }
        return v;
    }
    if (x != 0.0f) atomicOr(status, 4 /* ST_POW_RANGE */);
    return v;
}
// x^4 and x^3 as the device evaluates them before the exception table
// (host twins emu_pow4 / emu_pow3): a double-float product from 2^-4 up, and
// below 2^-4, where that product underflows, one double product rounded to
// float (x^2 is exact in double)
__device__ __forceinline__ float dev_pow4(float x) {
    if (x < 0.0625f) {
        const double d = (double)x, d2 = __dmul_rn(d, d);
        return __double2float_rn(__dmul_rn(d2, d2));
    }
    const float h = __fmul_rn(x, x);
    const float l = __fmaf_rn(x, x, -h);
    const float p = __fmul_rn(h, h);
    const float e = __fmaf_rn(h, h, -p);
    const float c = __fmaf_rn(__fmul_rn(2.0f, h), l, e);
    return __fadd_rn(p, c);
}
__device__ __forceinline__ float dev_pow3(float x) {
    if (x < 0.0625f) {
        const double d = (double)x;
        return __double2float_rn(__dmul_rn(__dmul_rn(d, d), d));
    }
    const float h = __fmul_rn(x, x);
    const float l = __fmaf_rn(x, x, -h);
    const float p = __fmul_rn(h, x);
    const float e = __fmaf_rn(h, x, -p);
    const float c = __fmaf_rn(l, x, e);
    return __fadd_rn(p, c);
}
// x^0.25 through two correctly rounded double square roots (host: emu_qroot)
__device__ __forceinline__ float dev_qroot(float x) { return (float)__dsqrt_rn(__dsqrt_rn((double)x)); }
#endif

// per-solve control words (device memory, updated by the advance kernel)
struct Ctl {
    int rev;        // next revolution index
    int active;     // 1 while the revolution loop runs
    int converged;  // reference `converged` flag
    int numconv;    // facets converged after the last revolution
};

struct DevSolve {
    int nf, nv, ntau, nx, revcap, mode;
    int nnz;
    int freeze;             // 1: converged facets are frozen (reference)
    // shape
    const double* vert;      // [nv][3]
    const int* fac;          // [nf][3]
    const int* dep_ptr;      // [nf+1]
    const int* dep_idx;      // [nnz]
    const float* dep_vf;     // [nnz]
    // forcing
    uint8_t* shadow;         // [nf][ntau]
    void* cosil;             // [nf][ntau] float (modes 0,2) / double (mode 1)
    void* Efm;               // [nf][ntau] R: scattering output, facet-major
    void* E;                 // [ntau][nf] R
    // state
    void* stemp0;            // [ntau][nf] R
    void* stemp1;            // [ntau][nf] R
    void* temp;              // [nx+1][nf] R
    void* Q;                 // [ntau][nf] R
    void* W;                 // [nf][ntau] R (FAST with tensor-core tiles: the sparse remainder's
                             // sums, [ntau][nf] FP32, which k_rem_add adds to Q)
    uint8_t* conv;           // [nf] frozen (reference astconverged)
    uint8_t* hot;            // [nf] some |stemp1-stemp0| >= TACC this revolution
    // facets still active after each convergence test (FAST, freeze on),
    // double-buffered by revolution parity: k_converge of revolution r fills
    // list (r+1)&1, the conduction of r+1 reads it, k_advance of r+1 clears it
    uint8_t* rb_act;         // [ceil(nf/128)] some facet of the 128-facet row block active (FAST)
    int* act_list;           // [2][nf]
    int* act_cnt;            // [5]: counts of the two lists, the revolution each list is for, and
                             // (batch leader) whether this revolution runs warp per facet
    int* counts;             // [revcap] numconverged after each revolution
    int* status;             // ST_* bits
    Ctl* ctl;
    double* diag;            // [4] FP64 energy-balance accumulators
    // scalars (float for modes 0/2, double for mode 1), computed on the host
    // in the reference's operand order
    float ti, oma, es, es4, m1, r, tacc, tacc10, alb, solar, sacc;
    double ti_d, oma_d, es_d, es4_d, m1_d, r_d, tacc_d, tacc10_d, alb_d, solar_d, sacc_d;
    int newton_cap;
    // non-synchronous binary: facets >= fsplit (the secondary) use r2 / m1_2,
    // from their own number of rotations per model period; fsplit = nf otherwise
    int fsplit;
    float r2, m1_2;
    double r2_d, m1_2_d;
    // weight of the self-heating sum: IR absorptivity x eps x sigma
    float es_w;
    double es_w_d;
    // FAST precision, tensor-core self-heating (atpm_spmm_tc.cu); null when off
    const int* tc_ptr;       // [nmb+1] tile range of each 128-facet row block
    const int* tc_col;       // [ntiles] 64-facet column block of each tile (bits 0-23), mask of its
                             // 16-wide K slices that hold an entry (bits 24-27)
    const void* tc_tiles;    // [ntiles][128*64] BF16, swizzled K-major
    const int* tc_lo;        // [ntiles] index into tc_lo_tiles, or -1
    const void* tc_lo_tiles; // [nlo][128*64] BF16 residual V - bf16(V) of tiles with large entries
    void* Wb;                // [nkb][nchunks][2][tc_n*64] BF16 eps*sigma*T^4 (hi, lo), swizzled
    int tc_n, tc_nchunks, tc_nmb, tc_nkb;
    // sparse remainder of the view-factor lists (FAST): the entries of the
    // (128-row, 64-column) cells too sparse for a tensor-core tile, per row
    // in list order (CSR, FP32 values), summed by k_spmm_rem against W32,
    // this solve's eps*sigma*T^4 facet-major in FP32
    const int* rem_ptr;      // [nf+1], or null when every entry is in a tile
    const int* rem_idx;      // [rem_nnz]
    const float* rem_vf;     // [rem_nnz]
    const uint8_t* rem_row;  // [rem_nnz] the entry's row within its 128-facet row block
    float* W32;              // [nf][w32_ld] FP32 (null without a remainder)
    int w32_ld;              // row stride of W32: ntau rounded up to 32 (the remainder's step chunks)
};

// element offset of (row, k) inside a 128-byte-swizzled K-major tile with 64
// BF16 per row: 16-byte chunk c of row r is stored at chunk c ^ (r % 8)
__host__ __device__ __forceinline__ uint32_t swz(uint32_t row, uint32_t k) {
    return row * 64u + ((((k >> 3) ^ (row & 7u)) << 3) | (k & 7u));
}

// ---------------------------------------------------------------- launchers
// (definitions in the .cu files; `stream` is a cudaStream_t)
using stream_t = void*;

// geometry + shadowing (atpm_geom.cu)
struct GeomWork {
    double* hp;      // [nv][ntau][3] heliocentric vertex positions
    double* hm;      // [nf][ntau][3] heliocentric facet midpoints
    double* nrm;     // [nf][ntau][3] unit normals
    double* dist;    // [nf][ntau] |hm|
    const double* rot;  // [ntau][2] cos, sin of the rotation angle (host libm)
    const double* rot2; // the same for vertices >= vsplit (non-synchronous secondary)
    int vsplit;         // first vertex of the secondary (nv when synchronous)
    double tm[9];    // pole transformation matrix
    double car[3];   // heliocentric centre (km)
    unsigned long long* tests;  // [64] exact ray-triangle tests of the culled drivers (or null)
};
int launch_geometry(const DevSolve& s, const GeomWork& g, stream_t st);
// vertex positions of every step (into g.hp), then the crater model's Sun
// vector [nfc][ntau][3] and the facet shadow flags [nfc][ntau] of facets
// f0 .. f0 + nfc - 1
int launch_crater_sun(const DevSolve& s, const GeomWork& g, int f0, int nfc, float* sun, int* shadow, stream_t st);
int launch_shadow_deplist(const DevSolve& s, const GeomWork& g, stream_t st);
int launch_shadow_allpairs(const DevSolve& s, const GeomWork& g, stream_t st);
// the same flags with the projected-box cull in front of the exact test
// (dependent lists, or all pairs over a per-step grid); -1: not applicable
// (body too close to the origin for a central projection), use the above
int launch_shadow_culled(const DevSolve& s, const GeomWork& g, bool all_pairs, stream_t st);

// scattering (atpm_scatter.cu)
int launch_single_scattering(const DevSolve& s, stream_t st);
int launch_multiple_scattering(const DevSolve& s, void* work, stream_t st);
size_t multiple_scattering_work_bytes(const DevSolve& s);
int launch_forcing_transpose(const DevSolve& s, stream_t st);
int launch_set_forcing(const DevSolve& s, const int32_t* shadow_d, const float* illum_d, stream_t st);
// [rows][cols] -> [cols][rows], element sizes 4 or 8 bytes (float / double)
int launch_transpose(const void* src, int src_bytes, void* dst, int dst_bytes, size_t rows, size_t cols, stream_t st);

// thermal (atpm_thermal.cu); batched over `n` solves in `tab` (device array)
struct Batch {
    const DevSolve* tab;     // device [n]
    int n;
    const int4* wmap;        // W/Q tile map: {solve, f0, s0, 0}
    int nw;
    const int2* fmap;        // facet-block map: {solve, f0}
    int nfb;
    int mode, nx;
    PowTab p4, p3;
    PowTab pq;               // x^0.25 (built only when a REFERENCE solve has TI 0)
    const int4* qmap;        // tensor-core work items {solve, row block, step chunk, 0}
    int nq;
    int4* tc_list;           // [nq] this launch's items whose row block has an active facet
    int* tc_work;            // [2] list length, next ticket (zeroed before every launch)
    int tc_nmax;             // largest step chunk in the batch
    int cond_variant;        // FAST conduction register/occupancy variant (1, 2, 3)
    int tc_stages;           // tensor-core pipeline depth (0: deepest that fits)
    int warp_tail;           // 1: FAST revolutions with few active facets sweep the active list
                             // (thread per facet; warp per facet below tail_limit)
    int tail_limit;          // active facets of the batch up to which they do
    int sms;                 // SMs of the device (persistent tensor-core grid)
    int rem_nmb, rem_ntau;   // largest row-block count / steps of the batch's solves with a
                             // sparse remainder (0: none; the remainder kernel's grid)
    // host handles: a second stream on which the remainder runs beside the
    // tensor-core product (forked and joined with the two events; null: the
    // remainder runs after the product on the batch's stream)
    void* side;
    void* ev_fork;
    void* ev_join;
};
// deepest tensor-core pipeline that fits shared memory for step chunk N
int tc_max_stages(int N);
int launch_revolution(const Batch& b, stream_t st);  // W, Q, conduction, convergence, advance
// per solve: control word (4), status, counts of the last `window` revolutions
int launch_progress(const Batch& b, int window, int* out, stream_t st);
int kernels_per_revolution(const Batch& b);          // kernels launch_revolution starts
// BF16 view-factor tiles (and residual tiles) of a solve from its uploaded
// lists: slot[mb * nkb + kb] = tile of (row block, column block), lo_of[t] =
// residual tile of tile t or -1; tiles must be zeroed (atpm_spmm_tc.cu)
// per (row block, column block) cell of the view-factor lists: largest
// |value| as float bits + 1 (0: no entry) and the mask of 16-wide K slices
// with an entry; cmax and cmask zeroed by the caller (atpm_spmm_tc.cu)
int launch_tc_cells(const DevSolve& s, int nkb, unsigned* cmax, unsigned* cmask, unsigned* count, stream_t st);
// the sparse remainder's per-row counts, then (rptr scanned) its lists in list order
int launch_rem_count(const DevSolve& s, int nkb, const int* slot, int* count, stream_t st);
int launch_rem_fill(const DevSolve& s, int nkb, const int* slot, const int* rptr, int* ridx, float* rvf, uint8_t* rrow,
                    stream_t st);
// cells whose tile needs the BF16 residual for some row's flux (need zeroed
// by the caller); returns 1 when the shape is too large for the per-row maps
int launch_tc_rowneed(const DevSolve& s, int nkb, unsigned* need, stream_t st);
int launch_tc_fill(const DevSolve& s, int nkb, const int* slot, const int* lo_of, void* tiles, void* lo_tiles,
                   stream_t st);
// part 0 W, 1 Q, 2 conduction, 3 convergence, 4 advance
int launch_revolution_part(const Batch& b, int part, stream_t st);
int launch_initial_mean(const DevSolve& s, void* mean_out, stream_t st);
// T0 = ((1-A) mean / (eps sigma))^0.25 (x^0.25 exact to libm through pq in REFERENCE)
int launch_fill_initial(const DevSolve& s, const void* mean, const PowTab& pq, stream_t st);
int launch_energy_balance(const DevSolve& s, stream_t st);

// disk-integrated flux (atpm_flux.cu)
constexpr int kMaxFluxWavelengths = 8;
struct FluxArgs {
    const double* rot;       // [ntau][2] cos, sin of the rotation angle (host libm)
    const double* rot2;      // vertices >= vsplit (non-synchronous secondary)
    int vsplit;
    double tm[9];            // pole matrix
    double car[3];           // body centre (km)
    double obs[3];           // observer (km)
    double eps;
    const uint8_t* visible;  // [nf][ntau] or null (horizon test only)
    int nwl;
    double b1[kMaxFluxWavelengths];  // 2 h c^2 / lambda^5
    double lk[kMaxFluxWavelengths];  // lambda * k
    double hc;                       // h * c
    double* partial;         // [ntau][blocks][nwl]
    double* out;             // [ntau][nwl]
    // rough surface (crater sub-facets); null for the smooth-surface sum
    const float* sub_T;      // [nf][ntau][nsf] sub-facet surface temperatures
    const float* sub_vis;    // [nf][ntau][nsf] visible fraction toward the observer
    const double* sub_geo;   // [nsf][4] unit normal, area
    int nsf;
    double sub_total;        // sum over sub-facets of area * normal_z
};
size_t flux_partial_bytes(const DevSolve& s, int nwl);
int launch_disk_flux(const DevSolve& s, const FluxArgs& a, stream_t st);
// tensor-core self-heating (atpm_spmm_tc.cu)
int launch_w_bf16_one(const DevSolve& s, stream_t st);
int launch_spmm_tc(const Batch& b, stream_t st);
int launch_wait_selftest(int* status, long long limit, stream_t st);
size_t spmm_tc_smem_bytes(int N, int stages = 0);  // 0: deepest ring that fits
int tc_max_chunk();  // largest step chunk N of the tensor-core product
bool conduction_nx_supported(int nx);

// crater (roughness) module (atpm_crater.cu); layouts [facet][step][sub-facet]
struct CraterDev {
    int nf, ntau, nx, nsf, mode;
    // crater model
    const float* V;          // [nsf][nsf] V[i][j]
    const float* cverts;     // [nsv][3]
    const int* cfac;         // [nsf][3]
    const float* ctri;       // [nsf][2][3]
    const float* cmult;      // [100][2] trivector multipliers
    const float* cnorm;      // [nsf][3] sub-facet unit normals (atpm_crater_set_surface), or null
    float PI, rot_period;
    // non-synchronous binaries (175706/Run-04/thermal_GPU.cu): revolutions of
    // each facet's body per model period (null: 1 for every facet) and the
    // IR absorptivity of crater self-heating (1 unless set)
    const float* numrevs;    // [nf] or null
    float ir_abs;
    // per facet
    uint8_t* conv;           // sfc_converged
    const float* albedo;
    const float* ti;
    uint8_t* hot;            // some |stemp1-stemp0| >= TACC in the last revolution
    // per facet, step (, sub-facet)
    const int* shadow;       // [nf][ntau]
    float* sfc_shadow;       // [nf][ntau][nsf]
    const float* illumvec;   // [nf][ntau][3]
    const float* illumangle; // [nf][ntau][nsf]
    float* RI;               // illumination [nf][ntau][nsf]
    const float* RGI;        // global illumination
    const float* RGH;        // global heating
    float* stemp0;           // [nf][ntau][nsf]
    float* stemp1;
    float* temp;             // [nf][nx+1][nsf]
    int* status;
};

// what: 0 partial shadow, 1 scattering, 2 revolution, 3 equilibrium,
// 4 converged, 5 initial mean, 6 initial self-heating, 7 fill, 8 fourth root
int crater_launch(int what, const CraterDev& c, const PowTab& p4, const PowTab& pq, const float* fargs, void* p0,
                  void* p1, stream_t st);
bool crater_nx_supported(int nx);
// the crater's forcing from a solve (atpm_crater_forcing.cu)
int launch_crater_surface(const CraterDev& c, float* illumangle, stream_t st);
int launch_crater_gvf(const CraterDev& c, const double* vert, const int* fac, const int* dep_ptr,
                      const float* dep_vf, int f0, const float* vec, float* gvf, stream_t st);
int launch_crater_gsum(const CraterDev& c, const int* dep_ptr, const int* dep_idx, int f0, const float* gvf,
                       const float* X, int ntau_x, int heat, float alb, float eps, float sigma, float* out,
                       stream_t st);
int launch_transpose_sf(const float* in, int ntau, int nf, float* out, stream_t st);

// pow exception tables (atpm_powtab.cpp)
struct HostPowTab {
    uint2* slots_dev = nullptr;
    uint32_t log2slots = 0, lo_bits = 0, hi_bits = 0;
    int64_t exceptions = 0;
};
// builds the table for exponent e in {3, 4} over the positive floats below
// 2^12, or for the quarter power (e = -4) below 2^44 (subnormals included),
// and uploads it
int build_pow_table(int e, HostPowTab* out, char* err, size_t errlen);
// host emulation of the device's double-float x^e (exact IEEE ops)
float emu_pow3(float x);
float emu_pow4(float x);
float emu_qroot(float x);

}  // namespace atpm
