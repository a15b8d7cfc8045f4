// Host-side objects of libatpm shared by the C ABI (atpm_capi.cpp) and the
// serving scheduler (atpm_server.cpp).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <atomic>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/atpm.h"
#include "atpm_internal.h"

// launch configuration chosen by the autotuner for one kind of batch
struct atpm_tune_choice {
    int cond_variant = 4;  // FAST conduction variant (1-3 register budgets, 4 paired facets)
    int tc_stages = 0;     // tensor-core pipeline depth (0: deepest)
    float rev_ms[5] = {0, 0, 0, 0, 0};  // the timed revolutions, one per candidate
};

// A context lives while its creator's handle or any solve, server or crater
// made from it does: atpm_context_destroy drops the creator's reference and
// the last object destroyed frees it, so destroy calls may come in any order
// (a garbage collector's, at interpreter exit, for one).
struct atpm_context {
    std::atomic<int> refs{1};
    int device = 0;
    int sm_count = 1;
    std::mutex mu;
    bool tables = false;
    atpm::HostPowTab p4, p3;
    atpm::HostPowTab pq;  // x^0.25, built on first need
    std::map<uint64_t, atpm_tune_choice> tune;  // by batch kind
};

// Read-only tensor-core view-factor tiles of one shape (FAST), shared by a
// solve and its clones: tiles | row-block tile ranges | column blocks |
// residual tiles | residual index | (row block, column block) slot table.
struct TcShared {
    std::atomic<int> refs{1};
    void* mem = nullptr;
    size_t bytes = 0;
    std::vector<int> rb_tiles;  // tiles per 128-facet row block (work ordering)
    size_t tiles = 0;           // tensor-core tiles
    size_t remainder = 0;       // list entries of the sparse remainder
    void* rem_mem = nullptr;    // the remainder's row offsets, columns and view factors
};

struct atpm_solve {
    atpm_context* ctx = nullptr;
    atpm_params P{};
    int nf = 0, nv = 0, nnz = 0;
    size_t rs = 4;  // bytes per state scalar
    cudaStream_t st = nullptr;
    void* arena = nullptr;
    size_t arena_bytes = 0;
    atpm::DevSolve ds{};
    atpm::DevSolve* ds_dev = nullptr;
    int4* wmap = nullptr;
    int2* fmap = nullptr;
    int nw = 0, nfb = 0;
    TcShared* tc = nullptr;   // tensor-core tiles (FAST), shared with clones
    void* wb_mem = nullptr;   // this solve's BF16 W tiles
    size_t wb_bytes = 0;
    void* w32_mem = nullptr;  // this solve's FP32 W rows for the sparse remainder
    size_t w32_bytes = 0;
    // the stream the sparse remainder of a batch this solve leads runs on
    // beside the tensor-core product, and its fork / join events (made on
    // first use)
    cudaStream_t side_st = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // the last atpm_geometry_shadow's shadow drivers
    double last_shadow_ms = 0.0;
    int64_t last_shadow_rays = 0, last_shadow_tests = -1;
    int4* qmap = nullptr;
    int nq = 0;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<double> vert_h;
    std::vector<int32_t> fac_h;
    bool have_forcing = false, have_temps = false;
    bool has_position = false;  // body centre set directly (atpm_set_position)
    // non-synchronous binary (atpm_set_binary_rotation): vertices/facets from
    // sec_vertex/sec_facet on turn revs_s times per model period, the rest
    // revs_p times; -1: synchronous (one rigid rotation)
    int sec_vertex = -1, sec_facet = -1, revs_p = 1, revs_s = 1;
    float ir_abs = 1.0f;  // IR absorptivity in the self-heating sum
    double position[3] = {0, 0, 0};  // km, heliocentric
    float ti = 0.0f;
    double last_ms = 0.0;
    int64_t last_launches = 0, last_facet_steps = 0;
    int last_cond_variant = 0, last_tc_stages = 0, last_tuned = 0;  // configuration of the last batch run
    int last_nrev = 0;
};


namespace atpm {
// one batched revolution chunk for solves that share precision and nx:
// k revolutions launched directly (no graph); `table` is a caller-owned
// device buffer of at least batch_table_bytes(solves, n) bytes
size_t batch_table_bytes(atpm_solve* const* solves, int n);
atpm_status batch_step(atpm_solve* const* solves, int n, int k, void* table, cudaStream_t st);
// a batch's device table and launch description, built once for a set of
// solves and reused for every tick until the set changes
struct BatchPlan {
    std::vector<atpm_solve*> solves;
    void* table = nullptr;
    size_t bytes = 0;
    Batch b{};
};
atpm_status batch_plan(atpm_solve* const* solves, int n, BatchPlan& plan, cudaStream_t st);
atpm_status batch_plan_step(const BatchPlan& plan, int k, cudaStream_t st);
void batch_plan_free(BatchPlan& plan);
// dst (a clone of src's shape) takes src's parameters and device state
// again by device copies, without allocating
atpm_status solve_refresh(atpm_solve* dst, atpm_solve* src);
// the crater model's Sun vectors [nfc][ntau][3] and facet shadows [nfc][ntau]
// of facets f0 .. f0 + nfc - 1 (device arrays), on stream st (synchronised)
atpm_status solve_crater_sun(atpm_solve* s, int f0, int nfc, float* sun, int* shadow, cudaStream_t st);
atpm_status fail_status(atpm_status s, const char* msg);
}  // namespace atpm

// a crater's device arrays and a wait for its queued work (atpm_crater_api.cpp)
const atpm::CraterDev& atpm_crater_device(const atpm_crater* c);
cudaError_t atpm_crater_sync(const atpm_crater* c);

// context references held by solves, servers and craters (atpm_capi.cpp)
void atpm_context_retain(atpm_context* c);
void atpm_context_release(atpm_context* c);
