// Serving scheduler: continuous batching of thermal solves on one GPU.
//
// The reference runs one compile-time-sized solve per process
// (3905/Thermal/NominalPole/main.cpp:3009-3052).  Here a single process keeps
// many solves resident and advances them together:
//
//   * shapes are registered once (atpm_server_add_shape): their geometry,
//     shadowing and scattered sunlight are computed on the device and kept as
//     a prototype solve, so each request only carries its thermal inertia;
//   * a request is admitted when a batch slot is free and its device
//     footprint fits the HBM budget left by the resident solves; it is a
//     device copy of the prototype (atpm_solve_clone: forcing, and the
//     prototype's tensor-core tiles shared) with its own temperatures, so
//     admission does no host work on the shape and overlaps the revolutions
//     of the solves already running;
//   * every scheduler tick advances all resident solves by K revolutions in
//     shared launches (one batch table, the tensor-core and conduction
//     kernels span every solve) and retires the ones that converged or hit
//     the revolution cap: their temperatures are copied out, their device
//     memory returns to the budget and waiting requests are admitted.
//
// Each solve's arithmetic is independent of the others in the batch, so a
// result is bit-identical whether the request ran alone or in a mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "atpm_host.h"

namespace {

using clock_t_ = std::chrono::steady_clock;

double now_s() {
    return std::chrono::duration<double>(clock_t_::now().time_since_epoch()).count();
}

struct ShapeEntry {
    std::vector<double> v;
    std::vector<int32_t> f, ptr, idx;
    std::vector<float> vf;
    atpm_shape shape{};
    atpm_params params{};
    atpm_solve* proto = nullptr;  // resident forcing
    uint64_t footprint = 0;
};

struct Request {
    int64_t id = 0;
    int shape = 0;
    float ti = 0.0f;
    double t_submit = 0, t_start = 0, t_done = 0;
    atpm_status status = ATPM_OK;
    bool done = false, cancelled = false;
    int nrev = 0;
    int64_t facet_steps = 0;
    std::vector<float> stemp1;
    atpm_solve* solve = nullptr;
    uint64_t footprint = 0;
};

}  // namespace

struct atpm_server {
    atpm_context* ctx = nullptr;
    int precision = ATPM_FAST;
    int nx = 0;
    uint64_t budget = 0, resident = 0;
    int max_active = 64;
    int revs_per_tick = 2;
    cudaStream_t run_st = nullptr, setup_st = nullptr;
    void* table = nullptr;
    size_t table_bytes = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> queue;
    std::vector<Request*> active;
    std::unordered_map<int64_t, std::unique_ptr<Request>> all;
    std::vector<std::unique_ptr<ShapeEntry>> shapes;
    std::vector<double> latencies;
    int64_t next_id = 1;
    int64_t done_facet_steps = 0;
    double t_first = 0, t_last = 0;
    bool stop = false;
    std::thread loop;
    atpm_status loop_error = ATPM_OK;
};

namespace {

atpm_status admit(atpm_server* S, Request* r) {
    ShapeEntry* sh;
    {
        // add_shape may grow the table on another thread: read it locked (the
        // entries themselves never move)
        std::lock_guard<std::mutex> lk(S->mu);
        sh = S->shapes[r->shape].get();
    }
    atpm_solve* s = nullptr;
    // a device copy of the prototype: forcing and (shared) tensor-core tiles
    // come along, no host work on the shape
    atpm_status st = atpm_solve_clone(sh->proto, &s);
    if (st) return st;
    if (!st) st = atpm_set_thermal_inertia(s, r->ti);
    if (!st && r->ti != 0.0f) st = atpm_initialise_temperatures(s);
    if (st) {
        atpm_solve_destroy(s);
        return st;
    }
    r->solve = s;
    r->t_start = now_s();
    return ATPM_OK;
}

void retire(atpm_server* S, Request* r, atpm_status st) {
    if (!st && r->solve) {
        r->stemp1.resize((size_t)r->solve->nf * r->solve->P.ntau);
        st = atpm_get_surface_temperature(r->solve, r->stemp1.data(), nullptr);
        r->nrev = r->solve->last_nrev;
    }
    if (r->solve) {
        atpm_solve_destroy(r->solve);
        r->solve = nullptr;
    }
    r->status = st;
    r->t_done = now_s();
    r->done = true;
}

// per-solve bookkeeping after a tick: counts -> revolutions and facet-steps
int64_t tick_facet_steps(atpm_solve* s, const atpm::Ctl& before, const atpm::Ctl& after) {
    const int nf = s->nf, ntau = s->P.ntau;
    const bool all_active = !s->P.freeze || s->ti == 0.0f;
    int64_t fs = 0;
    std::vector<int32_t> cnt(s->P.revcap, 0);
    if (after.rev > before.rev) {
        if (cudaMemcpy(cnt.data(), s->ds.counts, (size_t)s->P.revcap * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            return 0;
        for (int r = before.rev; r < after.rev; ++r) {
            int active = nf;
            if (!all_active && r - 1 > 5) active = nf - cnt[r - 1];
            fs += (int64_t)active * ntau;
        }
    }
    return fs;
}

void run_loop(atpm_server* S) {
    cudaSetDevice(S->ctx->device);
    std::vector<atpm::Ctl> before, after;
    while (true) {
        // admission (holding the lock only to pick requests)
        std::vector<Request*> to_admit;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] { return S->stop || !S->queue.empty() || !S->active.empty(); });
            if (S->stop) break;
            while (!S->queue.empty() && (int)(S->active.size() + to_admit.size()) < S->max_active) {
                Request* r = S->queue.front();
                if (r->cancelled) {
                    S->queue.pop_front();
                    r->status = ATPM_E_CANCELLED;
                    r->done = true;
                    r->t_done = now_s();
                    S->cv_done.notify_all();
                    continue;
                }
                if (S->resident + r->footprint > S->budget) break;  // wait for memory to free up
                S->queue.pop_front();
                S->resident += r->footprint;
                to_admit.push_back(r);
            }
        }
        for (Request* r : to_admit) {
            atpm_status st = admit(S, r);
            std::lock_guard<std::mutex> lk(S->mu);
            if (st) {
                S->resident -= r->footprint;
                retire(S, r, st);
                S->cv_done.notify_all();
            } else {
                S->active.push_back(r);
            }
        }
        std::vector<Request*> act;
        {
            std::lock_guard<std::mutex> lk(S->mu);
            act = S->active;
        }
        if (act.empty()) continue;
        // one tick: K revolutions of every resident solve in shared launches
        std::vector<atpm_solve*> sv;
        for (Request* r : act) sv.push_back(r->solve);
        const size_t need = atpm::batch_table_bytes(sv.data(), (int)sv.size());
        if (need > S->table_bytes) {
            if (S->table) cudaFree(S->table);
            S->table = nullptr;
            S->table_bytes = 0;
            if (cudaMalloc(&S->table, need * 2) != cudaSuccess) {
                S->loop_error = atpm::fail_status(ATPM_E_NOMEM, "server: batch table allocation failed");
                break;
            }
            S->table_bytes = need * 2;
        }
        before.resize(act.size());
        after.resize(act.size());
        for (size_t i = 0; i < act.size(); ++i)
            cudaMemcpy(&before[i], act[i]->solve->ds.ctl, sizeof(atpm::Ctl), cudaMemcpyDeviceToHost);
        atpm_status st = atpm::batch_step(sv.data(), (int)sv.size(), S->revs_per_tick, S->table, S->run_st);
        if (!st && cudaStreamSynchronize(S->run_st) != cudaSuccess)
            st = atpm::fail_status(ATPM_E_CUDA, "server: revolution tick failed");
        std::vector<int> status(act.size(), 0);
        for (size_t i = 0; i < act.size() && !st; ++i) {
            cudaMemcpy(&after[i], act[i]->solve->ds.ctl, sizeof(atpm::Ctl), cudaMemcpyDeviceToHost);
            cudaMemcpy(&status[i], act[i]->solve->ds.status, 4, cudaMemcpyDeviceToHost);
        }
        std::lock_guard<std::mutex> lk(S->mu);
        std::vector<Request*> keep;
        for (size_t i = 0; i < act.size(); ++i) {
            Request* r = act[i];
            if (st) {
                S->resident -= r->footprint;
                retire(S, r, st);
                continue;
            }
            const int64_t fs = tick_facet_steps(r->solve, before[i], after[i]);
            r->facet_steps += fs;
            S->done_facet_steps += fs;
            r->solve->last_nrev = after[i].rev;
            atpm_status rs = ATPM_OK;
            if (status[i] & atpm::ST_NONFINITE) rs = ATPM_E_NONFINITE;
            else if (status[i] & (atpm::ST_NEWTON_CAP | atpm::ST_TC_TIMEOUT)) rs = ATPM_E_ITERATION;
            if (!after[i].active || rs || r->cancelled) {
                S->resident -= r->footprint;
                retire(S, r, r->cancelled ? ATPM_E_CANCELLED : rs);
                if (!r->status) {
                    S->latencies.push_back(r->t_done - r->t_submit);
                    S->t_last = r->t_done;
                }
            } else {
                keep.push_back(r);
            }
        }
        S->active = keep;
        S->cv_done.notify_all();
    }
    std::lock_guard<std::mutex> lk(S->mu);
    for (Request* r : S->active) retire(S, r, ATPM_E_CANCELLED);
    S->active.clear();
    S->cv_done.notify_all();
}

}  // namespace

extern "C" {

ATPM_API atpm_status atpm_server_create(atpm_context* ctx, int32_t precision, int32_t nx, uint64_t budget_bytes,
                                        int32_t max_active, int32_t revs_per_tick, atpm_server** out) {
    if (!ctx || !out || max_active < 1 || revs_per_tick < 1)
        return atpm::fail_status(ATPM_E_INVALID, "server_create: bad arguments");
    auto* S = new atpm_server();
    S->ctx = ctx;
    atpm_context_retain(ctx);
    S->precision = precision;
    S->nx = nx;
    S->budget = budget_bytes;
    S->max_active = max_active;
    S->revs_per_tick = revs_per_tick;
    cudaSetDevice(ctx->device);
    if (cudaStreamCreateWithFlags(&S->run_st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&S->setup_st, cudaStreamNonBlocking) != cudaSuccess) {
        atpm_context_release(S->ctx);
        delete S;
        return atpm::fail_status(ATPM_E_CUDA, "server_create: stream creation failed");
    }
    S->loop = std::thread(run_loop, S);
    *out = S;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_server_add_shape(atpm_server* S, const atpm_shape* shape, const atpm_params* params,
                                           int32_t* shape_id) {
    if (!S || !shape || !params || !shape_id) return atpm::fail_status(ATPM_E_INVALID, "add_shape: bad arguments");
    if (params->precision != S->precision || params->nx != S->nx)
        return atpm::fail_status(ATPM_E_INVALID, "add_shape: precision and nx must match the server");
    auto e = std::make_unique<ShapeEntry>();
    const int nnz = shape->dep_ptr[shape->nf];
    e->v.assign(shape->vertices, shape->vertices + 3 * (size_t)shape->nv);
    e->f.assign(shape->facets, shape->facets + 3 * (size_t)shape->nf);
    e->ptr.assign(shape->dep_ptr, shape->dep_ptr + shape->nf + 1);
    if (nnz) {
        e->idx.assign(shape->dep_idx, shape->dep_idx + nnz);
        e->vf.assign(shape->dep_vf, shape->dep_vf + nnz);
    }
    e->shape = *shape;
    e->shape.vertices = e->v.data();
    e->shape.facets = e->f.data();
    e->shape.dep_ptr = e->ptr.data();
    e->shape.dep_idx = nnz ? e->idx.data() : nullptr;
    e->shape.dep_vf = nnz ? e->vf.data() : nullptr;
    e->params = *params;
    atpm_status st = atpm_solve_footprint(&e->shape, &e->params, &e->footprint);
    if (st) return st;
    st = atpm_solve_create(S->ctx, &e->shape, &e->params, &e->proto);
    if (!st) st = atpm_geometry_shadow(e->proto);
    if (!st) st = atpm_scattering(e->proto);
    if (st) {
        if (e->proto) atpm_solve_destroy(e->proto);
        return st;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    S->shapes.push_back(std::move(e));
    *shape_id = (int32_t)S->shapes.size() - 1;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_server_submit(atpm_server* S, int32_t shape_id, float ti, int64_t* request_id) {
    if (!S || !request_id) return atpm::fail_status(ATPM_E_INVALID, "submit: bad arguments");
    if (!(ti >= 0.0f) || !std::isfinite(ti)) return atpm::fail_status(ATPM_E_INVALID, "submit: bad thermal inertia");
    std::lock_guard<std::mutex> lk(S->mu);
    if (shape_id < 0 || shape_id >= (int)S->shapes.size())
        return atpm::fail_status(ATPM_E_INVALID, "submit: unknown shape");
    if (S->shapes[shape_id]->footprint > S->budget)
        return atpm::fail_status(ATPM_E_BUDGET, "submit: request larger than the HBM budget");
    auto r = std::make_unique<Request>();
    r->id = S->next_id++;
    r->shape = shape_id;
    r->ti = ti;
    r->footprint = S->shapes[shape_id]->footprint;
    r->t_submit = now_s();
    if (S->t_first == 0) S->t_first = r->t_submit;
    *request_id = r->id;
    S->queue.push_back(r.get());
    S->all[r->id] = std::move(r);
    S->cv_work.notify_all();
    return ATPM_OK;
}

ATPM_API atpm_status atpm_server_cancel(atpm_server* S, int64_t id) {
    if (!S) return atpm::fail_status(ATPM_E_INVALID, "cancel: null server");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) return atpm::fail_status(ATPM_E_INVALID, "cancel: unknown request");
    it->second->cancelled = true;
    S->cv_work.notify_all();
    return ATPM_OK;
}

ATPM_API atpm_status atpm_server_wait(atpm_server* S, int64_t id, double timeout_s, float* stemp1, int32_t* nrev,
                                      double* latency_s) {
    if (!S) return atpm::fail_status(ATPM_E_INVALID, "wait: null server");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) return atpm::fail_status(ATPM_E_INVALID, "wait: unknown request");
    Request* r = it->second.get();
    const auto deadline = clock_t_::now() + std::chrono::duration<double>(timeout_s);
    if (!S->cv_done.wait_until(lk, deadline, [&] { return r->done; }))
        return atpm::fail_status(ATPM_E_STATE, "wait: timed out (request still running)");
    if (r->status) return atpm::fail_status(r->status, "request failed");
    if (stemp1) std::memcpy(stemp1, r->stemp1.data(), r->stemp1.size() * 4);
    if (nrev) *nrev = r->nrev;
    if (latency_s) *latency_s = r->t_done - r->t_submit;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_server_stats(atpm_server* S, double* p50_s, double* p99_s, double* facet_steps_per_s,
                                       int64_t* completed, uint64_t* resident_bytes) {
    if (!S) return atpm::fail_status(ATPM_E_INVALID, "stats: null server");
    std::lock_guard<std::mutex> lk(S->mu);
    std::vector<double> l = S->latencies;
    std::sort(l.begin(), l.end());
    auto pct = [&](double p) {
        if (l.empty()) return 0.0;
        const size_t i = std::min(l.size() - 1, (size_t)(p * (double)(l.size() - 1) + 0.5));
        return l[i];
    };
    if (p50_s) *p50_s = pct(0.50);
    if (p99_s) *p99_s = pct(0.99);
    const double span = S->t_last - S->t_first;
    if (facet_steps_per_s) *facet_steps_per_s = span > 0 ? (double)S->done_facet_steps / span : 0.0;
    if (completed) *completed = (int64_t)l.size();
    if (resident_bytes) *resident_bytes = S->resident;
    return ATPM_OK;
}

ATPM_API atpm_status atpm_server_destroy(atpm_server* S) {
    if (!S) return ATPM_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        S->cv_work.notify_all();
    }
    if (S->loop.joinable()) S->loop.join();
    cudaSetDevice(S->ctx->device);
    for (auto& e : S->shapes)
        if (e->proto) atpm_solve_destroy(e->proto);
    if (S->table) cudaFree(S->table);
    if (S->run_st) cudaStreamDestroy(S->run_st);
    if (S->setup_st) cudaStreamDestroy(S->setup_st);
    atpm_status st = S->loop_error;
    atpm_context* ctx = S->ctx;
    delete S;
    atpm_context_release(ctx);
    return st;
}

}  // extern "C"
