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
    std::vector<atpm_solve*> pool;  // retired requests' solves, re-seeded from proto on admission
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
    bool pooled = false;  // solve taken from its shape's pool (re-seeded, not cloned)
    int last_rev = 0;     // revolutions done after the last tick
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
    atpm::BatchPlan plan;      // device table of the resident set, rebuilt when the set changes
    std::vector<int64_t> plan_ids;  // the requests the table was built for (ids are never reused)
    int* prog_dev = nullptr;   // per-tick progress records (atpm::launch_progress)
    int* prog_host = nullptr;  // page-locked read-back of them
    size_t prog_cap = 0;       // records the buffers hold
    uint64_t pooled = 0;       // bytes held by pooled solves (counted against the budget)
    bool pooling = true;       // ATPM_SERVER_POOL=0: retired solves are freed, admissions clone
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
    atpm_solve* s = r->solve;
    // a device copy of the prototype: forcing and (shared) tensor-core tiles
    // come along, no host work on the shape; a pooled solve of the shape
    // takes the prototype's state by device copies, without allocating
    atpm_status st = s ? atpm::solve_refresh(s, sh->proto) : atpm_solve_clone(sh->proto, &s);
    if (!st) st = atpm_set_thermal_inertia(s, r->ti);
    if (!st && r->ti != 0.0f) st = atpm_initialise_temperatures(s);
    if (st) {
        if (s) atpm_solve_destroy(s);
        r->solve = nullptr;
        return st;
    }
    r->solve = s;
    r->last_rev = 0;  // atpm_set_thermal_inertia restarts the revolution count
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
        if (S->pooling && !S->stop && !st) {
            S->shapes[r->shape]->pool.push_back(r->solve);
            S->pooled += r->footprint;
        } else {
            atpm_solve_destroy(r->solve);
        }
        r->solve = nullptr;
    }
    r->status = st;
    r->t_done = now_s();
    r->done = true;
}

// facet-steps of the revolutions a tick advanced a solve by: revolutions
// last_rev .. rev - 1, a frozen facet counted only while active; win holds
// the convergence counts of revolutions rev - W .. rev - 1
int64_t tick_facet_steps(const atpm_solve* s, int last_rev, int rev, const int* win, int W) {
    const int nf = s->nf, ntau = s->P.ntau;
    const bool all_active = !s->P.freeze || s->ti == 0.0f;
    int64_t fs = 0;
    for (int r = last_rev; r < rev; ++r) {
        int active = nf;
        if (!all_active && r - 1 > 5) {
            const int j = (r - 1) - (rev - W);
            active = nf - (j >= 0 && j < W ? win[j] : 0);
        }
        fs += (int64_t)active * ntau;
    }
    return fs;
}

void run_loop(atpm_server* S) {
    cudaSetDevice(S->ctx->device);
    std::vector<atpm_solve*> evict;
    const int W = S->revs_per_tick + 1;  // counts of the revolutions a tick can add, and the one before
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
                ShapeEntry* sh = S->shapes[r->shape].get();
                if (!sh->pool.empty()) {
                    // the memory of a pooled solve of this shape is already held
                    r->solve = sh->pool.back();
                    sh->pool.pop_back();
                    S->pooled -= r->footprint;
                } else {
                    // pooled solves of other shapes give their memory back first
                    for (auto& e : S->shapes) {
                        while (S->resident + S->pooled + r->footprint > S->budget && !e->pool.empty()) {
                            evict.push_back(e->pool.back());
                            e->pool.pop_back();
                            S->pooled -= e->footprint;
                        }
                    }
                    if (S->resident + S->pooled + r->footprint > S->budget) break;  // wait for memory to free up
                }
                S->queue.pop_front();
                S->resident += r->footprint;
                to_admit.push_back(r);
            }
        }
        for (atpm_solve* x : evict) atpm_solve_destroy(x);
        evict.clear();
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
        // one tick: K revolutions of every resident solve in shared launches;
        // the batch table is rebuilt only when the resident set changed
        std::vector<atpm_solve*> sv;
        std::vector<int64_t> ids;
        for (Request* r : act) {
            sv.push_back(r->solve);
            ids.push_back(r->id);
        }
        atpm_status st = ATPM_OK;
        if (ids != S->plan_ids) {
            // a new set (a solve's address may be reused, and a pooled solve
            // carries its new request's parameters): rebuild the table
            st = atpm::batch_plan(sv.data(), (int)sv.size(), S->plan, S->run_st);
            S->plan_ids = st ? std::vector<int64_t>() : ids;
        }
        const size_t rec = (size_t)(5 + W);
        if (!st && act.size() > S->prog_cap) {
            if (S->prog_dev) cudaFree(S->prog_dev);
            if (S->prog_host) cudaFreeHost(S->prog_host);
            S->prog_dev = nullptr;
            S->prog_host = nullptr;
            S->prog_cap = 0;
            const size_t cap = act.size() * 2;
            if (cudaMalloc((void**)&S->prog_dev, cap * rec * 4) != cudaSuccess ||
                cudaMallocHost((void**)&S->prog_host, cap * rec * 4) != cudaSuccess) {
                S->loop_error = atpm::fail_status(ATPM_E_NOMEM, "server: progress buffers");
                break;
            }
            S->prog_cap = cap;
        }
        if (!st) st = atpm::batch_plan_step(S->plan, S->revs_per_tick, S->run_st);
        // every solve's progress in one gather and one read-back
        if (!st && atpm::launch_progress(S->plan.b, W, S->prog_dev, S->run_st))
            st = atpm::fail_status(ATPM_E_CUDA, "server: progress gather launch");
        if (!st && (cudaMemcpyAsync(S->prog_host, S->prog_dev, act.size() * rec * 4, cudaMemcpyDeviceToHost,
                                    S->run_st) != cudaSuccess ||
                    cudaStreamSynchronize(S->run_st) != cudaSuccess))
            st = atpm::fail_status(ATPM_E_CUDA, "server: revolution tick failed");
        std::lock_guard<std::mutex> lk(S->mu);
        std::vector<Request*> keep;
        for (size_t i = 0; i < act.size(); ++i) {
            Request* r = act[i];
            if (st) {
                S->resident -= r->footprint;
                retire(S, r, st);
                continue;
            }
            const int* p = S->prog_host + i * rec;
            const int rev = p[0], active = p[1], status = p[4];
            const int64_t fs = tick_facet_steps(r->solve, r->last_rev, rev, p + 5, W);
            r->last_rev = rev;
            r->facet_steps += fs;
            S->done_facet_steps += fs;
            r->solve->last_nrev = rev;
            atpm_status rs = ATPM_OK;
            if (status & atpm::ST_NONFINITE) rs = ATPM_E_NONFINITE;
            else if (status & (atpm::ST_NEWTON_CAP | atpm::ST_TC_TIMEOUT)) rs = ATPM_E_ITERATION;
            if (!active || rs || r->cancelled) {
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
    {
        const char* e = std::getenv("ATPM_SERVER_POOL");
        S->pooling = !(e && e[0] == '0');
    }
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
    // the result is handed over once: the request (and its host copy of the
    // temperatures) is forgotten, so a long stream does not accumulate them
    const atpm_status rs = r->status;
    if (!rs) {
        if (stemp1) std::memcpy(stemp1, r->stemp1.data(), r->stemp1.size() * 4);
        if (nrev) *nrev = r->nrev;
        if (latency_s) *latency_s = r->t_done - r->t_submit;
    }
    S->all.erase(it);
    if (rs) return atpm::fail_status(rs, "request failed");
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
    for (auto& e : S->shapes) {
        for (atpm_solve* x : e->pool) atpm_solve_destroy(x);
        e->pool.clear();
        if (e->proto) atpm_solve_destroy(e->proto);
    }
    atpm::batch_plan_free(S->plan);
    if (S->prog_dev) cudaFree(S->prog_dev);
    if (S->prog_host) cudaFreeHost(S->prog_host);
    if (S->run_st) cudaStreamDestroy(S->run_st);
    if (S->setup_st) cudaStreamDestroy(S->setup_st);
    atpm_status st = S->loop_error;
    atpm_context* ctx = S->ctx;
    delete S;
    atpm_context_release(ctx);
    return st;
}

}  // extern "C"
