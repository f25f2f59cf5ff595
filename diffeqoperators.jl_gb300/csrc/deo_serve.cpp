// deo_serve.cpp -- a device-resident serving loop for method-of-lines solves
// (deo_serve_* in deo.h).  No reference counterpart: the reference leaves time
// stepping to OrdinaryDiffEq and has no serving layer; the right-hand side
// of each solve is a plan, i.e. the reference's (L)(du, u, p, t) = mul!(du, L, u)
// (DiffEqOperators.jl:67-76).
//
// Each request is K fixed SSP-RK3 steps (Shu-Osher) of du/dt = A u, and
// optionally K transposed steps from 2 u(T) for the gradient of ||u(T)||^2
// with respect to u0.  Its state is three device buffers, taken from the
// stream-ordered allocator at admission and returned after its result has
// been copied out; admission is FIFO under a byte budget.
//
// Two streams: `cs` runs the rounds; `xs` does the admissions' allocations
// and host-to-device copies, the results' device-to-host copies and the
// frees, ordered against `cs` by events, so copies overlap the rounds.
//
// deo_serve_pump does a round of bookkeeping and never waits for the device:
//   * requests whose result copy finished become DONE (deo_serve_poll hands
//     the result over);
//   * pending requests are admitted while their buffers fit the budget;
//   * while fewer than kDepth rounds are in flight, the next round is
//     enqueued: S = min(remaining steps) over the active requests (capped), so
//     no request finishes inside a round, and S steps of three batched stage
//     launches (libdeo's persistent work-list kernel, replayed from its CUDA
//     graph) advance EVERY active request, forward and transposed steps mixed.
//     Requests that finish at the end of the round have their state copied to
//     pinned host memory on the same stream (or, at the end of the forward
//     pass of a gradient request, scaled by 2 to seed the transposed steps).
// Rounds are therefore enqueued back to back: the host decides, from step
// counts alone, which requests leave after each round and which join, without
// synchronising with the device.  Every request's arithmetic is independent
// of the others (no cross-request reductions, a fixed per-point order), so
// its result is the same alone or in any mix.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "../../include/deo.h"
#include "deo_internal.h"

extern "C" int64_t deo_plan_points(const deo_plan* p);
extern "C" int deo_plan_dtype_code(const deo_plan* p);
extern "C" size_t deo_plan_table_bytes(const deo_plan* p);
extern "C" deo_status deo_set_error(deo_status s, const char* msg);

namespace {

constexpr int kDepth = 2;  // rounds in flight

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

enum class RS { Pending, Active, Retiring, Done, Rejected, Failed, Cancelled };

struct Req {
    int64_t rid = 0;
    const deo_plan* plan = nullptr;
    int K = 0;
    double dt = 0.0;
    bool grad = false;
    int64_t npts = 0;
    size_t state_bytes = 0;  // the three device buffers
    size_t vec_bytes = 0;
    RS st = RS::Pending;
    deo_status why = DEO_OK;
    int phase = 0;  // 0 forward, 1 transposed
    int step = 0;   // steps done in the phase
    void* u = nullptr;
    void* b1 = nullptr;
    void* b2 = nullptr;
    void* host_u = nullptr;  // pinned: u0 on the way in, u(T) on the way out
    void* host_g = nullptr;  // pinned: the gradient
    cudaEvent_t done_ev = nullptr;  // on xs: the result is in host memory
    double t_submit = 0.0, t_admit = 0.0, t_done = 0.0;
};

}  // namespace

struct deo_server {
    size_t budget = 0, in_use = 0;
    int dtype = 0;
    int max_steps = 64;
    cudaStream_t cs = nullptr;  // compute: the rounds (and a gradient request's seed)
    cudaStream_t xs = nullptr;  // copies: allocations, input and result copies, frees
    std::recursive_mutex mu;
    int64_t next_rid = 1;
    std::map<int64_t, Req> reqs;
    std::deque<int64_t> pending;
    std::vector<int64_t> active;
    std::vector<int64_t> retiring;
    deo_batch* stage[3] = {nullptr, nullptr, nullptr};
    bool stale = true;  // the active set (or a phase) changed since the batches were built
    std::vector<deo_batch*> graveyard;  // batches of earlier rounds, freed once the device is idle
    struct Round {
        cudaEvent_t start, end;  // timed
    };
    std::deque<Round> rounds;
    std::vector<cudaEvent_t> free_events, free_timed;
    double device_ms = 0.0;  // summed over retired rounds
    std::multimap<size_t, void*> pinned_pool;  // pinned host buffers by size, reused
    int inject_alloc_failures = 0;
    deo_serve_stats stats{};

    cudaEvent_t event() {
        if (!free_events.empty()) {
            cudaEvent_t e = free_events.back();
            free_events.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
        return e;
    }
    cudaEvent_t timed_event() {
        if (!free_timed.empty()) {
            cudaEvent_t e = free_timed.back();
            free_timed.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        return e;
    }
    // Makes `waiter` wait for the work enqueued on `on` so far.
    deo_status order(cudaStream_t on, cudaStream_t waiter) {
        cudaEvent_t e = event();
        if (!e) return deo_set_error(DEO_ERR_CUDA, "cudaEventCreate failed");
        cudaError_t err = cudaEventRecord(e, on);
        if (err == cudaSuccess) err = cudaStreamWaitEvent(waiter, e, 0);
        free_events.push_back(e);  // the wait has taken the event's state; it may be recorded again
        return err == cudaSuccess ? DEO_OK : deo_set_error(DEO_ERR_CUDA, cudaGetErrorString(err));
    }
    void* pinned(size_t bytes) {
        auto it = pinned_pool.lower_bound(bytes);
        if (it != pinned_pool.end() && it->first <= 2 * bytes) {
            void* p = it->second;
            pinned_pool.erase(it);
            return p;
        }
        void* p = nullptr;
        if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
        pinned_sizes[p] = bytes;
        return p;
    }
    void give_back(void* p) {
        if (p) pinned_pool.emplace(pinned_sizes[p], p);
    }
    std::map<void*, size_t> pinned_sizes;

    ~deo_server() {
        if (cs) cudaStreamSynchronize(cs);
        if (xs) cudaStreamSynchronize(xs);
        for (auto& kv : reqs) {
            Req& r = kv.second;
            if (r.u) cudaFreeAsync(r.u, xs);
            if (r.b1) cudaFreeAsync(r.b1, xs);
            if (r.b2) cudaFreeAsync(r.b2, xs);
            if (r.done_ev) cudaEventDestroy(r.done_ev);
            give_back(r.host_u);
            give_back(r.host_g);
        }
        if (xs) cudaStreamSynchronize(xs);
        for (deo_batch* b : stage)
            if (b) deo_batch_destroy(b);
        for (deo_batch* b : graveyard) deo_batch_destroy(b);
        for (const Round& q : rounds) {
            cudaEventDestroy(q.start);
            cudaEventDestroy(q.end);
        }
        for (cudaEvent_t e : free_events) cudaEventDestroy(e);
        for (cudaEvent_t e : free_timed) cudaEventDestroy(e);
        for (auto& kv : pinned_sizes) cudaFreeHost(kv.first);
        if (cs) cudaStreamDestroy(cs);
        if (xs) cudaStreamDestroy(xs);
    }

    // Frees the request's buffers on xs after the work enqueued so far on cs
    // (and, being on xs, after its result copy).
    deo_status release_device(Req& r) {
        const deo_status s = order(cs, xs);
        if (s != DEO_OK) return s;
        if (r.u) cudaFreeAsync(r.u, xs);
        if (r.b1) cudaFreeAsync(r.b1, xs);
        if (r.b2) cudaFreeAsync(r.b2, xs);
        r.u = r.b1 = r.b2 = nullptr;
        in_use -= r.state_bytes;
        return DEO_OK;
    }

    deo_status admit(Req& r) {
        if (inject_alloc_failures > 0) {
            --inject_alloc_failures;
            r.st = RS::Failed;
            r.why = DEO_ERR_OOM;
            ++stats.failed;
            return DEO_OK;
        }
        cudaError_t e = cudaMallocAsync(&r.u, r.vec_bytes, xs);
        if (e == cudaSuccess) e = cudaMallocAsync(&r.b1, r.vec_bytes, xs);
        if (e == cudaSuccess) e = cudaMallocAsync(&r.b2, r.vec_bytes, xs);
        if (e != cudaSuccess) {
            cudaGetLastError();
            if (r.u) cudaFreeAsync(r.u, xs);
            if (r.b1) cudaFreeAsync(r.b1, xs);
            r.u = r.b1 = r.b2 = nullptr;
            r.st = RS::Failed;
            r.why = DEO_ERR_OOM;
            ++stats.failed;
            return DEO_OK;
        }
        e = cudaMemcpyAsync(r.u, r.host_u, r.vec_bytes, cudaMemcpyHostToDevice, xs);
        if (e != cudaSuccess) return deo_set_error(DEO_ERR_CUDA, cudaGetErrorString(e));
        // the rounds enqueued from now on (the first with this request) wait
        // for the copy; the rounds already in flight do not
        const deo_status os = order(xs, cs);
        if (os != DEO_OK) return os;
        in_use += r.state_bytes;
        r.st = RS::Active;
        r.t_admit = now_s();
        active.push_back(r.rid);
        stale = true;
        ++stats.admitted;
        return DEO_OK;
    }

    // The three stage batches of one SSP-RK3 step (forward, or transposed for
    // requests in their second phase), for the current active set.
    deo_status rebuild() {
        for (deo_batch*& b : stage)
            if (b) {
                graveyard.push_back(b);
                b = nullptr;
            }
        std::vector<deo_stage> s1, s2, s3;
        for (int64_t id : active) {
            Req& r = reqs[id];
            const deo_plan* p = r.plan;
            if (r.phase == 0) {
                s1.push_back(deo_stage{p, nullptr, nullptr, r.u, r.b1, 0.0, 0.0, 1.0, r.dt, 0});
                s2.push_back(deo_stage{p, r.u, nullptr, r.b1, r.b2, 0.75, 0.0, 0.25, r.dt, 0});
                s3.push_back(deo_stage{p, r.u, nullptr, r.b2, r.u, 1.0 / 3.0, 0.0, 2.0 / 3.0, r.dt, 0});
            } else {
                s1.push_back(deo_stage{p, nullptr, nullptr, r.u, r.b2, 0.0, 0.0, 2.0 / 3.0, r.dt, 1});
                s2.push_back(deo_stage{p, nullptr, nullptr, r.b2, r.b1, 0.0, 0.0, 0.25, r.dt, 1});
                s3.push_back(deo_stage{p, r.u, r.b2, r.b1, r.u, 1.0 / 3.0, 0.75, 1.0, r.dt, 1});
            }
        }
        const std::vector<deo_stage>* sets[3] = {&s1, &s2, &s3};
        for (int k = 0; k < 3; ++k) {
            const deo_status s = deo_stage_batch_create((int)sets[k]->size(), sets[k]->data(), 0, 0, &stage[k]);
            if (s != DEO_OK) return s;
        }
        stale = false;
        ++stats.rebuilds;
        return DEO_OK;
    }

    deo_status round() {
        if (stale) {
            const deo_status s = rebuild();
            if (s != DEO_OK) return s;
        }
        int S = max_steps;
        for (int64_t id : active) {
            const Req& r = reqs[id];
            S = std::min(S, r.K - r.step);
        }
        S = std::max(S, 1);
        Round q{timed_event(), timed_event()};
        if (!q.start || !q.end) return deo_set_error(DEO_ERR_CUDA, "cudaEventCreate failed");
        cudaEventRecord(q.start, cs);
        for (int k = 0; k < S; ++k)
            for (deo_batch* b : stage) {
                const deo_status s = deo_batch_run(b, 1, cs);
                if (s != DEO_OK) return s;
            }
        stats.launches += 3 * (int64_t)S;
        stats.steps += S;
        ++stats.rounds;
        std::vector<int64_t> keep;
        for (int64_t id : active) {
            Req& r = reqs[id];
            r.step += S;
            if (r.step < r.K) {
                keep.push_back(id);
                continue;
            }
            stale = true;
            const deo_status os = order(cs, xs);  // the copy below reads the round's last state
            if (os != DEO_OK) return os;
            if (r.phase == 0) {
                cudaError_t e = cudaMemcpyAsync(r.host_u, r.u, r.vec_bytes, cudaMemcpyDeviceToHost, xs);
                if (e != cudaSuccess) return deo_set_error(DEO_ERR_CUDA, cudaGetErrorString(e));
                if (r.grad) {  // ubar(T) = 2 u(T) once u(T) is copied, then K transposed steps
                    const deo_status ws = order(xs, cs);
                    if (ws != DEO_OK) return ws;
                    const int ke = deo_k_scale(r.u, r.npts, dtype, 2.0, cs);
                    if (ke) return deo_set_error(DEO_ERR_CUDA, cudaGetErrorString((cudaError_t)ke));
                    r.phase = 1;
                    r.step = 0;
                    keep.push_back(id);
                    continue;
                }
            } else {
                cudaError_t e = cudaMemcpyAsync(r.host_g, r.u, r.vec_bytes, cudaMemcpyDeviceToHost, xs);
                if (e != cudaSuccess) return deo_set_error(DEO_ERR_CUDA, cudaGetErrorString(e));
            }
            r.done_ev = event();
            if (!r.done_ev) return deo_set_error(DEO_ERR_CUDA, "cudaEventCreate failed");
            cudaEventRecord(r.done_ev, xs);
            const deo_status rs = release_device(r);  // stream-ordered: after the copy
            if (rs != DEO_OK) return rs;
            r.st = RS::Retiring;
            retiring.push_back(id);
        }
        active.swap(keep);
        cudaEventRecord(q.end, cs);
        rounds.push_back(q);
        return DEO_OK;
    }

    deo_status pump() {
        // results whose copy finished
        std::vector<int64_t> still;
        for (int64_t id : retiring) {
            Req& r = reqs[id];
            const cudaError_t q = cudaEventQuery(r.done_ev);
            if (q == cudaSuccess) {
                r.st = RS::Done;
                r.t_done = now_s();
                free_events.push_back(r.done_ev);
                r.done_ev = nullptr;
                ++stats.completed;
            } else if (q == cudaErrorNotReady) {
                still.push_back(id);
            } else {
                return deo_set_error(DEO_ERR_CUDA, cudaGetErrorString(q));
            }
        }
        retiring.swap(still);
        while (!rounds.empty()) {
            const Round f = rounds.front();
            const cudaError_t q = cudaEventQuery(f.end);
            if (q == cudaErrorNotReady) break;
            if (q != cudaSuccess) return deo_set_error(DEO_ERR_CUDA, cudaGetErrorString(q));
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, f.start, f.end) == cudaSuccess) device_ms += ms;
            free_timed.push_back(f.start);
            free_timed.push_back(f.end);
            rounds.pop_front();
        }
        if (rounds.empty() && !graveyard.empty()) {  // the device no longer reads them
            for (deo_batch* b : graveyard) deo_batch_destroy(b);
            graveyard.clear();
        }
        // FIFO admission under the budget
        while (!pending.empty()) {
            Req& r = reqs[pending.front()];
            if (in_use + r.state_bytes > budget) break;
            pending.pop_front();
            const deo_status s = admit(r);
            if (s != DEO_OK) return s;
        }
        while (!active.empty() && (int)rounds.size() < kDepth) {
            const deo_status s = round();
            if (s != DEO_OK) return s;
        }
        stats.in_use_bytes = (int64_t)in_use;
        stats.device_us = (int64_t)(device_ms * 1e3);
        stats.active = (int64_t)active.size();
        stats.pending = (int64_t)pending.size();
        return DEO_OK;
    }
};

extern "C" deo_status deo_serve_create(size_t budget_bytes, deo_dtype dtype, int max_steps_per_round,
                                       deo_server** out) {
    if (!out) return deo_set_error(DEO_ERR_BAD_ARG, "null argument");
    *out = nullptr;
    if (dtype != DEO_F64 && dtype != DEO_F32) return deo_set_error(DEO_ERR_BAD_ARG, "unknown dtype");
    auto s = std::make_unique<deo_server>();
    s->budget = budget_bytes;
    s->dtype = dtype;
    s->max_steps = max_steps_per_round > 0 ? max_steps_per_round : 64;
    if (cudaStreamCreateWithFlags(&s->cs, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->xs, cudaStreamNonBlocking) != cudaSuccess)
        return deo_set_error(DEO_ERR_CUDA, "cudaStreamCreate failed");
    *out = s.release();
    return DEO_OK;
}

extern "C" deo_status deo_serve_submit(deo_server* s, const deo_request* q, int64_t* rid) {
    if (!s || !q || !rid || !q->plan || !q->u0) return deo_set_error(DEO_ERR_BAD_ARG, "null argument");
    if (q->nsteps < 1 || !(q->dt > 0.0)) return deo_set_error(DEO_ERR_BAD_ARG, "need nsteps >= 1 and dt > 0");
    if (deo_plan_dtype_code(q->plan) != s->dtype)
        return deo_set_error(DEO_ERR_BAD_ARG, "the request's plan has another dtype than the server");
    std::lock_guard<std::recursive_mutex> lk(s->mu);
    Req r;
    r.rid = s->next_rid++;
    r.plan = q->plan;
    r.K = q->nsteps;
    r.dt = q->dt;
    r.grad = q->want_grad != 0;
    r.npts = deo_plan_points(q->plan);
    r.vec_bytes = (size_t)r.npts * (s->dtype == DEO_F64 ? 8 : 4);
    // counted against the budget: the three state buffers, the plan's device tables, and the
    // request's entries in the three stage batches (work items of at least 1024 points)
    r.state_bytes = 3 * r.vec_bytes + deo_plan_table_bytes(q->plan) +
                    3 * (sizeof(deo::StageDev) + ((size_t)r.npts / 1024 + 1) * sizeof(deo::WorkItem));
    r.t_submit = now_s();
    *rid = r.rid;
    ++s->stats.submitted;
    if (r.state_bytes > s->budget) {
        r.st = RS::Rejected;
        r.why = DEO_ERR_REJECTED;
        ++s->stats.rejected;
        s->reqs.emplace(r.rid, r);
        return deo_set_error(DEO_ERR_REJECTED, "request larger than the server's device-memory budget");
    }
    r.host_u = s->pinned(r.vec_bytes);
    if (r.grad) r.host_g = s->pinned(r.vec_bytes);
    if (!r.host_u || (r.grad && !r.host_g)) {
        s->give_back(r.host_u);
        s->give_back(r.host_g);
        return deo_set_error(DEO_ERR_OOM, "pinned host staging buffer");
    }
    std::memcpy(r.host_u, q->u0, r.vec_bytes);
    s->pending.push_back(r.rid);
    s->reqs.emplace(r.rid, r);
    return DEO_OK;
}

extern "C" deo_status deo_serve_pump(deo_server* s) {
    if (!s) return deo_set_error(DEO_ERR_BAD_ARG, "null server");
    std::lock_guard<std::recursive_mutex> lk(s->mu);
    return s->pump();
}

extern "C" deo_status deo_serve_poll(deo_server* s, int64_t rid, void* uT, void* grad, double* latency_s) {
    if (!s) return deo_set_error(DEO_ERR_BAD_ARG, "null server");
    std::lock_guard<std::recursive_mutex> lk(s->mu);
    auto it = s->reqs.find(rid);
    if (it == s->reqs.end()) return deo_set_error(DEO_ERR_BAD_ARG, "unknown (or already collected) request");
    Req& r = it->second;
    deo_status out = DEO_OK;
    switch (r.st) {
        case RS::Pending:
        case RS::Active:
        case RS::Retiring:
            return DEO_ERR_NOT_READY;
        case RS::Done:
            if (uT) std::memcpy(uT, r.host_u, r.vec_bytes);
            if (grad && r.grad) std::memcpy(grad, r.host_g, r.vec_bytes);
            if (latency_s) *latency_s = r.t_done - r.t_submit;
            break;
        case RS::Rejected:
            out = deo_set_error(DEO_ERR_REJECTED, "request larger than the server's device-memory budget");
            break;
        case RS::Failed:
            out = deo_set_error(r.why, "device memory for the request's state could not be allocated");
            break;
        case RS::Cancelled:
            out = deo_set_error(DEO_ERR_BAD_ARG, "request cancelled");
            break;
    }
    s->give_back(r.host_u);
    s->give_back(r.host_g);
    s->reqs.erase(it);
    return out;
}

extern "C" deo_status deo_serve_cancel(deo_server* s, int64_t rid) {
    if (!s) return deo_set_error(DEO_ERR_BAD_ARG, "null server");
    std::lock_guard<std::recursive_mutex> lk(s->mu);
    auto it = s->reqs.find(rid);
    if (it == s->reqs.end()) return deo_set_error(DEO_ERR_BAD_ARG, "unknown (or already collected) request");
    Req& r = it->second;
    if (r.st == RS::Pending) {
        s->pending.erase(std::find(s->pending.begin(), s->pending.end(), rid));
    } else if (r.st == RS::Active) {
        // leaves before the next round; its buffers go back after the rounds already enqueued
        s->active.erase(std::find(s->active.begin(), s->active.end(), rid));
        const deo_status rs = s->release_device(r);
        if (rs != DEO_OK) return rs;
        s->stale = true;
    } else {
        return deo_set_error(DEO_ERR_BAD_ARG, "request already finished");
    }
    r.st = RS::Cancelled;
    ++s->stats.cancelled;
    return DEO_OK;
}

extern "C" deo_status deo_serve_stats_get(deo_server* s, deo_serve_stats* out) {
    if (!s || !out) return deo_set_error(DEO_ERR_BAD_ARG, "null argument");
    std::lock_guard<std::recursive_mutex> lk(s->mu);
    *out = s->stats;
    return DEO_OK;
}

extern "C" deo_status deo_serve_inject_alloc_failures(deo_server* s, int n) {
    if (!s || n < 0) return deo_set_error(DEO_ERR_BAD_ARG, "bad argument");
    std::lock_guard<std::recursive_mutex> lk(s->mu);
    s->inject_alloc_failures = n;
    return DEO_OK;
}

extern "C" void deo_serve_destroy(deo_server* s) { delete s; }
