// Continuous-batching serving loop over the batch engine.
//
// Requests ("simulate this mesh for K steps, return the final positions")
// are prepared on host worker threads (validation, element order, patch
// layout, gather tables), admitted in arrival order as soon as the HBM
// budget and a mesh slot allow, and stepped together with every other
// admitted mesh: each launch advances all of them by up to
// max_steps_per_launch steps (never past the nearest finishing request).
// A request that has run its K steps has its positions copied out, its slot
// and memory freed, and its latency (submission to completion) recorded;
// requests that arrive meanwhile join at the next launch boundary. The batch
// handle is used by the scheduler thread only.
//
// Admission policy: strict arrival order with head-of-line blocking -- the
// oldest waiting request is admitted as soon as a slot and a contiguous
// block of the HBM budget fit it, and nothing behind it is admitted first
// (a request larger than the whole budget fails instead of blocking).
// Requests can be cancelled (dropped from the queue at once, or removed from
// the GPU at the next launch boundary) and evicted (their state saved to host
// memory and their slot freed at the next launch boundary; they re-enter the
// queue behind the waiting requests and continue bit-exactly once admitted
// again).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "batch_internal.h"

namespace sgb {
void set_last_error(const std::string& msg);
}

using namespace sgb;
using Clock = std::chrono::steady_clock;

namespace {

struct Pending {
    sgb_request req;
    uint64_t seq = 0;
    Clock::time_point submitted;
    PreparedMesh pm;
    int prep_rc = SGB_OK;
    std::string prep_err;
    bool prepared = false;
    bool in_worker = false;  // a preparation worker holds it
    bool cancelled = false;
    // an evicted request: the state to resume from and the steps left
    bool resume = false;
    std::vector<double> sx, sv;
    long long saved_steps = 0;
    int remaining = 0;
};

struct Running {
    sgb_request req;
    uint64_t id = 0;
    int slot = -1;
    int remaining = 0;
    int n_steps = 0;
    long long tets = 0;
    double* out = nullptr;
    Clock::time_point submitted, admitted;
};

double ms_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

struct sgb_server {
    sgb_batch* batch = nullptr;
    int max_chunk = 8;
    std::mutex mu;
    std::condition_variable cv_prep, cv_sched, cv_idle;
    std::deque<Pending*> incoming;         // waiting for a preparation worker
    std::map<uint64_t, Pending*> ordered;  // every submitted, not yet admitted request, by arrival
    uint64_t next_seq = 0;
    std::vector<Running> running;          // scheduler thread only
    std::vector<sgb_completion> done;      // completions not yet polled
    std::vector<double> latencies;         // all completions
    std::vector<double> step_ms;           // one entry per step of every launch
    std::set<uint64_t> running_ids;        // requests on the GPU (kept by the scheduler)
    std::set<uint64_t> cancel_running, evict_running;  // asked for, done at the next launch boundary
    long long tet_steps = 0;
    long long completed = 0, failed = 0, submitted = 0, launches = 0, cancelled = 0, evicted = 0;
    double busy_s = 0.0;
    Clock::time_point first_submit;
    bool have_first = false;
    bool stop = false;
    std::vector<std::thread> workers;
    std::thread scheduler;
    std::atomic<int> in_flight{0};
};

static void complete(sgb_server* S, uint64_t id, int status, Clock::time_point submitted, Clock::time_point admitted,
                     int iters, long long tets, int steps);

static void prep_worker(sgb_server* S)
{
    for (;;) {
        Pending* p = nullptr;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_prep.wait(lk, [&] { return S->stop || !S->incoming.empty(); });
            if (S->stop && S->incoming.empty()) return;
            p = S->incoming.front();
            S->incoming.pop_front();
            p->in_worker = true;
        }
        const int rc = prepare_mesh(&p->req.mesh, S->batch->pe, S->batch->rs, p->pm, S->batch->fused_rhs);
        std::string err = rc ? std::string(sgb_last_error()) : std::string();
        bool drop = false;
        {
            std::lock_guard<std::mutex> lk(S->mu);
            p->prep_rc = rc;
            p->prep_err = err;
            p->prepared = true;
            p->in_worker = false;
            if (p->cancelled) {  // cancelled while it was being prepared
                S->ordered.erase(p->seq);
                drop = true;
            }
        }
        if (drop) {
            complete(S, p->req.id, SGB_ERR_CANCELLED, p->submitted, Clock::now(), 0, 0, 0);
            delete p;
            continue;
        }
        S->cv_sched.notify_one();
    }
}

static void complete(sgb_server* S, uint64_t id, int status, Clock::time_point submitted, Clock::time_point admitted,
                     int iters, long long tets, int steps)
{
    const auto now = Clock::now();
    sgb_completion c{};
    c.id = id;
    c.status = status;
    c.latency_ms = ms_between(submitted, now);
    c.queue_ms = ms_between(submitted, admitted);
    c.cg_iterations_last = iters;
    c.n_tets = tets;
    c.n_steps = steps;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->done.push_back(c);
        if (status == SGB_OK) {
            S->latencies.push_back(c.latency_ms);
            S->completed++;
            S->tet_steps += tets * steps;
        } else if (status == SGB_ERR_CANCELLED) {
            S->cancelled++;
        } else {
            S->failed++;
        }
        S->in_flight--;
    }
    S->cv_idle.notify_all();
}

// Cancellations and evictions of running requests, at a launch boundary
// (scheduler thread).
static void handle_running_requests(sgb_server* S)
{
    sgb_batch* B = S->batch;
    std::set<uint64_t> cancel, evict;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        cancel.swap(S->cancel_running);
        evict.swap(S->evict_running);
    }
    if (cancel.empty() && evict.empty()) return;
    std::vector<Running> keep;
    for (auto& r : S->running) {
        if (cancel.count(r.id)) {
            sgb_batch_remove_mesh(B, r.slot);
            {
                std::lock_guard<std::mutex> lk(S->mu);
                S->running_ids.erase(r.id);
            }
            complete(S, r.id, SGB_ERR_CANCELLED, r.submitted, r.admitted, 0, r.tets, 0);
        } else if (evict.count(r.id)) {
            Pending* p = new Pending();
            p->req = r.req;
            p->submitted = r.submitted;
            p->resume = true;
            p->remaining = r.remaining;
            p->sx.resize(3 * (size_t)r.req.mesh.n_nodes);
            p->sv.resize(3 * (size_t)r.req.mesh.n_nodes);
            const int rc = sgb_batch_save_mesh(B, r.slot, p->sx.data(), p->sv.data(), &p->saved_steps);
            sgb_batch_remove_mesh(B, r.slot);
            if (rc != SGB_OK) {
                delete p;
                {
                    std::lock_guard<std::mutex> lk(S->mu);
                    S->running_ids.erase(r.id);
                }
                complete(S, r.id, rc, r.submitted, r.admitted, 0, r.tets, 0);
                continue;
            }
            {
                // back into the queue, behind the requests already waiting;
                // the mesh layout is prepared again from its description
                std::lock_guard<std::mutex> lk(S->mu);
                S->running_ids.erase(r.id);
                p->seq = S->next_seq++;
                S->ordered[p->seq] = p;
                S->incoming.push_back(p);
                S->evicted++;
            }
            S->cv_prep.notify_one();
        } else {
            keep.push_back(r);
        }
    }
    S->running.swap(keep);
}

static void scheduler_loop(sgb_server* S)
{
    sgb_batch* B = S->batch;
    for (;;) {
        handle_running_requests(S);
        // admission, in arrival order, while the head fits
        std::vector<Pending*> to_admit;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            if (S->running.empty())
                S->cv_sched.wait(lk, [&] {
                    return S->stop || (!S->ordered.empty() && S->ordered.begin()->second->prepared);
                });
            if (S->stop && S->running.empty()) return;
            while (!S->ordered.empty() && S->ordered.begin()->second->prepared) {
                Pending* p = S->ordered.begin()->second;
                if (p->prep_rc == SGB_OK && p->req.n_steps > 0) {
                    // budget and slot check before taking it off the queue;
                    // a request larger than the whole budget fails rather
                    // than blocking the queue
                    bool slot_free = false;
                    for (auto& m : B->slots)
                        if (!m.active) {
                            slot_free = true;
                            break;
                        }
                    const bool fits = slot_free && B->arena.largest_free() >= p->pm.bytes;
                    if (!fits && !(S->running.empty() && p->pm.bytes > B->arena.size)) break;
                }
                S->ordered.erase(S->ordered.begin());
                to_admit.push_back(p);
                break;  // one per pass: the budget changes with each admission
            }
        }
        for (Pending* p : to_admit) {
            const auto t_admit = Clock::now();
            if (p->prep_rc != SGB_OK) {
                complete(S, p->req.id, p->prep_rc, p->submitted, t_admit, 0, 0, 0);
                delete p;
                continue;
            }
            if (p->req.n_steps <= 0) {
                // nothing to simulate: the rest positions are the answer
                std::copy(p->pm.rest.begin(), p->pm.rest.end(), p->req.positions_out_host);
                complete(S, p->req.id, SGB_OK, p->submitted, t_admit, 0, p->pm.E, 0);
                delete p;
                continue;
            }
            int slot = -1;
            int rc = admit_prepared(B, p->pm, &slot);
            if (rc == SGB_OK && p->resume) {
                rc = sgb_batch_restore_mesh(B, slot, p->sx.data(), p->sv.data(), p->saved_steps);
                if (rc != SGB_OK) sgb_batch_remove_mesh(B, slot);
            }
            if (rc != SGB_OK) {
                complete(S, p->req.id, rc, p->submitted, t_admit, 0, 0, 0);
            } else {
                Running r;
                r.req = p->req;
                r.id = p->req.id;
                r.slot = slot;
                r.remaining = p->resume ? p->remaining : p->req.n_steps;
                r.n_steps = p->req.n_steps;
                r.tets = p->pm.E;
                r.out = p->req.positions_out_host;
                r.submitted = p->submitted;
                r.admitted = t_admit;
                S->running.push_back(r);
                std::lock_guard<std::mutex> lk(S->mu);
                S->running_ids.insert(r.id);
            }
            delete p;
        }
        if (!to_admit.empty()) continue;  // try to admit more before stepping
        if (S->running.empty()) continue;
        // step every admitted mesh up to the nearest finish
        int k = S->max_chunk;
        for (auto& r : S->running) k = std::min(k, r.remaining);
        const auto t0 = Clock::now();
        int rc = sgb_batch_step(B, k);
        std::vector<Running> finished, keep;
        for (auto& r : S->running) {
            r.remaining -= k;
            (r.remaining == 0 ? finished : keep).push_back(r);
        }
        std::vector<int> iters(finished.size(), 0);
        for (size_t i = 0; i < finished.size() && rc == SGB_OK; ++i)
            rc = sgb_batch_get_positions_async(B, finished[i].slot, finished[i].out);
        cudaError_t ce = cudaStreamSynchronize(B->stream);
        const auto t1 = Clock::now();
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->busy_s += std::chrono::duration<double>(t1 - t0).count();
            S->launches++;
            const double per_step = ms_between(t0, t1) / k;
            for (int i = 0; i < k; ++i) S->step_ms.push_back(per_step);
        }
        for (size_t i = 0; i < finished.size(); ++i) {
            long long steps = 0;
            int st = (rc == SGB_OK && ce == cudaSuccess) ? SGB_OK : SGB_ERR_CUDA;
            if (st == SGB_OK) {
                int it = 0;
                double res = 0;
                st = sgb_batch_mesh_stats(B, finished[i].slot, &it, &res, &steps);
                iters[i] = it;
            }
            sgb_batch_remove_mesh(B, finished[i].slot);
            {
                std::lock_guard<std::mutex> lk(S->mu);
                S->running_ids.erase(finished[i].id);
            }
            complete(S, finished[i].id, st, finished[i].submitted, finished[i].admitted, iters[i], finished[i].tets,
                     finished[i].n_steps);
        }
        S->running.swap(keep);
        if (rc != SGB_OK || ce != cudaSuccess) {
            // a failed launch fails every running request; the server keeps serving new ones
            for (auto& r : S->running) {
                sgb_batch_remove_mesh(B, r.slot);
                {
                    std::lock_guard<std::mutex> lk(S->mu);
                    S->running_ids.erase(r.id);
                }
                complete(S, r.id, SGB_ERR_CUDA, r.submitted, r.admitted, 0, r.tets, 0);
            }
            S->running.clear();
        }
    }
}

extern "C" {

int sgb_server_create(sgb_server_t** out, int precision, size_t hbm_budget_bytes, int max_meshes,
                      int max_cg_iterations, int prep_threads, int max_steps_per_launch)
{
    if (!out) return (set_last_error("sgb_server_create: out is NULL"), SGB_ERR_INVALID_ARGUMENT);
    *out = nullptr;
    if (prep_threads < 1 || max_steps_per_launch < 1)
        return (set_last_error("sgb_server_create: need at least one preparation thread and one step per launch"),
                SGB_ERR_INVALID_ARGUMENT);
    sgb_batch* B = nullptr;
    int rc = sgb_batch_create(&B, precision, hbm_budget_bytes, max_meshes, max_cg_iterations);
    if (rc) return rc;
    sgb_server* S = new sgb_server();
    S->batch = B;
    S->max_chunk = max_steps_per_launch;
    int dev = 0;
    cudaGetDevice(&dev);
    for (int i = 0; i < prep_threads; ++i) S->workers.emplace_back(prep_worker, S);
    S->scheduler = std::thread([S, dev] {
        cudaSetDevice(dev);
        scheduler_loop(S);
    });
    *out = S;
    return SGB_OK;
}

int sgb_server_submit(sgb_server_t* S, const sgb_request* req)
{
    if (!S || !req || !req->positions_out_host)
        return (set_last_error("sgb_server_submit: NULL argument"), SGB_ERR_INVALID_ARGUMENT);
    Pending* p = new Pending();
    p->req = *req;
    p->submitted = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) {
            delete p;
            return (set_last_error("sgb_server_submit: the server is shutting down"), SGB_ERR_INVALID_ARGUMENT);
        }
        p->seq = S->next_seq++;
        S->ordered[p->seq] = p;
        S->incoming.push_back(p);
        S->submitted++;
        if (!S->have_first) {
            S->first_submit = p->submitted;
            S->have_first = true;
        }
    }
    S->in_flight++;
    S->cv_prep.notify_one();
    return SGB_OK;
}

int sgb_server_poll(sgb_server_t* S, sgb_completion* out, int max_out, int* n_out)
{
    if (!S || !n_out || (max_out > 0 && !out))
        return (set_last_error("sgb_server_poll: NULL argument"), SGB_ERR_INVALID_ARGUMENT);
    std::lock_guard<std::mutex> lk(S->mu);
    const int n = std::min<int>(max_out, (int)S->done.size());
    for (int i = 0; i < n; ++i) out[i] = S->done[(size_t)i];
    S->done.erase(S->done.begin(), S->done.begin() + n);
    *n_out = n;
    return SGB_OK;
}

int sgb_server_wait_idle(sgb_server_t* S, double timeout_s)
{
    if (!S) return (set_last_error("sgb_server_wait_idle: NULL server"), SGB_ERR_INVALID_ARGUMENT);
    std::unique_lock<std::mutex> lk(S->mu);
    const auto deadline = Clock::now() + std::chrono::duration<double>(timeout_s);
    while (S->in_flight.load() > 0) {
        if (S->cv_idle.wait_until(lk, deadline) == std::cv_status::timeout && S->in_flight.load() > 0)
            return (set_last_error("sgb_server_wait_idle: timed out"), SGB_ERR_NOT_FOUND);
    }
    return SGB_OK;
}

int sgb_server_get_stats(sgb_server_t* S, sgb_server_stats* st)
{
    if (!S || !st) return (set_last_error("sgb_server_get_stats: NULL argument"), SGB_ERR_INVALID_ARGUMENT);
    std::lock_guard<std::mutex> lk(S->mu);
    std::vector<double> l = S->latencies;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) {
        if (l.empty()) return 0.0;
        size_t i = (size_t)std::ceil(q * (double)l.size()) - 1;
        return l[std::min(i, l.size() - 1)];
    };
    st->submitted = S->submitted;
    st->completed = S->completed;
    st->failed = S->failed;
    st->tet_steps = S->tet_steps;
    st->p50_ms = pct(0.50);
    st->p99_ms = pct(0.99);
    st->max_ms = l.empty() ? 0.0 : l.back();
    st->busy_s = S->busy_s;
    st->wall_s = S->have_first ? std::chrono::duration<double>(Clock::now() - S->first_submit).count() : 0.0;
    std::vector<double> sm = S->step_ms;
    std::sort(sm.begin(), sm.end());
    auto spct = [&](double q) {
        if (sm.empty()) return 0.0;
        size_t i = (size_t)std::ceil(q * (double)sm.size()) - 1;
        return sm[std::min(i, sm.size() - 1)];
    };
    st->step_p50_ms = spct(0.50);
    st->step_p99_ms = spct(0.99);
    st->launches = S->launches;
    st->cancelled = S->cancelled;
    st->evicted = S->evicted;
    return SGB_OK;
}

int sgb_server_cancel(sgb_server_t* S, uint64_t id)
{
    if (!S) return (set_last_error("sgb_server_cancel: NULL server"), SGB_ERR_INVALID_ARGUMENT);
    Pending* drop = nullptr;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        for (auto it = S->ordered.begin(); it != S->ordered.end(); ++it) {
            Pending* p = it->second;
            if (p->req.id != id || p->cancelled) continue;
            if (p->in_worker) {
                p->cancelled = true;  // the worker completes it when it is done preparing
                return SGB_OK;
            }
            auto q = std::find(S->incoming.begin(), S->incoming.end(), p);
            if (q != S->incoming.end()) S->incoming.erase(q);
            S->ordered.erase(it);
            drop = p;
            break;
        }
        if (!drop) {
            if (S->running_ids.count(id) && !S->cancel_running.count(id)) {
                S->cancel_running.insert(id);
                return SGB_OK;
            }
            return (set_last_error("sgb_server_cancel: no queued or running request with that id"),
                    SGB_ERR_NOT_FOUND);
        }
    }
    complete(S, drop->req.id, SGB_ERR_CANCELLED, drop->submitted, Clock::now(), 0, 0, 0);
    delete drop;
    S->cv_sched.notify_one();
    return SGB_OK;
}

int sgb_server_evict(sgb_server_t* S, uint64_t id)
{
    if (!S) return (set_last_error("sgb_server_evict: NULL server"), SGB_ERR_INVALID_ARGUMENT);
    std::lock_guard<std::mutex> lk(S->mu);
    if (!S->running_ids.count(id) || S->cancel_running.count(id))
        return (set_last_error("sgb_server_evict: no running request with that id"), SGB_ERR_NOT_FOUND);
    S->evict_running.insert(id);
    return SGB_OK;
}

int sgb_server_destroy(sgb_server_t* S)
{
    if (!S) return SGB_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_prep.notify_all();
    S->cv_sched.notify_all();
    for (auto& t : S->workers) t.join();
    if (S->scheduler.joinable()) S->scheduler.join();
    for (auto& kv : S->ordered) delete kv.second;
    sgb_batch_destroy(S->batch);
    delete S;
    return SGB_OK;
}

}  // extern "C"
