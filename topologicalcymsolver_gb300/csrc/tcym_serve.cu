// Serving loop: continuous batching of independent trajectory requests.
//
// The reference runs one trajectory per process and seed (SU2Solver.cpp:148-169,
// SphaleronSimulation.cpp:571-616).  Here two kinds of host threads share one
// GPU:
//
//   * preparer threads take requests in arrival order while the device-memory
//     budget and the slot limit allow, and build each one's initial state on the
//     request's own stream: U = 1, E ~ N(0, T) from the request's Philox field
//     stream, Gauss-restored in the request's own storage -- the restore queues
//     its iterations in batches and learns of convergence from a device-side flag;
//   * the tick thread owns the running ensemble: at each tick boundary it joins
//     the prepared requests, advances every running request `stride` steps in
//     the ensemble's batched launches, appends (steps, N_CS) per request and
//     retires the finished ones, which frees their memory for the next arrivals.
//
// So a tick never waits for a preparation: their kernels share the device (the
// ensemble's streams have the higher priority), and the request lattices take
// their memory from a stream-ordered pool, whose allocations and releases do
// not synchronise the device the way cudaMalloc and cudaFree do.  Every wait
// has a time limit.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/tcym.h"
#include "tcym_internal.h"

namespace {

using Clock = std::chrono::steady_clock;
constexpr int kPreparers = 2;         // preparation threads
constexpr size_t kTickRecord = 8192;  // tick records kept for tcym_server_ticks

struct Req {
    tcym_request spec;
    int status = TCYM_REQ_QUEUED;
    int steps_done = 0;
    int target = 0;                 // steps rounded up to a multiple of the stride
    size_t footprint = 0;           // device bytes while running
    size_t prep_extra = 0;          // device bytes held only while it is prepared
    tcym_lattice lat = nullptr;
    std::vector<double> series;     // (steps, N_CS) pairs
    Clock::time_point submitted, finished;
    int error = TCYM_OK;
};

size_t reduction_bytes(size_t V, int sm_count) {
    return sizeof(double) * (12 * (size_t)sm_count * 8 + 16) + 8 * 32 * ((V + 255) / 256);
}
// links (ping-pong) + fields + reductions of a lattice in `fmt`
size_t lattice_bytes(int fmt, size_t V, int sm_count) {
    const size_t nst = tcym_stored_sites(fmt, (int64_t)V);
    return 2 * 3 * tcym_link_bytes(fmt) * nst + 3 * tcym_field_bytes(fmt) * nst + reduction_bytes(V, sm_count);
}

void footprint_of(const tcym_request &r, int sm_count, size_t &running, size_t &extra) {
    const int fmt = tcym_format_of(r.nc, r.precision);
    const size_t V = (size_t)r.L * r.L * r.L;
    const size_t na = r.nc == 2 ? 3 : 8;
    running = lattice_bytes(fmt, V, sm_count);
    extra = sizeof(double) * (na * V + 4);  // the restore's violation array, released once prepared
}

}  // namespace

struct tcym_server_s {
    tcym_ctx ctx = nullptr;
    size_t budget = 0, used = 0;
    int max_active = 0, stride = 20;
    std::mutex mu;
    std::condition_variable cv;       // work for the tick thread / stop
    std::condition_variable prep_cv;  // work for the preparers / stop
    std::condition_variable done_cv;  // completions
    std::deque<uint64_t> queue;       // submitted, not yet taken by a preparer
    std::deque<uint64_t> ready;       // prepared, not yet in the ensemble
    std::map<uint64_t, Req> reqs;
    std::vector<uint64_t> active;     // in ensemble order
    int preparing = 0;
    uint64_t next_id = 1;
    tcym_ensemble ens = nullptr;
    cudaMemPool_t pool = nullptr;
    std::thread ticker;
    std::thread preparers[kPreparers];
    bool stop = false;
    double link_updates = 0.0;
    uint64_t completed = 0, failed = 0, ticks = 0;
    double prep_seconds = 0.0;
    std::vector<tcym_tick> tick_log;  // the last ticks (at most kTickRecord)
    Clock::time_point last_tick_end{};
    int loop_error = TCYM_OK;
};

namespace {

// Initial state of a request: U = 1, E ~ N(0, T) per component (Philox field
// stream of the request's seed), Gauss-restored in the request's own storage,
// at most 400 iterations, to 1e-12 in FP64 and to 1e-6 in FP32 (the rounding of
// FP32 fields); the restore scratch is released.  FP32 requests are not restored
// through FP64: at config 4's mix the FP64 restore (DFMA-bound, ~4.4 s of GPU
// time for a 128^3 SU(3) lattice) took more of the device than the stepping.
int prepare(tcym_server srv, Req &r) {
    const tcym_request &q = r.spec;
    int rc = tcym_lattice_create_pooled(srv->ctx, q.nc, q.L, q.L, q.L, q.precision, srv->pool, &r.lat);
    if (!rc) rc = tcym_set_zero(r.lat);
    if (!rc) rc = tcym_gaussian_efield(r.lat, std::sqrt(q.T), q.seed);
    if (!rc) rc = tcym_gauss_restore(r.lat, q.precision == TCYM_FP64 ? 1e-12 : 1e-6, 400, nullptr, nullptr);
    if (!rc) tcym_lattice_release_scratch(r.lat);
    return rc;
}

// joined: the request is an ensemble member (only the tick thread touches the ensemble)
void retire(tcym_server srv, Req &r, int status, bool joined) {
    if (r.lat) {
        if (joined) tcym_ensemble_remove(srv->ens, r.lat);
        tcym_lattice_destroy(r.lat);  // pooled: releases without a device synchronisation
        r.lat = nullptr;
    }
    srv->used -= r.footprint;
    r.status = status;
    r.finished = Clock::now();
    if (status == TCYM_REQ_DONE) ++srv->completed; else ++srv->failed;
}

void prepare_loop(tcym_server srv) {
    cudaSetDevice(srv->ctx->device);
    std::unique_lock<std::mutex> lk(srv->mu);
    while (!srv->stop) {
        const int slots = (int)srv->active.size() + (int)srv->ready.size() + srv->preparing;
        if (srv->queue.empty() || slots >= srv->max_active) {
            srv->prep_cv.wait_for(lk, std::chrono::milliseconds(50));
            continue;
        }
        const uint64_t id = srv->queue.front();
        Req &r = srv->reqs[id];
        if (srv->used + r.footprint + r.prep_extra > srv->budget) {  // in arrival order: wait for memory
            srv->prep_cv.wait_for(lk, std::chrono::milliseconds(50));
            continue;
        }
        srv->queue.pop_front();
        srv->used += r.footprint + r.prep_extra;
        ++srv->preparing;
        lk.unlock();
        const auto t0 = Clock::now();
        const int rc = prepare(srv, r);
        const double secs = std::chrono::duration<double>(Clock::now() - t0).count();
        lk.lock();
        srv->prep_seconds += secs;
        srv->used -= r.prep_extra;
        --srv->preparing;
        if (rc) {
            r.error = rc;
            retire(srv, r, TCYM_REQ_FAILED, false);
            srv->done_cv.notify_all();
        } else {
            srv->ready.push_back(id);
            srv->cv.notify_all();
        }
        srv->prep_cv.notify_all();
    }
}

void tick_loop(tcym_server srv) {
    cudaSetDevice(srv->ctx->device);
    std::unique_lock<std::mutex> lk(srv->mu);
    while (!srv->stop) {
        // prepared requests join at the tick boundary
        while (!srv->ready.empty()) {
            const uint64_t id = srv->ready.front();
            srv->ready.pop_front();
            Req &r = srv->reqs[id];
            const tcym_request &q = r.spec;
            const int rc = tcym_ensemble_add(srv->ens, r.lat, q.dynamics, q.dt, q.gamma, q.T, q.seed, 0);
            if (rc) {
                r.error = rc;
                retire(srv, r, TCYM_REQ_FAILED, false);
                srv->done_cv.notify_all();
                continue;
            }
            r.status = TCYM_REQ_RUNNING;
            srv->active.push_back(id);
        }
        if (srv->active.empty()) {
            srv->cv.wait_for(lk, std::chrono::milliseconds(20));
            continue;
        }
        // one tick: every active request advances `stride` steps and is sampled
        const int n = (int)srv->active.size();
        tcym_tick rec{};
        rec.active = n;
        rec.preparing = srv->preparing;
        for (uint64_t id : srv->active) {
            const tcym_request &q = srv->reqs[id].spec;
            rec.link_updates += 3.0 * (double)q.L * q.L * q.L * srv->stride;
        }
        std::vector<double> ncs(n), edb(n);
        lk.unlock();
        const auto t0 = Clock::now();
        int rc = tcym_ensemble_step(srv->ens, srv->stride);
        if (!rc) rc = tcym_ensemble_measure(srv->ens, srv->stride, edb.data(), ncs.data());
        const auto t1 = Clock::now();
        rec.ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        lk.lock();
        rec.gap_ms = srv->ticks ? std::chrono::duration<double, std::milli>(t0 - srv->last_tick_end).count() : 0.0;
        srv->last_tick_end = t1;
        ++srv->ticks;
        if (srv->tick_log.size() >= kTickRecord)
            srv->tick_log.erase(srv->tick_log.begin(), srv->tick_log.begin() + kTickRecord / 2);
        srv->tick_log.push_back(rec);
        if (rc) {  // a device failure ends the loop; every pending request fails
            srv->loop_error = rc;
            for (uint64_t id : srv->active) retire(srv, srv->reqs[id], TCYM_REQ_FAILED, true);
            srv->active.clear();
            srv->stop = true;
            srv->prep_cv.notify_all();
            srv->done_cv.notify_all();
            break;
        }
        std::vector<uint64_t> still;
        for (int i = 0; i < n; ++i) {
            Req &r = srv->reqs[srv->active[i]];
            r.steps_done += srv->stride;
            srv->link_updates += 3.0 * (double)r.spec.L * r.spec.L * r.spec.L * srv->stride;
            r.series.push_back((double)r.steps_done);
            r.series.push_back(ncs[i]);
            if (!std::isfinite(edb[i]) || !std::isfinite(ncs[i])) {  // health check: non-finite state
                r.error = TCYM_ERR_NONFINITE;
                retire(srv, r, TCYM_REQ_FAILED, true);
            } else if (r.steps_done >= r.target) {
                retire(srv, r, TCYM_REQ_DONE, true);
            } else {
                still.push_back(srv->active[i]);
            }
        }
        if (still.size() != srv->active.size()) {
            srv->done_cv.notify_all();
            srv->prep_cv.notify_all();  // memory and slots were freed
        }
        srv->active.swap(still);
    }
}

}  // namespace

extern "C" int tcym_server_create(tcym_ctx ctx, size_t hbm_budget_bytes, int max_active, int stride,
                                  tcym_server *out) {
    if (!ctx || !out || max_active < 1 || stride < 1 || hbm_budget_bytes == 0) return TCYM_ERR_ARG;
    *out = nullptr;
    tcym_server srv = new (std::nothrow) tcym_server_s();
    if (!srv) return TCYM_ERR_OOM;
    srv->ctx = ctx;
    srv->budget = hbm_budget_bytes;
    srv->max_active = max_active;
    srv->stride = stride;
    cudaSetDevice(ctx->device);
    // the request lattices' pool keeps up to the budget in reserve once used, so
    // later requests reuse memory without going back to the driver
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = ctx->device;
    cudaError_t e = cudaMemPoolCreate(&srv->pool, &props);
    if (e == cudaSuccess) {
        uint64_t keep = hbm_budget_bytes;
        e = cudaMemPoolSetAttribute(srv->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e != cudaSuccess) {
        tcym_set_error(ctx, "tcym_server_create: memory pool: %s", cudaGetErrorString(e));
        if (srv->pool) cudaMemPoolDestroy(srv->pool);
        delete srv;
        return TCYM_ERR_CUDA;
    }
    int rc = tcym_ensemble_create(ctx, &srv->ens);
    if (rc) {
        cudaMemPoolDestroy(srv->pool);
        delete srv;
        return rc;
    }
    srv->ticker = std::thread(tick_loop, srv);
    for (auto &t : srv->preparers) t = std::thread(prepare_loop, srv);
    *out = srv;
    return TCYM_OK;
}

extern "C" int tcym_server_destroy(tcym_server srv) {
    if (!srv) return TCYM_ERR_ARG;
    {
        std::lock_guard<std::mutex> g(srv->mu);
        srv->stop = true;
    }
    srv->cv.notify_all();
    srv->prep_cv.notify_all();
    if (srv->ticker.joinable()) srv->ticker.join();
    for (auto &t : srv->preparers)
        if (t.joinable()) t.join();
    tcym_ensemble_destroy(srv->ens);
    for (auto &kv : srv->reqs)
        if (kv.second.lat) tcym_lattice_destroy(kv.second.lat);
    cudaSetDevice(srv->ctx->device);
    cudaDeviceSynchronize();  // the pooled releases, before the pool goes
    cudaMemPoolDestroy(srv->pool);
    delete srv;
    return TCYM_OK;
}

extern "C" int tcym_server_submit(tcym_server srv, const tcym_request *req, uint64_t *id) {
    if (!srv || !req || !id) return TCYM_ERR_ARG;
    const tcym_request &q = *req;
    if ((q.nc != 2 && q.nc != 3) || q.L < 2 || q.nsteps < 0 || q.dt < 0 || q.T < 0 || q.gamma < 0 ||
        (q.precision != TCYM_FP32 && q.precision != TCYM_FP64) ||
        (q.dynamics != TCYM_DYN_LEAPFROG && q.dynamics != TCYM_DYN_LANGEVIN))
        return TCYM_ERR_ARG;
    Req r;
    r.spec = q;
    footprint_of(q, srv->ctx->sm_count, r.footprint, r.prep_extra);
    if (r.footprint + r.prep_extra > srv->budget) {
        tcym_set_error(srv->ctx,
                       "tcym_server_submit: the request needs %zu bytes (%zu while it is prepared), more than the "
                       "budget %zu",
                       r.footprint, r.footprint + r.prep_extra, srv->budget);
        return TCYM_ERR_ADMISSION;
    }
    r.target = ((q.nsteps + srv->stride - 1) / srv->stride) * srv->stride;
    r.submitted = Clock::now();
    {
        std::lock_guard<std::mutex> g(srv->mu);
        if (srv->loop_error) return srv->loop_error;
        *id = srv->next_id++;
        srv->reqs.emplace(*id, std::move(r));
        srv->queue.push_back(*id);
    }
    srv->prep_cv.notify_all();
    return TCYM_OK;
}

extern "C" int tcym_server_status(tcym_server srv, uint64_t id, int *status, int *steps_done) {
    if (!srv) return TCYM_ERR_ARG;
    std::lock_guard<std::mutex> g(srv->mu);
    auto it = srv->reqs.find(id);
    if (it == srv->reqs.end()) return TCYM_ERR_ARG;
    if (status) *status = it->second.status;
    if (steps_done) *steps_done = it->second.steps_done;
    return TCYM_OK;
}

extern "C" int tcym_server_wait(tcym_server srv, uint64_t id, double timeout_s) {
    if (!srv || timeout_s < 0) return TCYM_ERR_ARG;
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(id);
    if (it == srv->reqs.end()) return TCYM_ERR_ARG;
    const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s));
    while (it->second.status != TCYM_REQ_DONE && it->second.status != TCYM_REQ_FAILED) {
        if (srv->done_cv.wait_until(lk, until) == std::cv_status::timeout &&
            it->second.status != TCYM_REQ_DONE && it->second.status != TCYM_REQ_FAILED)
            return TCYM_ERR_TIMEOUT;
    }
    return it->second.status == TCYM_REQ_DONE ? TCYM_OK : (it->second.error ? it->second.error : TCYM_ERR_STATE);
}

extern "C" int tcym_server_result(tcym_server srv, uint64_t id, double *series, int capacity, int *n_samples,
                                  double *latency_s) {
    if (!srv) return TCYM_ERR_ARG;
    std::lock_guard<std::mutex> g(srv->mu);
    auto it = srv->reqs.find(id);
    if (it == srv->reqs.end()) return TCYM_ERR_ARG;
    const Req &r = it->second;
    if (r.status != TCYM_REQ_DONE && r.status != TCYM_REQ_FAILED) return TCYM_ERR_STATE;
    const int ns = (int)(r.series.size() / 2);
    if (n_samples) *n_samples = ns;
    if (series)
        for (int i = 0; i < 2 * std::min(ns, capacity); ++i) series[i] = r.series[i];
    if (latency_s) *latency_s = std::chrono::duration<double>(r.finished - r.submitted).count();
    return r.status == TCYM_REQ_DONE ? TCYM_OK : (r.error ? r.error : TCYM_ERR_STATE);
}

extern "C" int tcym_server_stats(tcym_server srv, tcym_server_info *out) {
    if (!srv || !out) return TCYM_ERR_ARG;
    std::lock_guard<std::mutex> g(srv->mu);
    out->queued = (int)srv->queue.size();
    out->active = (int)srv->active.size();
    out->completed = srv->completed;
    out->failed = srv->failed;
    out->bytes_in_use = srv->used;
    out->link_updates = srv->link_updates;
    out->preparing = srv->preparing + (int)srv->ready.size();
    out->ticks = srv->ticks;
    out->prep_seconds = srv->prep_seconds;
    return TCYM_OK;
}

extern "C" int tcym_server_ticks(tcym_server srv, double *ms, double *preparing, int capacity, int *n) {
    if (!srv || capacity < 0) return TCYM_ERR_ARG;
    std::lock_guard<std::mutex> g(srv->mu);
    const int total = (int)srv->tick_log.size();
    const int k = std::min(total, capacity);
    for (int i = 0; i < k; ++i) {
        if (ms) ms[i] = srv->tick_log[total - k + i].ms;
        if (preparing) preparing[i] = (double)srv->tick_log[total - k + i].preparing;
    }
    if (n) *n = k;
    return TCYM_OK;
}

extern "C" int tcym_server_tick_log(tcym_server srv, tcym_tick *ticks, int capacity, int *n) {
    if (!srv || capacity < 0 || (capacity > 0 && !ticks)) return TCYM_ERR_ARG;
    std::lock_guard<std::mutex> g(srv->mu);
    const int total = (int)srv->tick_log.size();
    const int k = std::min(total, capacity);
    for (int i = 0; i < k; ++i) ticks[i] = srv->tick_log[total - k + i];
    if (n) *n = k;
    return TCYM_OK;
}
