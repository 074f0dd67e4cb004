// Serving loop: continuous batching of independent trajectory requests.
//
// The reference runs one trajectory per process and seed (SU2Solver.cpp:148-169,
// SphaleronSimulation.cpp:571-616).  Here a background thread owns an
// ensemble; requests are admitted in arrival order while the device-memory
// budget and the slot limit allow, stepped together, sampled every `stride`
// steps (N_CS time series) and retired as soon as they finish, which frees
// their memory for the next arrivals.  Every wait has a time limit.
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

struct Req {
    tcym_request spec;
    int status = TCYM_REQ_QUEUED;
    int steps_done = 0;
    int target = 0;                 // steps rounded up to a multiple of the stride
    size_t footprint = 0;
    tcym_lattice lat = nullptr;
    std::vector<double> series;     // (steps, N_CS) pairs
    Clock::time_point submitted, finished;
    int error = TCYM_OK;
};

size_t footprint_of(const tcym_request &r, int sm_count) {
    const int fmt = tcym_format_of(r.nc, r.precision);
    const size_t V = (size_t)r.L * r.L * r.L;
    const size_t na = r.nc == 2 ? 3 : 8;
    const size_t nst = tcym_stored_sites(fmt, (int64_t)V);
    return 2 * 3 * tcym_link_bytes(fmt) * nst + 3 * tcym_field_bytes(fmt) * nst + sizeof(double) * na * V  // restore scratch
           + sizeof(double) * (12 * (size_t)sm_count * 8 + 16) + 8 * 32 * ((V + 255) / 256);                  // reductions
}

}  // namespace

struct tcym_server_s {
    tcym_ctx ctx = nullptr;
    size_t budget = 0, used = 0;
    int max_active = 0, stride = 20;
    std::mutex mu;
    std::condition_variable cv;       // submissions / stop
    std::condition_variable done_cv;  // completions
    std::deque<uint64_t> queue;
    std::map<uint64_t, Req> reqs;
    std::vector<uint64_t> active;     // in ensemble order
    uint64_t next_id = 1;
    tcym_ensemble ens = nullptr;
    std::thread worker;
    bool stop = false;
    double link_updates = 0.0;
    uint64_t completed = 0, failed = 0;
    int loop_error = TCYM_OK;
};

namespace {

// Initial state of a request: U = 1, E ~ N(0, T) per component (Philox field
// stream of the request's seed), Gauss-restored; the restore scratch is freed.
int prepare(tcym_server srv, Req &r) {
    const tcym_request &q = r.spec;
    int rc = tcym_lattice_create(srv->ctx, q.nc, q.L, q.L, q.L, q.precision, &r.lat);
    if (rc) return rc;
    if ((rc = tcym_set_zero(r.lat))) return rc;
    if ((rc = tcym_gaussian_efield(r.lat, std::sqrt(q.T), q.seed))) return rc;
    const double tol = q.precision == TCYM_FP64 ? 1e-12 : 1e-6;
    if ((rc = tcym_gauss_restore(r.lat, tol, 400, nullptr, nullptr))) return rc;
    tcym_lattice_release_scratch(r.lat);
    return tcym_ensemble_add(srv->ens, r.lat, q.dynamics, q.dt, q.gamma, q.T, q.seed, 0);
}

void retire(tcym_server srv, Req &r, int status) {
    if (r.lat) {
        tcym_ensemble_remove(srv->ens, r.lat);
        tcym_lattice_destroy(r.lat);
        r.lat = nullptr;
    }
    srv->used -= r.footprint;
    r.status = status;
    r.finished = Clock::now();
    if (status == TCYM_REQ_DONE) ++srv->completed; else ++srv->failed;
}

void loop(tcym_server srv) {
    cudaSetDevice(srv->ctx->device);
    std::unique_lock<std::mutex> lk(srv->mu);
    while (!srv->stop) {
        // admission, in arrival order, while memory and slots allow
        while (!srv->queue.empty() && (int)srv->active.size() < srv->max_active) {
            Req &r = srv->reqs[srv->queue.front()];
            if (srv->used + r.footprint > srv->budget) break;
            const uint64_t id = srv->queue.front();
            srv->queue.pop_front();
            srv->used += r.footprint;
            lk.unlock();
            int rc = prepare(srv, r);
            lk.lock();
            if (rc) {
                r.error = rc;
                retire(srv, r, TCYM_REQ_FAILED);
                srv->done_cv.notify_all();
                continue;
            }
            r.status = TCYM_REQ_RUNNING;
            srv->active.push_back(id);
        }
        if (srv->active.empty()) {
            srv->cv.wait_for(lk, std::chrono::milliseconds(50));
            continue;
        }
        // one tick: every active request advances `stride` steps and is sampled
        const int n = (int)srv->active.size();
        std::vector<double> ncs(n), edb(n);
        lk.unlock();
        int rc = tcym_ensemble_step(srv->ens, srv->stride);
        if (!rc) rc = tcym_ensemble_measure(srv->ens, srv->stride, edb.data(), ncs.data());
        lk.lock();
        if (rc) {  // a device failure ends the loop; every pending request fails
            srv->loop_error = rc;
            for (uint64_t id : srv->active) retire(srv, srv->reqs[id], TCYM_REQ_FAILED);
            srv->active.clear();
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
                retire(srv, r, TCYM_REQ_FAILED);
            } else if (r.steps_done >= r.target) {
                retire(srv, r, TCYM_REQ_DONE);
            } else {
                still.push_back(srv->active[i]);
            }
        }
        if (still.size() != srv->active.size()) srv->done_cv.notify_all();
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
    int rc = tcym_ensemble_create(ctx, &srv->ens);
    if (rc) {
        delete srv;
        return rc;
    }
    srv->worker = std::thread(loop, srv);
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
    if (srv->worker.joinable()) srv->worker.join();
    for (auto &kv : srv->reqs)
        if (kv.second.lat) tcym_lattice_destroy(kv.second.lat);
    tcym_ensemble_destroy(srv->ens);
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
    r.footprint = footprint_of(q, srv->ctx->sm_count);
    if (r.footprint > srv->budget) {
        tcym_set_error(srv->ctx, "tcym_server_submit: the request needs %zu bytes, more than the budget %zu",
                       r.footprint, srv->budget);
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
    srv->cv.notify_all();
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
    return TCYM_OK;
}
