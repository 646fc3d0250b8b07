// C ABI, request server (include/lfm_gpu.h, lfm_server_*): continuous batching
// of solve requests on one GPU.
//
// Submitting threads validate and pack each request on the host (its arena
// image is built there, so the worker never waits on host preparation). One
// worker thread owns a batch and loops: admit queued requests in arrival
// order while a case slot and an arena block of their footprint are free
// (a request that does not fit is passed over, but only max_bypass times
// before admission waits for it); advance every admitted request together
// by a chunk of steps -- the smallest remaining step count, at most
// chunk_steps -- in the batch's persistent stage kernels; retire the
// requests that have finished (or whose state became non-finite), copying
// their state out and freeing their slot and block. Requests arriving while
// others run join at the next chunk boundary, so their work overlaps on the
// device.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../host/capi_internal.h"
#include "batch_internal.h"
#include "lfm_gpu.h"

namespace {

struct Request {
    int64_t id = 0;
    std::unique_ptr<lfm::batch::PreparedCase> pc;
    size_t bytes = 0;
    int nsteps = 0, remaining = 0;
    int slot = -1;
    int state = 0;   // 0 queued, 1 running, 2 done
    int status = LFM_OK;
    int bypassed = 0;
    bool tried = false;   // an admission pass has considered it
    double tSubmit = 0, tAdmit = -1, tDone = -1;
    int nq = 0, nc = 0;
    std::vector<double> result;
};

double since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct lfm_server {
    lfm_batch* batch = nullptr;
    int device = 0;
    int rkOrder = 5;
    int chunkSteps = 50;
    int maxBypass = 8;
    std::chrono::steady_clock::time_point t0;
    std::mutex mu;
    std::condition_variable cvWork, cvDone;
    std::deque<Request*> pending;
    std::vector<Request*> active;
    std::unordered_map<int64_t, std::unique_ptr<Request>> all;
    int64_t nextId = 1;
    int64_t completed = 0;
    int64_t chunks = 0;
    bool stop = false;
    int workerError = LFM_OK;
    std::string workerMsg;
    std::thread worker;
};

namespace {

void fail(lfm_server* s, int code) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->workerError = code;
    s->workerMsg = lfm_last_error();
    for (Request* r : s->pending) {
        r->state = 2;
        r->status = code;
        r->tDone = since(s->t0);
    }
    for (Request* r : s->active) {
        r->state = 2;
        r->status = code;
        r->tDone = since(s->t0);
    }
    s->pending.clear();
    s->active.clear();
    s->cvDone.notify_all();
}

// Admission pass: arrival order; a request that does not fit is passed over,
// except that once the oldest waiting request has been passed over
// maxBypass times nothing behind it is admitted until it fits.
int admit(lfm_server* s) {
    std::vector<Request*> queue;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        queue.assign(s->pending.begin(), s->pending.end());
    }
    std::vector<Request*> admitted, rejected;
    size_t largest = 0, total = 0, arena = 0;
    lfm_batch_memory(s->batch, &largest, &total, &arena);
    for (size_t k = 0; k < queue.size(); ++k) {
        Request* r = queue[k];
        r->tried = true;
        if (r->bytes > arena) {   // can never fit
            rejected.push_back(r);
            continue;
        }
        int slot = -1;
        const int rc = lfm::batch::commitCase(s->batch, *r->pc, &slot);
        if (rc == LFM_OK) {
            r->slot = slot;
            admitted.push_back(r);
            continue;
        }
        if (rc != LFM_ERR_NOMEM) return rc;
        if (++r->bypassed > s->maxBypass) break;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    const double now = since(s->t0);
    for (Request* r : admitted) {
        r->state = 1;
        r->tAdmit = now;
        r->pc.reset();   // the image is on the device now
        s->active.push_back(r);
    }
    for (Request* r : rejected) {
        r->state = 2;
        r->status = LFM_ERR_NOMEM;
        r->tDone = now;
        r->pc.reset();
    }
    if (!admitted.empty() || !rejected.empty()) {
        std::deque<Request*> rest;
        for (Request* r : s->pending)
            if (r->state == 0) rest.push_back(r);
        s->pending.swap(rest);
    }
    if (!rejected.empty()) s->cvDone.notify_all();
    return LFM_OK;
}

void workerLoop(lfm_server* s) {
    if (cudaSetDevice(s->device) != cudaSuccess) {
        lfm::setError(LFM_ERR_CUDA, "server worker: cudaSetDevice failed");
        fail(s, LFM_ERR_CUDA);
        return;
    }
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cvWork.wait(lk, [&] { return s->stop || !s->pending.empty() || !s->active.empty(); });
            if (s->stop) return;
        }
        int rc = admit(s);
        if (rc) {
            fail(s, rc);
            return;
        }
        std::vector<Request*> act;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            act = s->active;
            if (act.empty() && !s->pending.empty() && s->pending.front()->tried) {
                // nothing runs and the oldest request still cannot be placed
                Request* r = s->pending.front();
                s->pending.pop_front();
                r->state = 2;
                r->status = LFM_ERR_NOMEM;
                r->tDone = since(s->t0);
                r->pc.reset();
                s->cvDone.notify_all();
            }
        }
        if (act.empty()) continue;
        int n = s->chunkSteps;
        for (Request* r : act) n = std::min(n, r->remaining);
        if ((rc = lfm_batch_step(s->batch, n)) != LFM_OK) {
            fail(s, rc);
            return;
        }
        rc = lfm_batch_sync(s->batch);
        if (rc != LFM_OK && rc != LFM_ERR_NUMERIC) {
            fail(s, rc);
            return;
        }
        ++s->chunks;
        std::vector<Request*> done;
        for (Request* r : act) {
            r->remaining -= n;
            int st = LFM_OK;
            if (rc == LFM_ERR_NUMERIC && lfm_batch_case_status(s->batch, r->slot, &st) != LFM_OK) st = LFM_ERR_CUDA;
            if (st != LFM_OK) r->status = st;
            if (r->remaining == 0 || r->status != LFM_OK) done.push_back(r);
        }
        for (Request* r : done) {
            r->result.resize((size_t)r->nq * r->nc);
            int e1 = lfm_batch_get_state(s->batch, r->slot, r->result.data());
            int e2 = lfm_batch_remove(s->batch, r->slot);
            if (e1 || e2) {
                fail(s, e1 ? e1 : e2);
                return;
            }
        }
        if (!done.empty()) {
            std::lock_guard<std::mutex> lk(s->mu);
            const double now = since(s->t0);
            for (Request* r : done) {
                r->state = 2;
                r->tDone = now;
                r->slot = -1;
                ++s->completed;
            }
            s->active.erase(std::remove_if(s->active.begin(), s->active.end(),
                                           [](Request* r) { return r->state == 2; }),
                            s->active.end());
            s->cvDone.notify_all();
        }
    }
}

void fillInfo(const lfm_server* s, const Request& r, lfm_request_info* info) {
    (void)s;
    info->state = r.state;
    info->status = r.status;
    info->cells = r.nc;
    info->steps = r.nsteps;
    info->t_submit = r.tSubmit;
    info->t_admit = r.tAdmit;
    info->t_done = r.tDone;
    info->footprint_bytes = r.bytes;
}

}  // namespace

extern "C" int lfm_server_create(const lfm_server_opts* opts, lfm_server** out) {
    if (!opts || !out) return lfm::setError(LFM_ERR_INVALID, "null argument");
    *out = nullptr;
    lfm_batch_opts bo{opts->device, opts->rk_order, opts->arena_bytes, opts->max_cases};
    lfm_batch* b = nullptr;
    int rc = lfm_batch_create(&bo, &b);
    if (rc) return rc;
    if (opts->tuning.block) {
        rc = lfm_batch_set_tuning(b, &opts->tuning);
        if (rc) {
            lfm_batch_destroy(b);
            return rc;
        }
    }
    lfm_server* s = new lfm_server;
    s->batch = b;
    s->device = opts->device;
    s->rkOrder = opts->rk_order;
    s->chunkSteps = opts->chunk_steps > 0 ? opts->chunk_steps : 50;
    s->maxBypass = opts->max_bypass == 0 ? 8 : std::max(0, opts->max_bypass);
    s->t0 = std::chrono::steady_clock::now();
    s->worker = std::thread(workerLoop, s);
    *out = s;
    return LFM_OK;
}

extern "C" void lfm_server_destroy(lfm_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cvWork.notify_all();
    if (s->worker.joinable()) s->worker.join();
    lfm_batch_destroy(s->batch);
    delete s;
}

extern "C" int lfm_server_submit(lfm_server* s, const lfm_solver_desc* d, double dt, int nsteps, int64_t* id) {
    if (!s || !id) return lfm::setError(LFM_ERR_INVALID, "null argument");
    *id = 0;
    if (nsteps <= 0) return lfm::setError(LFM_ERR_INVALID, "nsteps must be positive");
    const double tSubmit = since(s->t0);
    lfm::batch::PreparedCase* pc = nullptr;
    int rc = lfm::batch::prepareCase(d, dt, s->rkOrder, &pc);
    if (rc) return rc;
    std::unique_ptr<Request> r(new Request);
    r->pc.reset(pc);
    r->bytes = pc->layout.total;
    r->nsteps = r->remaining = nsteps;
    r->nq = pc->nq;
    r->nc = pc->nc;
    r->tSubmit = tSubmit;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->workerError) return lfm::setError(s->workerError, "server stopped: " + s->workerMsg);
        r->id = s->nextId++;
        *id = r->id;
        s->pending.push_back(r.get());
        s->all[r->id] = std::move(r);
    }
    s->cvWork.notify_all();
    return LFM_OK;
}

extern "C" int lfm_server_info(lfm_server* s, int64_t id, lfm_request_info* info) {
    if (!s || !info) return lfm::setError(LFM_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return lfm::setError(LFM_ERR_INVALID, "unknown request " + std::to_string(id));
    fillInfo(s, *it->second, info);
    return LFM_OK;
}

extern "C" int lfm_server_wait(lfm_server* s, int64_t id, double timeout_s, int* done) {
    if (!s) return lfm::setError(LFM_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return lfm::setError(LFM_ERR_INVALID, "unknown request " + std::to_string(id));
    Request* r = it->second.get();
    auto pred = [&] { return r->state == 2; };
    if (timeout_s < 0)
        s->cvDone.wait(lk, pred);
    else
        s->cvDone.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
    if (done) *done = r->state == 2 ? 1 : 0;
    return LFM_OK;
}

extern "C" int lfm_server_result(lfm_server* s, int64_t id, double* q, lfm_request_info* info) {
    if (!s) return lfm::setError(LFM_ERR_INVALID, "null server");
    std::unique_ptr<Request> r;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->all.find(id);
        if (it == s->all.end()) return lfm::setError(LFM_ERR_INVALID, "unknown request " + std::to_string(id));
        if (it->second->state != 2) return lfm::setError(LFM_ERR_INVALID, "request " + std::to_string(id) + " is not done");
        r = std::move(it->second);
        s->all.erase(it);
    }
    if (info) fillInfo(s, *r, info);
    if (q && !r->result.empty()) std::copy(r->result.begin(), r->result.end(), q);
    return LFM_OK;
}

extern "C" int lfm_server_get_stats(lfm_server* s, lfm_server_stats* st) {
    if (!s || !st) return lfm::setError(LFM_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    st->queued = (int)s->pending.size();
    st->running = (int)s->active.size();
    st->completed = s->completed;
    st->chunks = s->chunks;
    st->t_now = since(s->t0);
    if (s->workerError) return lfm::setError(s->workerError, "server stopped: " + s->workerMsg);
    return LFM_OK;
}
