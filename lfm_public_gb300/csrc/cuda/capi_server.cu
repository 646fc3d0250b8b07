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
// device. Large requests (solo_cells) run instead on their own single-case
// FP32-bulk solver, built from a host copy of their description by a second
// thread (the preparer) while the worker's chunks run, admitted once built,
// and stepped chunk by chunk on its own stream beside the batch (the batch
// kernel is a generic one; the single-case kernels are faster on large cases
// and give the same bits).
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

// A host copy of a solver description (the caller's may be freed once
// lfm_server_submit returns): every array it points to, owned.
struct OwnedDesc {
    lfm_solver_desc d{};
    std::vector<int64_t> i64[8];
    std::vector<double> f64[18];
    std::vector<uint8_t> u8;
    std::vector<int8_t> s8;
    std::vector<int> ik;
    std::vector<int32_t> i32;

    template <typename T>
    static const T* keep(std::vector<T>& v, const T* src, size_t n) {
        if (!src) return nullptr;
        v.assign(src, src + n);
        return v.data();
    }

    explicit OwnedDesc(const lfm_solver_desc* s) : d(*s) {
        const size_t nf = (size_t)s->n_faces, nc = (size_t)s->n_cells, ng = (size_t)s->n_ghosts;
        const size_t D = (size_t)s->dim, nh = (size_t)s->n_halos;
        const size_t ne = s->cell_face_offsets ? (size_t)s->cell_face_offsets[nc] : 0;
        const size_t ns = s->cell_s_offsets ? (size_t)s->cell_s_offsets[nc] : 0;
        d.face_p = keep(i64[0], s->face_p, nf);
        d.face_n = keep(i64[1], s->face_n, nf);
        d.face_ghost = keep(u8, s->face_ghost, nf);
        d.S = keep(f64[0], s->S, D * nf);
        d.d = keep(f64[1], s->d, D * nf);
        d.w = keep(f64[2], s->w, nf);
        d.smag = keep(f64[3], s->smag, nf);
        d.dmag_inv = keep(f64[4], s->dmag_inv, nf);
        d.dnorm = keep(f64[5], s->dnorm, D * nf);
        d.delta_mag = keep(f64[6], s->delta_mag, nf);
        d.K = keep(f64[7], s->K, D * nf);
        d.vol_inv = keep(f64[8], s->vol_inv, nc);
        d.sponge = keep(f64[9], s->sponge, nc);
        d.ghost_cell = keep(i64[2], s->ghost_cell, ng);
        d.ghost_kind = keep(ik, s->ghost_kind, ng);
        d.cell_face_offsets = keep(i64[3], s->cell_face_offsets, nc + 1);
        d.cell_faces = keep(i64[4], s->cell_faces, ne);
        d.cell_face_sign = keep(s8, s->cell_face_sign, ne);
        d.cell_s_offsets = keep(i64[5], s->cell_s_offsets, nc + 1);
        d.cell_s = keep(f64[10], s->cell_s, D * ns);
        d.q0 = keep(f64[11], s->q0, (size_t)s->nq * nc);
        d.rkA = keep(f64[12], s->rkA, (size_t)std::max(s->rk_order, 0));
        d.rkB = keep(f64[13], s->rkB, (size_t)std::max(s->rk_order, 0));
        d.halo_src_part = keep(i64[6], s->halo_src_part, nh);
        d.halo_src_cell = keep(i64[7], s->halo_src_cell, nh);
        d.ghost_patch = keep(i32, s->ghost_patch, ng);
        d.smag_c = keep(f64[14], s->smag_c, nc);
    }
};

struct Request {
    int64_t id = 0;
    std::unique_ptr<lfm::batch::PreparedCase> pc;
    // solo requests: their description until admission, then their solver;
    // prep (guarded by the server's mutex): 0 waiting for the preparer, 1
    // being built, 2 built, 3 refused (status says why); nomemAt: the
    // server's solo retirement count when a build ran out of memory (retried
    // once another solo request has retired)
    std::unique_ptr<OwnedDesc> desc;
    lfm_solver* solver = nullptr;
    double dt = 0;
    int prep = 0;
    int64_t nomemAt = -1;
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

    ~Request() {
        if (solver) lfm_solver_destroy(solver);
    }
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
    int64_t soloCells = 0;   // requests of at least this many cells run on their own solver (0: none)
    int maxSolo = 2;
    // guarded by mu: solo requests running, built or being built but not yet
    // admitted, and retired so far
    int soloActive = 0, soloPrepared = 0;
    int64_t soloRetired = 0;
    std::condition_variable cvPrep;
    std::thread preparer;
    std::chrono::steady_clock::time_point t0;
    std::mutex mu;
    std::condition_variable cvWork, cvDone;
    std::deque<Request*> pending;
    std::vector<Request*> active;
    std::unordered_map<int64_t, std::unique_ptr<Request>> all;
    int64_t nextId = 1;
    int64_t completed = 0;
    int64_t chunks = 0;
    double busy = 0;          // seconds spent advancing chunks
    double cellStages = 0;    // cell-RK-stage updates advanced
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

// Admission pass: arrival order; a batched request that does not fit is
// passed over, except that once the oldest waiting one has been passed over
// maxBypass times no batched request behind it is admitted until it fits.
// Solo requests take no arena: each is admitted once its solver is built.
int admit(lfm_server* s) {
    std::vector<Request*> queue;
    std::vector<int> prep;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        queue.assign(s->pending.begin(), s->pending.end());
        for (Request* r : queue) prep.push_back(r->prep);
    }
    std::vector<Request*> admitted, rejected;
    size_t largest = 0, total = 0, arena = 0;
    lfm_batch_memory(s->batch, &largest, &total, &arena);
    int soloAdmitted = 0;
    bool arenaClosed = false;   // a batched request waits: no batched request behind it goes first
    for (size_t k = 0; k < queue.size(); ++k) {
        Request* r = queue[k];
        if (r->desc) {   // its own solver, built by the preparer thread (no arena)
            if (prep[k] == 2) {
                ++soloAdmitted;
                admitted.push_back(r);
            } else if (prep[k] == 3) {   // a description the solver refuses
                rejected.push_back(r);
            }
            continue;
        }
        if (arenaClosed) continue;
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
        if (++r->bypassed > s->maxBypass) arenaClosed = true;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    const double now = since(s->t0);
    for (Request* r : admitted) {
        r->state = 1;
        r->tAdmit = now;
        r->pc.reset();   // the image (or the solver's copy) is on the device now
        r->desc.reset();
        s->active.push_back(r);
    }
    s->soloActive += soloAdmitted;
    s->soloPrepared -= soloAdmitted;
    for (Request* r : rejected) {
        r->state = 2;
        if (r->status == LFM_OK) r->status = LFM_ERR_NOMEM;
        r->tDone = now;
        r->pc.reset();
        r->desc.reset();
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
            // something to run or to admit: a batched request, or a solo
            // request whose solver the preparer has built (or refused)
            s->cvWork.wait(lk, [&] {
                if (s->stop || !s->active.empty()) return true;
                for (const Request* r : s->pending)
                    if (!r->desc || r->prep >= 2) return true;
                return false;
            });
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
            Request* oldest = nullptr;   // the oldest batched request
            for (Request* r : s->pending)
                if (!r->desc) {
                    oldest = r;
                    break;
                }
            if (act.empty() && oldest && oldest->tried) {
                // nothing runs and the oldest batched request still cannot be placed
                s->pending.erase(std::find(s->pending.begin(), s->pending.end(), oldest));
                oldest->state = 2;
                oldest->status = LFM_ERR_NOMEM;
                oldest->tDone = since(s->t0);
                oldest->pc.reset();
                s->cvDone.notify_all();
            }
        }
        if (act.empty()) continue;
        int n = s->chunkSteps;
        bool batched = false;
        for (Request* r : act) {
            n = std::min(n, r->remaining);
            batched = batched || !r->solver;
        }
        const double tChunk = since(s->t0);
        // the solo requests' steps on their own streams, then the batch's;
        // all run on the device together, one synchronisation each
        for (Request* r : act)
            if (r->solver && (rc = lfm_solver_step(r->solver, n, r->dt)) != LFM_OK) {
                fail(s, rc);
                return;
            }
        if (batched && (rc = lfm_batch_step(s->batch, n)) != LFM_OK) {
            fail(s, rc);
            return;
        }
        rc = batched ? lfm_batch_sync(s->batch) : LFM_OK;
        if (rc != LFM_OK && rc != LFM_ERR_NUMERIC) {
            fail(s, rc);
            return;
        }
        // each request's status after the chunk (applied under the lock
        // below: lfm_server_info reads it from other threads)
        std::vector<int> stat(act.size(), LFM_OK);
        for (size_t k = 0; k < act.size(); ++k) {
            Request* r = act[k];
            if (r->solver) {
                const int st = lfm_solver_sync(r->solver);
                if (st == LFM_ERR_NUMERIC) {
                    stat[k] = st;
                } else if (st != LFM_OK) {
                    fail(s, st);
                    return;
                }
            } else if (rc == LFM_ERR_NUMERIC) {
                int st = LFM_OK;
                if (lfm_batch_case_status(s->batch, r->slot, &st) != LFM_OK) st = LFM_ERR_CUDA;
                stat[k] = st;
            }
        }
        std::vector<Request*> done;
        {
            double cells = 0;
            for (Request* r : act) cells += (double)r->nc;
            std::lock_guard<std::mutex> lk(s->mu);
            ++s->chunks;
            s->busy += since(s->t0) - tChunk;
            s->cellStages += cells * (double)n * (double)s->rkOrder;
            for (size_t k = 0; k < act.size(); ++k) {
                Request* r = act[k];
                r->remaining -= n;
                if (stat[k] != LFM_OK) r->status = stat[k];
                if (r->remaining == 0 || r->status != LFM_OK) done.push_back(r);
            }
        }
        for (Request* r : done) {
            r->result.resize((size_t)r->nq * r->nc);
            int e1, e2 = LFM_OK;
            if (r->solver) {
                e1 = lfm_solver_get_state(r->solver, r->result.data());
                lfm_solver_destroy(r->solver);
                r->solver = nullptr;
                {
                    std::lock_guard<std::mutex> lk(s->mu);
                    --s->soloActive;
                    ++s->soloRetired;
                }
                s->cvPrep.notify_all();
            } else {
                e1 = lfm_batch_get_state(s->batch, r->slot, r->result.data());
                e2 = lfm_batch_remove(s->batch, r->slot);
            }
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

// The preparer thread builds the solvers of solo requests ahead of their
// admission (host set-up and uploads, overlapping the chunks the worker runs),
// in arrival order, while fewer than maxSolo are running or built. A build
// that runs out of device memory is retried once another solo request has
// retired; one the solver refuses marks the request for rejection.
Request* nextToPrepare(lfm_server* s) {
    if (s->soloActive + s->soloPrepared >= s->maxSolo) return nullptr;
    for (Request* r : s->pending)
        if (r->desc && r->prep == 0 && r->nomemAt < s->soloRetired) return r;
    return nullptr;
}

void preparerLoop(lfm_server* s) {
    if (cudaSetDevice(s->device) != cudaSuccess) {
        lfm::setError(LFM_ERR_CUDA, "server preparer: cudaSetDevice failed");
        fail(s, LFM_ERR_CUDA);
        return;
    }
    for (;;) {
        Request* r = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cvPrep.wait(lk, [&] { return s->stop || (r = nextToPrepare(s)) != nullptr; });
            if (s->stop) return;
            r->prep = 1;
            ++s->soloPrepared;
        }
        // r stays in the pending queue and owned by the server while its
        // prep is 1: nothing else touches its description
        lfm_solver_opts o{LFM_FP32_BULK, s->device, 0};
        lfm_solver* sv = nullptr;
        const int rc = lfm_solver_create(&r->desc->d, &o, &sv);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (rc == LFM_OK) {
                r->solver = sv;
                r->prep = 2;
            } else {
                --s->soloPrepared;
                if (rc == LFM_ERR_NOMEM && s->soloActive + s->soloPrepared > 0) {
                    // other solvers hold memory that their retirement frees
                    r->prep = 0;
                    r->nomemAt = s->soloRetired;
                } else {   // refused, or out of memory with no other solver to wait for
                    r->prep = 3;
                    r->status = rc;
                }
            }
        }
        s->cvWork.notify_all();
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
    info->steps_done = r.nsteps - r.remaining;
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
    s->soloCells = std::max<int64_t>(0, opts->solo_cells);
    s->maxSolo = opts->max_solo > 0 ? opts->max_solo : 2;
    s->t0 = std::chrono::steady_clock::now();
    s->worker = std::thread(workerLoop, s);
    if (s->soloCells > 0) s->preparer = std::thread(preparerLoop, s);
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
    s->cvPrep.notify_all();
    if (s->worker.joinable()) s->worker.join();
    if (s->preparer.joinable()) s->preparer.join();
    lfm_batch_destroy(s->batch);
    delete s;
}

extern "C" int lfm_server_submit(lfm_server* s, const lfm_solver_desc* d, double dt, int nsteps, int64_t* id) {
    if (!s || !id) return lfm::setError(LFM_ERR_INVALID, "null argument");
    *id = 0;
    if (nsteps <= 0) return lfm::setError(LFM_ERR_INVALID, "nsteps must be positive");
    const double tSubmit = since(s->t0);
    std::unique_ptr<Request> r(new Request);
    if (s->soloCells > 0 && d && d->n_cells >= s->soloCells && d->n_halos == 0) {
        if (d->rk_order != s->rkOrder)
            return lfm::setError(LFM_ERR_INVALID, "the request's rk_order differs from the server's");
        if (!d->q0) return lfm::setError(LFM_ERR_INVALID, "the request has no initial state (desc->q0)");
        if (!(dt > 0.0)) return lfm::setError(LFM_ERR_INVALID, "dt must be positive");
        try {
            r->desc.reset(new OwnedDesc(d));
        } catch (const std::bad_alloc&) {
            return lfm::setError(LFM_ERR_NOMEM, "host copy of the request");
        }
        r->nq = d->nq;
        r->nc = (int)d->n_cells;
        r->dt = dt;
    } else {
        lfm::batch::PreparedCase* pc = nullptr;
        int rc = lfm::batch::prepareCase(d, dt, s->rkOrder, &pc);
        if (rc) return rc;
        r->pc.reset(pc);
        r->bytes = pc->layout.total;
        r->nq = pc->nq;
        r->nc = pc->nc;
    }
    r->nsteps = r->remaining = nsteps;
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
    s->cvPrep.notify_all();
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
    st->busy_s = s->busy;
    st->cell_stages = s->cellStages;
    if (s->workerError) return lfm::setError(s->workerError, "server stopped: " + s->workerMsg);
    return LFM_OK;
}
