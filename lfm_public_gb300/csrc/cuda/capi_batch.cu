// C ABI, batch engine (include/lfm_gpu.h, lfm_batch_*).
//
// A batch owns one device arena (a single allocation sized at creation) in
// which every admitted case gets one contiguous block holding all its arrays
// (FP32-bulk layout of a single-case solver). Admission is by footprint: a
// case is admitted when a free block of its size exists (first fit, blocks
// coalesce when cases leave). A time step of all cases is one CUDA graph --
// a memset of the barrier counters and one persistent kernel per RK stage --
// whose kernels read the case table and tile lists from device memory, so
// admissions and removals between steps only rewrite those tables.
#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../host/capi_internal.h"
#include "args_setup.h"
#include "batch.cuh"
#include "batch_internal.h"
#include "lfm_gpu.h"
#include "solver_launch.h"

using lfm::dev::Args;
using lfm::dev::BatchArgs;
using lfm::dev::BatchCase;
using lfm::dev::BatchCtl;
using lfm::dev::BatchTile;
using lfm::dev::kBatchMaxStages;
using lfm::dev::kBatchPhases;
using lfm::batch::Arena;
using lfm::batch::CaseLayout;
using lfm::batch::PreparedCase;
using lfm::batch::Slot;
using lfm::batch::roundUp;


namespace {

int cudaFail(cudaError_t e, const char* what) {
    return lfm::setError(e == cudaErrorMemoryAllocation ? LFM_ERR_NOMEM : LFM_ERR_CUDA,
                         std::string(what) + ": " + cudaGetErrorString(e));
}

#define LFM_CUDA(call)                                       \
    do {                                                     \
        cudaError_t e__ = (call);                            \
        if (e__ != cudaSuccess) return cudaFail(e__, #call); \
    } while (0)

// Host image of a case's arena block: constant arrays and the initial state
// (as q - qRef) in their final device layout, scratch zero-filled (the viscous
// terms and gradients of ghosts are read as zeros).
std::vector<unsigned char> packCase(const lfm_solver_desc* d, const CaseLayout& L, const double* qRef) {
    std::vector<unsigned char> img(L.total, 0);
    const size_t D = (size_t)d->dim, nq = (size_t)d->nq, nc = (size_t)d->n_cells, ng = (size_t)d->n_ghosts;
    const size_t nt = nc + ng, nf = (size_t)d->n_faces;
    auto f64 = [&](size_t off) { return reinterpret_cast<double*>(img.data() + off); };
    auto f32 = [&](size_t off) { return reinterpret_cast<float*>(img.data() + off); };
    auto i32 = [&](size_t off) { return reinterpret_cast<int*>(img.data() + off); };
    auto conv = [&](size_t off, const double* src, size_t n) {
        float* p = f32(off);
        for (size_t k = 0; k < n; ++k) p[k] = (float)src[k];
    };
    for (size_t v = 0; v < nq; ++v) {
        double* row = f64(L.q) + v * nt;
        for (size_t c = 0; c < nc; ++c) row[c] = (d->q0 ? d->q0[v * nc + c] : 0.0) - qRef[v];
    }
    conv(L.S, d->S, D * nf);
    conv(L.d, d->d, D * nf);
    conv(L.w, d->w, nf);
    conv(L.dinv, d->dmag_inv, nf);
    conv(L.dnorm, d->dnorm, D * nf);
    conv(L.K, d->K, D * nf);
    lfm::setup::DescIndex ix(d);
    conv(L.lapc, ix.lapc.data(), nf);
    std::memcpy(i32(L.fP), ix.fP.data(), nf * 4);
    std::memcpy(i32(L.fN), ix.fN.data(), nf * 4);
    std::memcpy(img.data() + L.fGhost, d->face_ghost, nf);
    std::memcpy(f64(L.volInv), d->vol_inv, nc * 8);
    conv(L.volInv32, d->vol_inv, nc);
    conv(L.sponge, d->sponge, nc);
    std::memcpy(i32(L.cfOff), ix.cfOff.data(), (nc + 1) * 4);
    std::memcpy(i32(L.cfList), ix.cfList.data(), ix.cfList.size() * 4);
    std::memcpy(i32(L.cfNbr), ix.cfNbr.data(), ix.cfNbr.size() * 4);
    if (L.cfEll != CaseLayout::npos()) {   // entry k of cell c at k * nc + c, padded
        const size_t W = (size_t)(D == 2 ? lfm::dev::kEllWidth<2> : lfm::dev::kEllWidth<3>);
        int* ell = i32(L.cfEll);
        for (size_t k = 0; k < W * nc; ++k) ell[k] = lfm::dev::kEllPad;
        for (size_t c = 0; c < nc; ++c)
            for (int e = ix.cfOff[c]; e < ix.cfOff[c + 1]; ++e)
                ell[(size_t)(e - ix.cfOff[c]) * nc + c] = ix.cfList[(size_t)e];
    }
    unsigned char* cg = img.data() + L.cellGhosts;   // cells whose update writes ghosts
    for (size_t f = 0; f < nf; ++f)
        if (ix.fN[f] >= (int)nc && ix.fN[f] < (int)(nc + ng)) cg[(size_t)ix.fP[f]] = 1;
    if (ng) {
        std::memcpy(i32(L.gCell), ix.gCell.data(), ng * 4);
        std::memcpy(i32(L.gKind), ix.gKind.data(), ng * 4);
        std::memcpy(i32(L.gFace), ix.gFace.data(), ng * 4);
    }
    return img;
}

}  // namespace

namespace {

// The stage-kernel variant that covers every case in the batch.
int currentVariant(const lfm_batch* b) {
    bool d3 = false, full = false;
    for (const Slot& sl : b->slots) {
        if (!sl.used) continue;
        d3 = d3 || sl.D == 3;
        full = full || sl.needGradVis;
    }
    if (d3) return lfm::dev::kBatchVariantGeneral;
    return full ? lfm::dev::kBatchVariant2D : lfm::dev::kBatchVariant2DInviscid;
}

int rebuildTiles(lfm_batch* b) {
    const int tileSize = b->tune.block * b->tune.items_per_thread;
    std::vector<BatchTile> tl[kBatchPhases];
    for (int s = 0; s < (int)b->slots.size(); ++s) {
        const Slot& sl = b->slots[(size_t)s];
        if (!sl.used) continue;
        // the update phase keeps the primitives of the cells and ghosts
        // current: preparation runs only in a case's first step after a new state
        const int first[kBatchPhases] = {0, 0, 0, 0};
        const int end[kBatchPhases] = {sl.primsValid ? 0 : sl.nt, sl.needGradVis ? sl.nc : 0, sl.nf, sl.nc};
        for (int ph = 0; ph < kBatchPhases; ++ph)
            for (int st = first[ph]; st < end[ph]; st += tileSize)
                tl[ph].push_back(BatchTile{s, st, std::min(tileSize, end[ph] - st), 0});
    }
    int n[kBatchPhases];
    bool realloc = false;
    for (int ph = 0; ph < kBatchPhases; ++ph) {
        n[ph] = (int)tl[ph].size();
        if (tl[ph].size() > b->tileCap[ph] || !b->dTiles[ph]) {
            LFM_CUDA(cudaStreamSynchronize(b->stream));
            if (b->dTiles[ph]) cudaFree(b->dTiles[ph]);
            b->dTiles[ph] = nullptr;
            const size_t cap = std::max<size_t>(1024, tl[ph].size() + tl[ph].size() / 2);
            LFM_CUDA(cudaMalloc(&b->dTiles[ph], cap * sizeof(BatchTile)));
            b->tileCap[ph] = cap;
            realloc = true;
        }
        if (n[ph])
            LFM_CUDA(cudaMemcpyAsync(b->dTiles[ph], tl[ph].data(), tl[ph].size() * sizeof(BatchTile),
                                     cudaMemcpyHostToDevice, b->stream));
    }
    LFM_CUDA(cudaMemcpyAsync(b->dNTiles, n, sizeof(n), cudaMemcpyHostToDevice, b->stream));
    // the host vectors die here: wait for the copies out of them
    LFM_CUDA(cudaStreamSynchronize(b->stream));
    const int variant = currentVariant(b);
    if ((realloc || variant != b->variant) && b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->variant = variant;
    b->tilesDirty = false;
    return LFM_OK;
}

BatchArgs makeArgs(lfm_batch* b) {
    BatchArgs a{};
    a.cases = b->dCases;
    for (int ph = 0; ph < kBatchPhases; ++ph) a.tiles[ph] = b->dTiles[ph];
    a.nTiles = b->dNTiles;
    a.ctl = b->dCtl;
    a.error = b->dError;
    a.itemsPerThread = b->tune.items_per_thread;
    a.barrierExtra = b->barrierExtra;
    return a;
}

int captureStep(lfm_batch* b, bool cooperative, cudaGraphExec_t* out) {
    const BatchArgs args = makeArgs(b);
    cudaGraph_t g = nullptr;
    LFM_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaMemsetAsync(b->dCtl, 0, sizeof(BatchCtl), b->stream);
    for (int k = 0; k < b->rkOrder && le == cudaSuccess; ++k)
        le = b->tune.phased ? lfm::dev::launch_batch_phased(args, k, b->tune.block, b->variant, b->tune.blocks_per_sm,
                                                            b->sms, b->stream)
                            : lfm::dev::launch_batch_stage(args, k, b->tune.block, b->variant, b->grid, cooperative,
                                                           b->stream);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (le != cudaSuccess || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return cudaFail(le != cudaSuccess ? le : e, "batch step capture");
    }
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cudaFail(e, "cudaGraphInstantiate");
    }
    return LFM_OK;
}

// Grid of the persistent kernel: blocks_per_sm (0 = all that fit) x SMs,
// never above the resident capacity (the grid barriers need every block
// resident).
int ensureGraph(lfm_batch* b) {
    if (b->tilesDirty) {
        int rc = rebuildTiles(b);
        if (rc) return rc;
    }
    if (b->graph) return LFM_OK;
    if (b->tune.phased) return captureStep(b, false, &b->graph);   // no co-residency needed
    const int fit = lfm::dev::batch_blocks_per_sm(b->tune.block, b->variant);
    if (fit <= 0) return lfm::setError(LFM_ERR_UNSUPPORTED, "batch kernel does not fit on an SM");
    const int bps = b->tune.blocks_per_sm > 0 ? std::min(b->tune.blocks_per_sm, fit) : fit;
    b->grid = bps * b->sms;
    // A cooperative launch guarantees co-residency; where capture of one is
    // refused, a grid within the resident capacity is launched plainly.
    int rc = LFM_ERR_CUDA;
    if (b->tune.cooperative) rc = captureStep(b, true, &b->graph);
    if (rc != LFM_OK) {
        b->tune.cooperative = 0;
        rc = captureStep(b, false, &b->graph);
    }
    return rc;
}

// Device buffer for a case's absolute state in transit to or from the host.
int ensureStage(lfm_batch* b, size_t bytes) {
    if (bytes <= b->stageBytes) return LFM_OK;
    LFM_CUDA(cudaStreamSynchronize(b->stream));
    if (b->dStage) cudaFree(b->dStage);
    b->dStage = nullptr;
    b->stageBytes = 0;
    LFM_CUDA(cudaMalloc(&b->dStage, bytes));
    b->stageBytes = bytes;
    return LFM_OK;
}

int checkSlot(const lfm_batch* b, int slot) {
    if (!b) return lfm::setError(LFM_ERR_INVALID, "null batch");
    if (slot < 0 || slot >= (int)b->slots.size() || !b->slots[(size_t)slot].used)
        return lfm::setError(LFM_ERR_INVALID, "no case in slot " + std::to_string(slot));
    return LFM_OK;
}

}  // namespace

extern "C" int lfm_batch_case_bytes(const lfm_solver_desc* d, size_t* bytes) {
    if (!bytes) return lfm::setError(LFM_ERR_INVALID, "null argument");
    int rc = lfm::setup::validateDesc(d);
    if (rc) return rc;
    *bytes = CaseLayout(d).total;
    return LFM_OK;
}

extern "C" int lfm_batch_create(const lfm_batch_opts* opts, lfm_batch** out) {
    if (!out) return lfm::setError(LFM_ERR_INVALID, "null output handle");
    *out = nullptr;
    lfm_batch_opts o{0, 5, 0, 256};
    if (opts) o = *opts;
    if (o.rk_order < 1 || o.rk_order > kBatchMaxStages) return lfm::setError(LFM_ERR_INVALID, "rk_order out of range");
    if (o.max_cases <= 0) o.max_cases = 256;
    LFM_CUDA(cudaSetDevice(o.device));
    lfm_batch* b = new lfm_batch;
    b->device = o.device;
    b->rkOrder = o.rk_order;
    b->maxCases = o.max_cases;
    auto fail = [&](int rc) {
        lfm_batch_destroy(b);
        return rc;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(cudaFail(e, "cudaStreamCreate"));
    cudaEventCreate(&b->ev0);
    cudaEventCreate(&b->ev1);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    size_t arena = o.arena_bytes;
    if (arena == 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        arena = fr / 4;
    }
    arena = roundUp(arena);
    if ((e = cudaMalloc(&b->arenaBase, arena)) != cudaSuccess) return fail(cudaFail(e, "cudaMalloc arena"));
    b->arena.reset(arena);
    if ((e = cudaMalloc(&b->dCases, sizeof(BatchCase) * (size_t)b->maxCases)) != cudaSuccess ||
        (e = cudaMalloc(&b->dFlags, sizeof(int) * (size_t)b->maxCases)) != cudaSuccess ||
        (e = cudaMalloc(&b->dError, sizeof(int))) != cudaSuccess ||
        (e = cudaMalloc(&b->dCtl, sizeof(BatchCtl))) != cudaSuccess ||
        (e = cudaMalloc(&b->dNTiles, sizeof(int) * kBatchPhases)) != cudaSuccess)
        return fail(cudaFail(e, "cudaMalloc batch tables"));
    cudaMemsetAsync(b->dFlags, 0, sizeof(int) * (size_t)b->maxCases, b->stream);
    cudaMemsetAsync(b->dError, 0, sizeof(int), b->stream);
    cudaMemsetAsync(b->dNTiles, 0, sizeof(int) * kBatchPhases, b->stream);
    b->slots.resize((size_t)b->maxCases);
    if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) return fail(cudaFail(e, "batch create"));
    *out = b;
    return LFM_OK;
}

extern "C" void lfm_batch_destroy(lfm_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (int ph = 0; ph < kBatchPhases; ++ph)
        if (b->dTiles[ph]) cudaFree(b->dTiles[ph]);
    cudaFree(b->arenaBase);
    cudaFree(b->dCases);
    cudaFree(b->dFlags);
    cudaFree(b->dError);
    cudaFree(b->dCtl);
    cudaFree(b->dNTiles);
    if (b->dStage) cudaFree(b->dStage);
    if (b->scrub) cudaFree(b->scrub);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

namespace lfm {
namespace batch {

int prepareCase(const lfm_solver_desc* d, double dt, int rkOrder, PreparedCase** out) {
    *out = nullptr;
    int rc = lfm::setup::validateDesc(d);
    if (rc) return rc;
    if (d->rk_order != rkOrder)
        return lfm::setError(LFM_ERR_INVALID, "case rk_order " + std::to_string(d->rk_order) +
                                                  " differs from the batch's " + std::to_string(rkOrder));
    if (!(dt > 0.0)) return lfm::setError(LFM_ERR_INVALID, "dt must be positive");
    if (d->smag_c)
        return lfm::setError(LFM_ERR_UNSUPPORTED, "Smagorinsky LES cases run in the single-case solver, not in a batch");
    if (d->n_halos > 0)
        return lfm::setError(LFM_ERR_UNSUPPORTED, "partitions of a decomposed case run in an lfm_partitioned");
    PreparedCase* pc = new PreparedCase(d);
    BatchCase& bc = pc->bc;
    std::memset(&bc, 0, sizeof(bc));
    lfm::setup::setConstants(bc.a, d);
    pc->image = packCase(d, pc->layout, bc.a.qRef);
    bc.dt = dt;
    bc.dt32 = (float)dt;
    for (int k = 0; k < d->rk_order; ++k) {
        bc.rkA[k] = d->rkA[k];
        bc.rkB[k] = d->rkB[k];
    }
    bc.scheme = d->solver;
    bc.needGrad = lfm::setup::needGrad(d) ? 1 : 0;
    bc.needVis = lfm::setup::needVis(d) ? 1 : 0;
    bc.residuals = d->residuals ? 1 : 0;
    pc->D = d->dim;
    pc->nq = d->nq;
    pc->nc = (int)d->n_cells;
    pc->ng = (int)d->n_ghosts;
    pc->nf = (int)d->n_faces;
    pc->needGradVis = bc.needGrad || bc.needVis;
    *out = pc;
    return LFM_OK;
}

int commitCase(lfm_batch* b, const PreparedCase& pc, int* slot) {
    *slot = -1;
    int s = -1;
    for (int k = 0; k < (int)b->slots.size(); ++k)
        if (!b->slots[(size_t)k].used) {
            s = k;
            break;
        }
    if (s < 0) return lfm::setError(LFM_ERR_NOMEM, "batch has no free case slot");
    const CaseLayout& L = pc.layout;
    size_t off = 0;
    if (!b->arena.alloc(L.total, &off))
        return lfm::setError(LFM_ERR_NOMEM, "case needs " + std::to_string(L.total) + " bytes; largest free arena block " +
                                                std::to_string(b->arena.largest()));
    LFM_CUDA(cudaSetDevice(b->device));
    unsigned char* base = b->arenaBase + off;
    cudaError_t e = cudaMemcpyAsync(base, pc.image.data(), pc.image.size(), cudaMemcpyHostToDevice, b->stream);
    BatchCase bc = pc.bc;
    Args<float>& a = bc.a;
    auto P = [&](size_t o) -> unsigned char* { return o == CaseLayout::npos() ? nullptr : base + o; };
    a.q = reinterpret_cast<double*>(P(L.q));
    a.dq = reinterpret_cast<float*>(P(L.dq));
    a.res = reinterpret_cast<double*>(P(L.res));
    a.prim = reinterpret_cast<float*>(P(L.prim));
    a.primW = a.prim;
    a.V = reinterpret_cast<float*>(P(L.V));
    a.grad = reinterpret_cast<float*>(P(L.grad));
    a.flux = reinterpret_cast<float*>(P(L.flux));
    a.S = reinterpret_cast<const float*>(P(L.S));
    a.d = reinterpret_cast<const float*>(P(L.d));
    a.w = reinterpret_cast<const float*>(P(L.w));
    a.dinv = reinterpret_cast<const float*>(P(L.dinv));
    a.dnorm = reinterpret_cast<const float*>(P(L.dnorm));
    a.K = reinterpret_cast<const float*>(P(L.K));
    a.lapc = reinterpret_cast<const float*>(P(L.lapc));
    a.fP = reinterpret_cast<const int*>(P(L.fP));
    a.fN = reinterpret_cast<const int*>(P(L.fN));
    a.fGhost = reinterpret_cast<const uint8_t*>(P(L.fGhost));
    a.volInv = reinterpret_cast<const double*>(P(L.volInv));
    a.volInv32 = reinterpret_cast<const float*>(P(L.volInv32));
    a.sponge = reinterpret_cast<const float*>(P(L.sponge));
    a.cfOff = reinterpret_cast<const int*>(P(L.cfOff));
    a.cfList = reinterpret_cast<const int*>(P(L.cfList));
    a.cfNbr = reinterpret_cast<const int*>(P(L.cfNbr));
    a.cellGhosts = reinterpret_cast<const uint8_t*>(P(L.cellGhosts));
    a.cfEll = reinterpret_cast<const int*>(P(L.cfEll));
    a.smagC = nullptr;
    a.gCell = reinterpret_cast<const int*>(P(L.gCell));
    a.gKind = reinterpret_cast<const int*>(P(L.gKind));
    a.gFace = reinterpret_cast<const int*>(P(L.gFace));
    a.flag = b->dFlags + s;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->dCases + s, &bc, sizeof(bc), cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->dFlags + s, 0, sizeof(int), b->stream);
    // bc is a host temporary: the copies must finish before it goes
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) {
        b->arena.release(off, L.total);
        return cudaFail(e, "batch case upload");
    }
    Slot& sl = b->slots[(size_t)s];
    sl.used = true;
    sl.off = off;
    sl.bytes = L.total;
    sl.D = pc.D;
    sl.nq = pc.nq;
    sl.nc = pc.nc;
    sl.ng = pc.ng;
    sl.nf = pc.nf;
    sl.nt = pc.nc + pc.ng;
    sl.needGradVis = pc.needGradVis;
    sl.primsValid = false;
    for (int v = 0; v < 5; ++v) sl.qRef[v] = pc.bc.a.qRef[v];
    sl.q = a.q;
    sl.a = a;
    b->tilesDirty = true;
    *slot = s;
    return LFM_OK;
}

}  // namespace batch
}  // namespace lfm

extern "C" int lfm_batch_add(lfm_batch* b, const lfm_solver_desc* d, double dt, int* slot) {
    if (!b || !slot) return lfm::setError(LFM_ERR_INVALID, "null argument");
    *slot = -1;
    PreparedCase* pc = nullptr;
    int rc = lfm::batch::prepareCase(d, dt, b->rkOrder, &pc);
    if (rc) return rc;
    rc = lfm::batch::commitCase(b, *pc, slot);
    delete pc;
    return rc;
}

extern "C" int lfm_batch_remove(lfm_batch* b, int slot) {
    int rc = checkSlot(b, slot);
    if (rc) return rc;
    LFM_CUDA(cudaSetDevice(b->device));
    // the arena block may still be in use by queued steps
    LFM_CUDA(cudaStreamSynchronize(b->stream));
    Slot& sl = b->slots[(size_t)slot];
    b->arena.release(sl.off, sl.bytes);
    sl = Slot();
    b->tilesDirty = true;
    return LFM_OK;
}

namespace {

// The state copies of one case, enqueued on the batch stream through the
// shared staging buffer (stream order keeps successive cases apart).
int enqueueBatchSet(lfm_batch* b, int slot, const double* q) {
    Slot& sl = b->slots[(size_t)slot];
    // a new state starts with a clear non-finite flag
    LFM_CUDA(cudaMemsetAsync(b->dFlags + slot, 0, sizeof(int), b->stream));
    const size_t bytes = (size_t)sl.nq * sl.nc * sizeof(double);
    int rc = ensureStage(b, bytes);
    if (rc) return rc;
    LFM_CUDA(cudaMemcpyAsync(b->dStage, q, bytes, cudaMemcpyHostToDevice, b->stream));
    // stored as q - qRef, with the primitives of the cells and their ghosts
    // derived in the same pass: the tile lists need no preparation phase
    lfm::dev::launch_set_state32(sl.a, b->dStage, sl.nc, b->stream);
    LFM_CUDA(cudaGetLastError());
    return LFM_OK;
}

int enqueueBatchGet(lfm_batch* b, int slot, double* q) {
    const Slot& sl = b->slots[(size_t)slot];
    const size_t bytes = (size_t)sl.nq * sl.nc * sizeof(double);
    int rc = ensureStage(b, bytes);
    if (rc) return rc;
    lfm::dev::QOffset qo;   // stored as q - qRef
    for (int v = 0; v < 5; ++v) qo.v[v] = sl.qRef[v];
    lfm::dev::launch_offset_rows(b->dStage, sl.nc, sl.q, sl.nt, sl.nc, sl.nq, qo, 1.0, b->stream);
    LFM_CUDA(cudaGetLastError());
    LFM_CUDA(cudaMemcpyAsync(q, b->dStage, bytes, cudaMemcpyDeviceToHost, b->stream));
    return LFM_OK;
}

}  // namespace

extern "C" int lfm_batch_set_state(lfm_batch* b, int slot, const double* q) {
    int rc = checkSlot(b, slot);
    if (rc) return rc;
    if (!q) return lfm::setError(LFM_ERR_INVALID, "null state");
    LFM_CUDA(cudaSetDevice(b->device));
    if ((rc = enqueueBatchSet(b, slot, q))) return rc;
    LFM_CUDA(cudaStreamSynchronize(b->stream));
    return LFM_OK;
}

extern "C" int lfm_batch_get_state(lfm_batch* b, int slot, double* q) {
    int rc = checkSlot(b, slot);
    if (rc) return rc;
    if (!q) return lfm::setError(LFM_ERR_INVALID, "null state");
    LFM_CUDA(cudaSetDevice(b->device));
    if ((rc = enqueueBatchGet(b, slot, q))) return rc;
    LFM_CUDA(cudaStreamSynchronize(b->stream));
    return LFM_OK;
}

extern "C" int lfm_batch_advance(lfm_batch* b, int n, const int* slots, const double* const* q_in, int nsteps,
                                 double* const* q_out) {
    if (!b || n < 0 || (n > 0 && !slots) || nsteps < 0) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    size_t most = 0;
    for (int i = 0; i < n; ++i) {
        int rc = checkSlot(b, slots[i]);
        if (rc) return rc;
        const Slot& sl = b->slots[(size_t)slots[i]];
        most = std::max(most, (size_t)sl.nq * sl.nc * sizeof(double));
    }
    LFM_CUDA(cudaSetDevice(b->device));
    int rc = ensureStage(b, most);   // sized once, before anything is enqueued
    for (int i = 0; i < n && !rc && q_in; ++i)
        if (q_in[i]) rc = enqueueBatchSet(b, slots[i], q_in[i]);
    if (!rc && nsteps > 0) rc = lfm_batch_step(b, nsteps);
    for (int i = 0; i < n && !rc && q_out; ++i)
        if (q_out[i]) rc = enqueueBatchGet(b, slots[i], q_out[i]);
    if (rc) return rc;
    return lfm_batch_sync(b);
}

extern "C" int lfm_batch_step(lfm_batch* b, int nsteps) {
    if (!b) return lfm::setError(LFM_ERR_INVALID, "null batch");
    if (nsteps < 0) return lfm::setError(LFM_ERR_INVALID, "negative step count");
    LFM_CUDA(cudaSetDevice(b->device));
    int rc = ensureGraph(b);
    if (rc) return rc;
    if (nsteps == 0) return LFM_OK;
    // Cases whose state was just set prepare all their cells in the first
    // step; after it the update phase keeps their primitives current and the
    // tile lists shrink to their ghosts.
    bool stale = false;
    for (Slot& sl : b->slots)
        if (sl.used && !sl.primsValid) {
            stale = true;
            sl.primsValid = true;
        }
    LFM_CUDA(cudaGraphLaunch(b->graph, b->stream));
    if (stale) {
        b->tilesDirty = true;
        if ((rc = ensureGraph(b))) return rc;
    }
    for (int k = 1; k < nsteps; ++k) LFM_CUDA(cudaGraphLaunch(b->graph, b->stream));
    return LFM_OK;
}

extern "C" int lfm_batch_sync(lfm_batch* b) {
    if (!b) return lfm::setError(LFM_ERR_INVALID, "null batch");
    LFM_CUDA(cudaSetDevice(b->device));
    LFM_CUDA(cudaStreamSynchronize(b->stream));
    int err = 0;
    LFM_CUDA(cudaMemcpy(&err, b->dError, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) return lfm::setError(LFM_ERR_CUDA, "batch stage kernel: a grid barrier gave up waiting");
    std::vector<int> flags((size_t)b->maxCases);
    LFM_CUDA(cudaMemcpy(flags.data(), b->dFlags, flags.size() * sizeof(int), cudaMemcpyDeviceToHost));
    std::string bad;
    for (int s = 0; s < b->maxCases; ++s)
        if (b->slots[(size_t)s].used && flags[(size_t)s]) bad += (bad.empty() ? "" : ", ") + std::to_string(s);
    if (!bad.empty()) return lfm::setError(LFM_ERR_NUMERIC, "non-finite state in batch slot(s) " + bad);
    return LFM_OK;
}

extern "C" int lfm_batch_case_status(lfm_batch* b, int slot, int* status) {
    int rc = checkSlot(b, slot);
    if (rc) return rc;
    if (!status) return lfm::setError(LFM_ERR_INVALID, "null argument");
    LFM_CUDA(cudaSetDevice(b->device));
    LFM_CUDA(cudaStreamSynchronize(b->stream));
    int f = 0;
    LFM_CUDA(cudaMemcpy(&f, b->dFlags + slot, sizeof(int), cudaMemcpyDeviceToHost));
    *status = f ? LFM_ERR_NUMERIC : LFM_OK;
    return LFM_OK;
}

extern "C" int lfm_batch_memory(const lfm_batch* b, size_t* largest_free, size_t* total_free, size_t* arena_bytes) {
    if (!b) return lfm::setError(LFM_ERR_INVALID, "null batch");
    if (largest_free) *largest_free = b->arena.largest();
    if (total_free) *total_free = b->arena.total();
    if (arena_bytes) *arena_bytes = b->arena.size();
    return LFM_OK;
}

extern "C" int lfm_batch_cells(const lfm_batch* b, int64_t* cells, int* cases) {
    if (!b) return lfm::setError(LFM_ERR_INVALID, "null batch");
    int64_t n = 0;
    int k = 0;
    for (const Slot& s : b->slots)
        if (s.used) {
            n += s.nc;
            ++k;
        }
    if (cells) *cells = n;
    if (cases) *cases = k;
    return LFM_OK;
}

extern "C" int lfm_batch_get_tuning(const lfm_batch* b, lfm_batch_tuning* t) {
    if (!b || !t) return lfm::setError(LFM_ERR_INVALID, "null argument");
    *t = b->tune;
    return LFM_OK;
}

extern "C" int lfm_batch_set_tuning(lfm_batch* b, const lfm_batch_tuning* t) {
    if (!b || !t) return lfm::setError(LFM_ERR_INVALID, "null argument");
    if (t->block != 128 && t->block != 256 && t->block != 512)
        return lfm::setError(LFM_ERR_INVALID, "block must be 128, 256 or 512");
    if (t->items_per_thread < 1 || t->items_per_thread > 16 || t->blocks_per_sm < 0)
        return lfm::setError(LFM_ERR_INVALID, "items_per_thread must be 1..16 and blocks_per_sm >= 0");
    LFM_CUDA(cudaSetDevice(b->device));
    LFM_CUDA(cudaStreamSynchronize(b->stream));
    b->tune = *t;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->tilesDirty = true;
    return LFM_OK;
}

extern "C" int lfm_batch_debug_barrier(lfm_batch* b, int extra_arrivals) {
    if (!b || extra_arrivals < 0) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    LFM_CUDA(cudaSetDevice(b->device));
    LFM_CUDA(cudaStreamSynchronize(b->stream));
    b->barrierExtra = (unsigned)extra_arrivals;
    if (b->graph) {   // the step graph holds the kernels' arguments
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return LFM_OK;
}

namespace {

int flushL2(lfm_batch* b, size_t bytes) {
    if (bytes == 0) return LFM_OK;
    if (b->scrubBytes < bytes) {
        if (b->scrub) cudaFree(b->scrub);
        b->scrub = nullptr;
        b->scrubBytes = 0;
        LFM_CUDA(cudaMalloc(&b->scrub, bytes));
        b->scrubBytes = bytes;
    }
    LFM_CUDA(cudaMemsetAsync(b->scrub, 0x5a, bytes, b->stream));
    return LFM_OK;
}

}  // namespace

extern "C" int lfm_batch_bench(lfm_batch* b, int nsteps, size_t flush_bytes, float* ms) {
    if (!b || !ms || nsteps < 0) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    LFM_CUDA(cudaSetDevice(b->device));
    int rc = ensureGraph(b);
    if (rc) return rc;
    std::vector<cudaEvent_t> ev(2 * (size_t)nsteps);
    for (auto& e : ev) LFM_CUDA(cudaEventCreate(&e));
    bool stale = false;   // as in lfm_batch_step: stale cases prepare all cells in the first step
    for (Slot& sl : b->slots)
        if (sl.used && !sl.primsValid) {
            stale = true;
            sl.primsValid = true;
        }
    for (int k = 0; k < nsteps; ++k) {
        if ((rc = flushL2(b, flush_bytes))) break;
        cudaEventRecord(ev[2 * (size_t)k], b->stream);
        cudaGraphLaunch(b->graph, b->stream);
        cudaEventRecord(ev[2 * (size_t)k + 1], b->stream);
        if (k == 0 && stale) {
            b->tilesDirty = true;
            if ((rc = ensureGraph(b))) break;
        }
    }
    cudaError_t e = cudaStreamSynchronize(b->stream);
    for (int k = 0; k < nsteps && e == cudaSuccess; ++k)
        e = cudaEventElapsedTime(&ms[k], ev[2 * (size_t)k], ev[2 * (size_t)k + 1]);
    for (auto& x : ev) cudaEventDestroy(x);
    if (rc) return rc;
    if (e != cudaSuccess) return cudaFail(e, "batch bench");
    // a timing run reports barrier failures; the cases' numeric state is
    // left to lfm_batch_sync / lfm_batch_case_status
    int err = 0;
    LFM_CUDA(cudaMemcpy(&err, b->dError, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) return lfm::setError(LFM_ERR_CUDA, "batch stage kernel: a grid barrier gave up waiting");
    return LFM_OK;
}

// Tries every (block, items per thread, blocks per SM) candidate on the
// batch's current cases for `trial_steps` steps each and keeps the fastest.
// The cases' states are saved before and restored after.
extern "C" int lfm_batch_autotune(lfm_batch* b, int trial_steps, lfm_batch_tuning* chosen) {
    if (!b) return lfm::setError(LFM_ERR_INVALID, "null batch");
    if (trial_steps < 1) trial_steps = 2;
    LFM_CUDA(cudaSetDevice(b->device));
    LFM_CUDA(cudaStreamSynchronize(b->stream));
    // snapshot of every case's q (cells and ghosts)
    size_t snapBytes = 0;
    for (const Slot& s : b->slots)
        if (s.used) snapBytes += (size_t)s.nq * s.nt * sizeof(double);
    double* snap = nullptr;
    if (snapBytes) LFM_CUDA(cudaMalloc(&snap, snapBytes));
    auto copyStates = [&](bool save) -> cudaError_t {
        size_t at = 0;
        for (const Slot& s : b->slots) {
            if (!s.used) continue;
            const size_t n = (size_t)s.nq * s.nt;
            cudaError_t e = save ? cudaMemcpyAsync(snap + at, s.q, n * 8, cudaMemcpyDeviceToDevice, b->stream)
                                 : cudaMemcpyAsync(s.q, snap + at, n * 8, cudaMemcpyDeviceToDevice, b->stream);
            if (e != cudaSuccess) return e;
            at += n;
        }
        return cudaSuccess;
    };
    cudaError_t e = copyStates(true);
    const lfm_batch_tuning start = b->tune;
    lfm_batch_tuning best = start;
    float bestMs = 1e30f;
    const int blocks[3] = {128, 256, 512};
    const int ipts[3] = {1, 2, 4};
    int rc = LFM_OK;
    for (int bi = 0; bi < 3 && e == cudaSuccess && rc == LFM_OK; ++bi) {
        const int fit = lfm::dev::batch_blocks_per_sm(blocks[bi], currentVariant(b));
        for (int ii = 0; ii < 3 && rc == LFM_OK; ++ii) {
            // persistent kernel at 1..fit blocks per SM, then the phased mode
            // at full occupancy (bps 0)
            for (int bps = 1; bps <= fit + 1 && rc == LFM_OK; ++bps) {
                const bool phased = bps == fit + 1;
                lfm_batch_tuning t{blocks[bi], ipts[ii], phased ? 0 : bps, start.cooperative, phased ? 1 : 0};
                if ((rc = lfm_batch_set_tuning(b, &t))) break;
                if ((rc = lfm_batch_step(b, 1))) break;   // warm-up, builds tiles and graph
                cudaEventRecord(b->ev0, b->stream);
                if ((rc = lfm_batch_step(b, trial_steps))) break;
                cudaEventRecord(b->ev1, b->stream);
                if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) break;
                float ms = 0;
                cudaEventElapsedTime(&ms, b->ev0, b->ev1);
                if (ms < bestMs) {
                    bestMs = ms;
                    best = b->tune;
                }
            }
        }
    }
    if (e == cudaSuccess) e = copyStates(false);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->dFlags, 0, sizeof(int) * (size_t)b->maxCases, b->stream);
    for (Slot& sl : b->slots) sl.primsValid = false;   // restored states: primitives are stale
    b->tilesDirty = true;
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (snap) cudaFree(snap);
    if (rc) return rc;
    if (e != cudaSuccess) return cudaFail(e, "batch autotune");
    rc = lfm_batch_set_tuning(b, &best);
    if (rc) return rc;
    if (chosen) *chosen = best;
    return LFM_OK;
}

extern "C" int lfm_batch_launches_per_step(const lfm_batch* b, int* launches) {
    if (!b || !launches) return lfm::setError(LFM_ERR_INVALID, "null argument");
    *launches = b->rkOrder;
    return LFM_OK;
}
