// Host-side internals of the batch engine shared by the batch C ABI
// (capi_batch.cu) and the request server (capi_server.cu).
#pragma once

#include <cstddef>
#include <map>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "args_setup.h"
#include "batch.cuh"
#include "lfm_gpu.h"
#include "solver_launch.h"

namespace lfm {
namespace batch {

constexpr size_t kAlign = 256;
inline size_t roundUp(size_t b) { return (b + kAlign - 1) & ~(kAlign - 1); }

// First-fit allocator over [0, size) in 256-byte granules; free ranges are
// kept sorted by offset and coalesced on release.
class Arena {
public:
    void reset(size_t size) {
        free_.clear();
        size_ = size & ~(kAlign - 1);
        if (size_) free_[0] = size_;
    }
    bool alloc(size_t bytes, size_t* off) {
        bytes = roundUp(bytes);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes;
                const size_t at = it->first + bytes;
                free_.erase(it);
                if (rest) free_[at] = rest;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = roundUp(bytes);
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t largest() const {
        size_t m = 0;
        for (auto& kv : free_) m = std::max(m, kv.second);
        return m;
    }
    size_t total() const {
        size_t m = 0;
        for (auto& kv : free_) m += kv.second;
        return m;
    }
    size_t size() const { return size_; }

private:
    std::map<size_t, size_t> free_;
    size_t size_ = 0;
};

// Byte offsets of every array of one case inside its arena block.
struct CaseLayout {
    size_t total = 0;
    size_t q, dq, res, prim, V, grad, flux, S, d, w, dinv, dnorm, K, lapc, fP, fN, fGhost, volInv, volInv32,
        sponge, cfOff, cfList, cfNbr, cfEll, cellGhosts, gCell, gKind, gFace;

    explicit CaseLayout(const lfm_solver_desc* d) {
        const size_t D = (size_t)d->dim, nq = (size_t)d->nq, nc = (size_t)d->n_cells, ng = (size_t)d->n_ghosts;
        const size_t nt = nc + ng, nf = (size_t)d->n_faces, ne = (size_t)d->cell_face_offsets[nc];
        const bool ausm = d->solver == LFM_SOLVER_M2AUSM;
        q = add(nq * nt * 8);
        dq = add(nq * nc * 4);
        res = d->residuals ? add(nq * nc * 8) : npos();
        prim = add((size_t)lfm::dev::primRows<float>(d->dim) * nt * 4);
        V = lfm::setup::needVis(d) ? add((D * D + 2 * D) * nt * 4) : npos();
        grad = ausm ? add((2 * D + D * D) * nt * 4) : npos();
        flux = add(nq * nf * 4);
        S = add(D * nf * 4);
        this->d = add(D * nf * 4);
        w = add(nf * 4);
        dinv = add(nf * 4);
        dnorm = add(D * nf * 4);
        K = add(D * nf * 4);
        lapc = add(nf * 4);
        fP = add(nf * 4);
        fN = add(nf * 4);
        fGhost = add(nf);
        volInv = add(nc * 8);
        volInv32 = add(nc * 4);
        sponge = add(nc * 4);
        cfOff = add((nc + 1) * 4);
        cfList = add(ne * 4);
        cfNbr = add(ne * 4);
        // the update's fixed-width cell -> face table, when every cell fits it
        const size_t W = (size_t)(D == 2 ? lfm::dev::kEllWidth<2> : lfm::dev::kEllWidth<3>);
        bool fits = true;
        for (size_t c = 0; c < nc && fits; ++c)
            fits = (size_t)(d->cell_face_offsets[c + 1] - d->cell_face_offsets[c]) <= W;
        cfEll = fits ? add(W * nc * 4) : npos();
        cellGhosts = add(nc);
        gCell = add(ng * 4);
        gKind = add(ng * 4);
        gFace = add(ng * 4);
    }
    static size_t npos() { return ~(size_t)0; }

private:
    size_t add(size_t bytes) {
        const size_t at = total;
        total += roundUp(bytes ? bytes : 1);
        return at;
    }
};

struct Slot {
    bool used = false;
    size_t off = 0, bytes = 0;
    int D = 2, nq = 4, nc = 0, ng = 0, nf = 0, nt = 0;
    bool needGradVis = false;
    bool primsValid = false;   // cells' primitives current (kept so by the update phase)
    double qRef[5] = {0, 0, 0, 0, 0};   // the device state is q - qRef
    double* q = nullptr;   // device
    lfm::dev::Args<float> a{};   // the case's kernel arguments (host copy)
};

// A case ready for admission: its arena block image (constant arrays and
// initial state in device layout) and its kernel constants. Built on the host
// only, so a server can prepare requests on the submitting thread.
struct PreparedCase {
    CaseLayout layout;
    std::vector<unsigned char> image;
    dev::BatchCase bc{};          // constants; device pointers filled at admission
    int D = 2, nq = 4, nc = 0, ng = 0, nf = 0;
    bool needGradVis = false;
    explicit PreparedCase(const lfm_solver_desc* d) : layout(d) {}
};

// Validates a description against the batch's RK order and builds its image.
int prepareCase(const lfm_solver_desc* d, double dt, int rkOrder, PreparedCase** out);
// Admits a prepared case: arena block, upload, case table. LFM_ERR_NOMEM when
// no slot or no arena block of its size is free.
int commitCase(lfm_batch* b, const PreparedCase& pc, int* slot);

}  // namespace batch
}  // namespace lfm

struct lfm_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    int rkOrder = 5;
    int maxCases = 0;
    unsigned char* arenaBase = nullptr;
    lfm::batch::Arena arena;
    lfm::dev::BatchCase* dCases = nullptr;
    int* dFlags = nullptr;
    int* dError = nullptr;
    lfm::dev::BatchCtl* dCtl = nullptr;
    lfm::dev::BatchTile* dTiles[lfm::dev::kBatchPhases] = {};
    size_t tileCap[lfm::dev::kBatchPhases] = {};
    int* dNTiles = nullptr;
    std::vector<lfm::batch::Slot> slots;
    int sms = 0;
    lfm_batch_tuning tune{256, 1, 0, 1, 0};
    int variant = lfm::dev::kBatchVariantGeneral;   // stage-kernel variant of the current cases
    int grid = 0;
    bool tilesDirty = true;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    void* scrub = nullptr;
    size_t scrubBytes = 0;
    double* dStage = nullptr;   // a case's absolute state in transit to or from the host
    size_t stageBytes = 0;
    unsigned barrierExtra = 0;  // lfm_batch_debug_barrier
};
