// C ABI, device half: the solver handle (include/lfm_gpu.h).
//
// A solver owns its device arrays and one CUDA stream. A full time step
// (rk_order stages of 3-5 kernels) is captured once into a CUDA graph and
// replayed; the graph is captured again only when dt changes.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../host/capi_internal.h"
#include "lfm_gpu.h"
#include "../host/tiles.h"
#include "args_setup.h"
#include "solver_launch.h"

using lfm::dev::Args;
using lfm::dev::StageConfig;

namespace {

struct DevBuf {
    void* p = nullptr;
};

}  // namespace

struct lfm_solver {
    int precision = LFM_FP64;
    int device = 0;
    cudaStream_t stream = nullptr;
    int D = 2, nq = 4;
    int nc = 0, ng = 0, nf = 0, nt = 0;
    int scheme = 0, rkOrder = 0;
    bool needGrad = false, needVis = true, residuals = false;
    std::vector<double> rkA, rkB;
    std::vector<void*> allocations;
    Args<double> a64{};
    Args<float> a32{};
    double* q = nullptr;
    double* res = nullptr;
    double* partial = nullptr;
    double* scalar = nullptr;
    int* flag = nullptr;
    int* sOff = nullptr;
    double* cellS = nullptr;
    double* volInv = nullptr;
    cudaGraphExec_t graph = nullptr;
    double graphDt = 0;
    // FP32-bulk: q holds q - q_ref, and the update kernel keeps the cells'
    // primitives current; they are stale after a new state is set.
    bool primsValid = false;
    double qRef[5] = {0, 0, 0, 0, 0};
    double* stage = nullptr;   // FP32-bulk: absolute state [nq][nc] in transit to or from the host
    int nh = 0;                // processor-face halos (partitions of a decomposed case)
    bool ownStream = true;     // false for the partitions of an lfm_partitioned
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    void* scrub = nullptr;
    size_t scrubBytes = 0;
    // post-processing
    double* gS = nullptr;        // [D][ng] FP64 face vector of each ghost's face
    double* gD = nullptr;        // [D][ng] FP64 cell-to-ghost vector
    int* gPatch = nullptr;       // [ng] boundary patch of each ghost (null: not described)
    bool ghostRowsValid = false; // a stage ran since the last set_state (FP64: ghost states stored)
    double lastStageB = 0;       // B coefficient of the last stage run
    double* statAvg = nullptr;   // [nc] sum of p
    double* statRms = nullptr;   // [nc] sum of (p - mean)^2
    double* forceTerms = nullptr;   // [D + D*D][ng]
    int* dPatches = nullptr;
    double* dForces = nullptr;      // [2][patch capacity * D]
    int patchCap = 0;
    int* probeCells = nullptr;
    double* probeHist = nullptr;
    int nProbes = 0, probeCap = 0, probeRecords = 0;
    // fused tile stages (FP32-bulk without halos, tile_kernels.cu): the tiles
    // on the device, a second primitive buffer, and which of the two holds
    // the current primitives (0: a32.prim)
    bool tiled = false;
    lfm::dev::TileArgs tile{};
    float* prim1 = nullptr;
    int primParity = 0;
    // fused flux + update stages (FP32-bulk single case): two primitive
    // buffers alternate like the tile stages'
    bool fluxUpdate = false;
    // FP32-bulk flux kernel variants (lfm_solver_tuning): whether they apply,
    // the cell-centred kernel's owner offsets (kept while another variant
    // runs), and the staged kernel's configuration (stages 0: not staged)
    bool fluxVariants = false;
    int* fOwnDev = nullptr;
    lfm::dev::FluxStaging fluxStaging;
    cudaGraphExec_t graphOdd = nullptr;   // the step graph starting from prim1
    // the non-finite flag's host copy (page-locked: read after one stream sync)
    int* flagHost = nullptr;
    // lfm_solver_advance between page-locked host states as one graph (copy
    // in, conversion, primitives, steps, conversion, copy out, flag), kept
    // for the pointers, step count and dt it was captured with
    cudaGraphExec_t advGraph = nullptr;
    const double* advIn = nullptr;
    double* advOut = nullptr;
    int advSteps = 0;
    double advDt = 0;
};

namespace {

int cudaFail(cudaError_t e, const char* what) {
    return lfm::setError(e == cudaErrorMemoryAllocation ? LFM_ERR_NOMEM : LFM_ERR_CUDA,
                         std::string(what) + ": " + cudaGetErrorString(e));
}

#define LFM_CUDA(call)                                    \
    do {                                                  \
        cudaError_t e__ = (call);                         \
        if (e__ != cudaSuccess) return cudaFail(e__, #call); \
    } while (0)

template <typename X>
int devAlloc(lfm_solver* s, X** out, size_t n) {
    *out = nullptr;
    if (n == 0) n = 1;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, n * sizeof(X));
    if (e != cudaSuccess) return cudaFail(e, "cudaMalloc");
    s->allocations.push_back(p);
    e = cudaMemsetAsync(p, 0, n * sizeof(X), s->stream);
    if (e != cudaSuccess) return cudaFail(e, "cudaMemsetAsync");
    *out = static_cast<X*>(p);
    return LFM_OK;
}

template <typename X>
int upload(lfm_solver* s, X** out, const X* src, size_t n) {
    int rc = devAlloc(s, out, n);
    if (rc) return rc;
    if (n) LFM_CUDA(cudaMemcpyAsync(*out, src, n * sizeof(X), cudaMemcpyHostToDevice, s->stream));
    return LFM_OK;
}

// Converts an FP64 host array to T and uploads it.
template <typename T>
int uploadAs(lfm_solver* s, T** out, const double* src, size_t n) {
    std::vector<T> tmp(n);
    for (size_t k = 0; k < n; ++k) tmp[k] = (T)src[k];
    int rc = upload(s, out, tmp.data(), n);
    if (rc) return rc;
    return cudaStreamSynchronize(s->stream) == cudaSuccess ? LFM_OK : cudaFail(cudaGetLastError(), "upload");
}

std::vector<int> toInt(const int64_t* p, size_t n) {
    std::vector<int> v(n);
    for (size_t k = 0; k < n; ++k) v[k] = (int)p[k];
    return v;
}

template <typename T>
int buildArgs(lfm_solver* s, const lfm_solver_desc* d, Args<T>& a, const int* fP, const int* fN,
              const uint8_t* fGhost, const int* cfOff, const int* cfList, const int* cfNbr, const int* gCell,
              const int* gKind,
              const int* gFace) {
    lfm::setup::setConstants(a, d);
    a.q = s->q;
    a.res = s->res;
    a.fP = fP;
    a.fN = fN;
    a.fGhost = fGhost;
    a.volInv = s->volInv;
    a.cfOff = cfOff;
    a.cfList = cfList;
    a.cfNbr = cfNbr;
    a.gCell = gCell;
    a.gKind = gKind;
    a.gFace = gFace;
    a.flag = s->flag;
    a.cellGhosts = nullptr;
    a.cfEll = nullptr;
    a.fOwn = nullptr;
    a.smagC = nullptr;
    a.wN = nullptr;
    a.cfSoN = nullptr;
    a.cellSoW = nullptr;
    a.primC = s->scheme == LFM_SOLVER_M2AUSM ? 1 : 0;
    const size_t nt = (size_t)s->nt, nf = (size_t)s->nf, D = (size_t)s->D;
    int rc;
    if ((rc = devAlloc(s, &a.dq, (size_t)s->nq * s->nc))) return rc;
    if ((rc = devAlloc(s, &a.prim, (size_t)lfm::dev::primRows<T>(s->D) * nt))) return rc;
    a.primW = a.prim;
    if ((rc = devAlloc(s, &a.V, (D * D + 2 * D + (d->smag_c ? D * D : 0)) * nt))) return rc;
    // M2AUSM always reads the gradients (all zero when minmod is off, as in the
    // reference, whose prepare_for_RKstep zeroes them every stage).
    if ((rc = devAlloc(s, &a.grad, (2 * D + D * D) * (s->scheme == LFM_SOLVER_M2AUSM ? nt : 1)))) return rc;
    if ((rc = devAlloc(s, &a.flux, (size_t)s->nq * nf))) return rc;
    T* p;
    if ((rc = uploadAs<T>(s, &p, d->S, D * nf))) return rc;
    a.S = p;
    if ((rc = uploadAs<T>(s, &p, d->d, D * nf))) return rc;
    a.d = p;
    if ((rc = uploadAs<T>(s, &p, d->w, nf))) return rc;
    a.w = p;
    if ((rc = uploadAs<T>(s, &p, d->smag, nf))) return rc;
    a.smag = p;
    if ((rc = uploadAs<T>(s, &p, d->dmag_inv, nf))) return rc;
    a.dinv = p;
    if ((rc = uploadAs<T>(s, &p, d->dnorm, D * nf))) return rc;
    a.dnorm = p;
    if ((rc = uploadAs<T>(s, &p, d->delta_mag, nf))) return rc;
    a.dmag = p;
    if ((rc = uploadAs<T>(s, &p, d->K, D * nf))) return rc;
    a.K = p;
    if ((rc = uploadAs<T>(s, &p, d->sponge, (size_t)s->nc))) return rc;
    a.sponge = p;
    if (d->smag_c) {
        // Smagorinsky LES: a cell's tauMC ends with the constant of the cell
        // that visits it last in the reference's face loop, the owner of the
        // last face (in processing order) it touches - itself unless it owns
        // no face (calc_VIS_Smagorinsky, src/cfd_v0.cpp:1596-1737)
        std::vector<double> cf((size_t)s->nc);
        for (int64_t c = 0; c < s->nc; ++c) {
            // a cell's entries are in processing order: the last is its last face
            const int64_t e0 = d->cell_face_offsets[c], e1 = d->cell_face_offsets[c + 1];
            cf[(size_t)c] = d->smag_c[e1 > e0 ? d->face_p[d->cell_faces[e1 - 1]] : c];
        }
        if ((rc = uploadAs<T>(s, &p, cf.data(), cf.size()))) return rc;
        a.smagC = p;
    }
    {
        std::vector<double> lapc(nf);
        for (size_t f = 0; f < nf; ++f) lapc[f] = d->delta_mag[f] * d->dmag_inv[f];
        if ((rc = uploadAs<T>(s, &p, lapc.data(), nf))) return rc;
        a.lapc = p;
    }
    if (sizeof(T) == sizeof(double)) {
        // FP64 face, face-entry and cell constants, each the value the kernels
        // would otherwise compute per face visit: 1 - w per face; for the
        // Gauss gradients, with the face value v_f = w v_P + (1 - w) v_N and
        // so_e = S/V of entry e's face seen from its cell c,
        //   sum_e v_f so_e = v_c sum_e w_own so_e + sum_e v_across w_across so_e,
        // the first sum a cell constant, w_across so_e an entry constant
        // (w_own = w where c is P, 1 - w where c is N)
        std::vector<double> wN(nf);
        for (size_t f = 0; f < nf; ++f) wN[f] = 1.0 - d->w[f];
        if ((rc = uploadAs<T>(s, &p, wN.data(), nf))) return rc;
        a.wN = p;
        const size_t ne = (size_t)d->cell_face_offsets[s->nc], nc = (size_t)s->nc;
        std::vector<double> soN(D * ne), soW(D * nc, 0.0);
        for (size_t c = 0; c < nc; ++c)
            for (int64_t e = d->cell_face_offsets[c]; e < d->cell_face_offsets[c + 1]; ++e) {
                const int64_t f = d->cell_faces[e];
                const bool isP = d->cell_face_sign[e] > 0;
                const double wOwn = isP ? d->w[f] : wN[(size_t)f], wAcross = isP ? wN[(size_t)f] : d->w[f];
                for (size_t k = 0; k < D; ++k) {
                    const double Sk = d->S[k * nf + (size_t)f];
                    const double so = isP ? Sk * d->vol_inv[c] : -Sk * d->vol_inv[c];
                    soN[(size_t)e * D + k] = wAcross * so;   // entry-major: one entry's D values together
                    soW[c * D + k] += wOwn * so;
                }
            }
        if ((rc = uploadAs<T>(s, &p, soN.data(), soN.size()))) return rc;
        a.cfSoN = p;
        if ((rc = uploadAs<T>(s, &p, soW.data(), soW.size()))) return rc;
        a.cellSoW = p;
    }
    a.volInv32 = nullptr;
    if (sizeof(T) == sizeof(float)) {
        float* v32;
        if ((rc = uploadAs<float>(s, &v32, d->vol_inv, (size_t)s->nc))) return rc;
        a.volInv32 = v32;
    }
    return LFM_OK;
}

StageConfig stageConfig(const lfm_solver* s, int k, double dt) {
    StageConfig c;
    c.scheme = s->scheme;
    c.needGrad = s->needGrad;
    c.needVis = s->needVis;
    c.A = s->rkA[(size_t)k];
    c.B = s->rkB[(size_t)k];
    c.dt = dt;
    c.first = (k == 0);
    c.withRes = (s->residuals && k == 0) ? 1 : 0;
    c.fullPrep = false;   // FP32-bulk: cells' primitives come from the previous update
    if (s->precision == LFM_FP32_BULK) c.fluxStaging = s->fluxStaging;
    return c;
}

template <typename T>
void stageAll(lfm_solver* s, const Args<T>& a, double dt) {
    for (int k = 0; k < s->rkOrder; ++k) lfm::dev::launch_stage<T>(a, stageConfig(s, k, dt), s->stream);
}

// Fused tile stage k of a step that starts from primitive buffer `parity`:
// reads buffer (parity + k) % 2, writes the other.
void tileStage(lfm_solver* s, int k, double dt, int parity) {
    float* buf[2] = {s->a32.prim, s->prim1};
    const int in = (parity + k) & 1;
    Args<float> g = s->a32;
    g.prim = buf[in ^ 1];
    g.primW = g.prim;
    lfm::dev::TileArgs t = s->tile;
    t.primIn = buf[in];
    lfm::dev::launch_tile_stage(g, t, stageConfig(s, k, dt), s->stream);
}

// Stage kernels that alternate two primitive buffers (tile stages, fused
// flux + update stages).
bool alternating(const lfm_solver* s) { return s->tiled || s->fluxUpdate; }

// Fused flux + update stage k of a step that starts from primitive buffer
// `parity`: the preparation (halos and ghosts it still has), gradient and
// viscous kernels read buffer (parity + k) % 2, the fused kernel writes the
// other.
void fluxUpdateStage(lfm_solver* s, int k, double dt, int parity) {
    float* buf[2] = {s->a32.prim, s->prim1};
    const int in = (parity + k) & 1;
    Args<float> g = s->a32;
    g.prim = buf[in];
    g.primW = buf[in ^ 1];
    const StageConfig c = stageConfig(s, k, dt);
    for (int w = 0; w < 3; ++w) lfm::dev::launch_kernel<float>(g, c, w, s->stream);   // prep, grad, vis
    lfm::dev::launch_fluxupdate32(g, c, s->stream);
}

// The alternating stages keep the current primitives in either buffer; the
// other kernels read a32.prim. Before those run, the primitives are rebuilt
// there from the state when they sit in the other buffer.
void untile(lfm_solver* s) {
    if (alternating(s) && s->primParity != 0) {
        s->primsValid = false;
        s->primParity = 0;
    }
}

// Called before stages are launched: primitives of every cell (and the
// ghosts' states and primitives) from the stored state, once after a new state
// -- the update kernels keep them current afterwards.
int ensurePrims(lfm_solver* s) {
    s->ghostRowsValid = true;
    s->lastStageB = s->rkB.empty() ? 0.0 : s->rkB.back();
    if (s->primsValid) return LFM_OK;
    s->primParity = 0;   // rebuilt into a32.prim
    StageConfig c;
    c.fullPrep = true;
    if (s->precision == LFM_FP32_BULK)
        lfm::dev::launch_kernel<float>(s->a32, c, 0, s->stream);
    else
        lfm::dev::launch_kernel<double>(s->a64, c, 0, s->stream);
    LFM_CUDA(cudaGetLastError());
    s->primsValid = true;
    return LFM_OK;
}

void launchStep(lfm_solver* s, double dt, int parity) {
    if (s->tiled)
        for (int k = 0; k < s->rkOrder; ++k) tileStage(s, k, dt, parity);
    else if (s->fluxUpdate)
        for (int k = 0; k < s->rkOrder; ++k) fluxUpdateStage(s, k, dt, parity);
    else if (s->precision == LFM_FP32_BULK)
        stageAll<float>(s, s->a32, dt);
    else
        stageAll<double>(s, s->a64, dt);
}

int captureStep(lfm_solver* s, double dt, int parity, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    LFM_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    launchStep(s, dt, parity);
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (e != cudaSuccess) return cudaFail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cudaFail(e, "cudaGraphInstantiate");
    return LFM_OK;
}

// One graph per time step; with tile stages a second one for steps that
// start from prim1 (an odd stage count swaps the buffers every step).
int ensureGraph(lfm_solver* s, double dt) {
    if (s->graph && s->graphDt == dt) return LFM_OK;
    if (s->graph) cudaGraphExecDestroy(s->graph);
    if (s->graphOdd) cudaGraphExecDestroy(s->graphOdd);
    s->graph = s->graphOdd = nullptr;
    int rc = captureStep(s, dt, 0, &s->graph);
    if (!rc && alternating(s)) rc = captureStep(s, dt, 1, &s->graphOdd);
    if (rc) return rc;
    s->graphDt = dt;
    return LFM_OK;
}

// Launches the step graph matching the current primitive buffer.
cudaError_t launchStepGraph(lfm_solver* s) {
    const cudaError_t e = cudaGraphLaunch(alternating(s) && s->primParity ? s->graphOdd : s->graph, s->stream);
    if (alternating(s)) s->primParity ^= (s->rkOrder & 1);
    return e;
}

}  // namespace

namespace {

// FP32-bulk: the update kernel writes the boundary ghosts' next state (no
// preparation launch per stage) up to these cell counts. The ghost branch
// raises the update kernel's registers (2D 32 -> 48, 3D 32 -> 58); measured on
// GB300 the saved launch wins for a 393k-cell 2D case (0.224 against 0.239 ms
// per step) and the lower occupancy loses for a 1.57M-cell 2D case (0.838
// against 0.826) and for a 9.4M-cell 3D case (8.65 against 7.75 ms).
constexpr int kFuseGhostCells2D = 1 << 20;
constexpr int kFuseGhostCells3D = 1 << 18;

// Fused tile stages (tile_kernels.cu): cells per tile, 0 = off. Off by
// default: measured on GB300 (768x512 cylinder, Hilbert order, FP32-bulk M1)
// a step took 0.352 ms in 256-cell tiles against 0.226 ms with the separate
// kernels - each block runs its load, viscous, flux and update phases one
// after another at 3-4 resident blocks per SM, which hides less latency
// than the separate kernels at full occupancy. LFM_TILE_CELLS=<n> in the
// environment turns them on for a solver created afterwards.
constexpr int kTileCells = 0;
constexpr int kTileMaxLocal2D = 600;   // a tile's cells with their two rings
constexpr int kTileMaxLocal3D = 360;
constexpr size_t kMaxTileSmem = 96 * 1024;
// Cells staged per cell (tile cells and their rings) above which the separate
// kernels are used instead: a cell order whose runs are strips rather than
// patches (renumbering fixes that, lfm_params.renumber).
constexpr double kMaxTileStaging = 2.5;

// Arrays the flux reads: viscous terms when they are computed or M2AUSM
// reads them (its shock sensor), gradients for M2AUSM (zero without minmod).
bool tileHaveV(const lfm_solver* s) { return s->needVis || s->scheme == LFM_SOLVER_M2AUSM; }
bool tileHaveGrad(const lfm_solver* s) { return s->scheme == LFM_SOLVER_M2AUSM; }

int tileCellsOption() {
    const char* e = getenv("LFM_TILE_CELLS");
    return e ? atoi(e) : kTileCells;
}

// Faces stored by owned-face slot (orderFacesBySlot), by dimension.
constexpr bool kFaceOrderBySlot3D = false;

// Fused flux + update stages (LFM_FLUX_UPDATE=0/1 in the environment
// overrides for a solver created afterwards). Measured on GB300, FP32-bulk,
// per step: the 256 x 256 inviscid M1 vortex 0.075 -> 0.070 ms; the 768 x 512
// viscous cylinder 0.192 -> 0.259 ms (M1), 0.198 -> 0.255 (M2), 0.45 -> 0.89
// (M2AUSM); a 96 x 64 x 24 viscous 3D wake 0.201 -> 0.263. Each face is
// evaluated twice, and with the viscous rows of both cells the fused kernel
// needs 64 (2D) to 123 (3D M2AUSM) registers: it gains only where the flux is
// short, the inviscid M1/M2 cases.
bool fluxUpdateOption(const lfm_solver* s) {
    const char* e = getenv("LFM_FLUX_UPDATE");
    if (e) return atoi(e) != 0;
    return s->D == 2 && !s->needVis && s->scheme != LFM_SOLVER_M2AUSM;
}

// Cell-centred flux kernel (flux32_cell), on for 3D cases. Measured on
// GB300, FP32-bulk M2, per step: the 9.4M-cell wake's flux 3.42 -> 3.27 ms
// (the step 6.97 -> 6.82), the 1.18M-cell wake's 0.445 -> 0.416; the 768 x 512
// M1 cylinder's 0.068 -> 0.085 (a 2D cell owns two faces, too few to repay
// the registers it keeps). LFM_FLUX_CELL=0/1 in the environment overrides
// for a solver created afterwards.
bool fluxCellOption(const lfm_solver* s) {
    const char* e = getenv("LFM_FLUX_CELL");
    return e ? atoi(e) != 0 : s->D == 3;
}

// Staged flux kernel (flux_staged_fp32.cu): shared-memory buffers per
// thread (the staging depth; 0 = the plain or cell-centred flux kernel, 1 =
// the slot form) and faces per block. Off: measured slower in every
// configuration (flux_staged_fp32.cu gives the numbers).
// LFM_FLUX_STAGES=<0..4> and LFM_FLUX_FACES=<32..256> in the environment
// override the defaults for a solver created afterwards.
constexpr int kFluxStages = 0;
constexpr int kFluxFaces = 128;

lfm::dev::FluxStaging fluxStagingOption(const lfm_solver* s) {
    (void)s;
    lfm::dev::FluxStaging fs;
    const char* e = getenv("LFM_FLUX_STAGES");
    fs.stages = e ? atoi(e) : kFluxStages;
    if (fs.stages < 1 || fs.stages > 4) fs.stages = 0;
    const char* f = getenv("LFM_FLUX_FACES");
    fs.faces = f ? atoi(f) : kFluxFaces;
    return fs;
}

// Device storage order of the flux faces. The description lists them in the
// reference's processing order, cell by cell: face f is the k-th face that
// its cell P owns (k = its slot). Stored by slot instead -- every cell's
// first owned face, then every cell's second, ... -- the threads of a warp in
// the flux kernel read 32 consecutive cells on the P side and, on a
// structured mesh, 32 consecutive cells on the N side, and every face array
// in whole lines. Each face's rhs is the same value in either order and each
// cell still sums its faces in processing order (the entries of its face
// list keep their order, only the indices are renamed), so results keep
// their bits. LFM_FACE_ORDER=processing|slot in the environment overrides
// the default for a solver created afterwards.
struct FaceOrder {
    lfm_solver_desc desc{};
    std::vector<int64_t> faceP, faceN, cellFaces;
    std::vector<uint8_t> ghost;
    std::vector<double> S, dv, w, smag, dinv, dnorm, dmag, K;
};

bool faceOrderBySlot(const lfm_solver_desc* d) {
    if (tileCellsOption() > 0) return false;   // the tiles are cut from the processing order
    const char* e = getenv("LFM_FACE_ORDER");
    if (e) return std::string(e) == "slot";
    return kFaceOrderBySlot3D && d->dim == 3;
}

// fo.desc = *d with the faces in slot order.
void orderFacesBySlot(const lfm_solver_desc* d, FaceOrder& fo) {
    const size_t nf = (size_t)d->n_faces, D = (size_t)d->dim;
    std::vector<int> slot(nf, 0);
    for (size_t f = 1; f < nf; ++f) slot[f] = d->face_p[f] == d->face_p[f - 1] ? slot[f - 1] + 1 : 0;
    std::vector<int64_t> order(nf);   // new position -> original face
    for (size_t f = 0; f < nf; ++f) order[f] = (int64_t)f;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return slot[(size_t)a] < slot[(size_t)b]; });
    std::vector<int64_t> pos(nf);     // original face -> new position
    for (size_t i = 0; i < nf; ++i) pos[(size_t)order[i]] = (int64_t)i;
    auto perm1 = [&](const auto* src, auto& dst) {
        dst.resize(nf);
        for (size_t i = 0; i < nf; ++i) dst[i] = src[order[i]];
    };
    auto permD = [&](const double* src, std::vector<double>& dst) {
        dst.resize(D * nf);
        for (size_t k = 0; k < D; ++k)
            for (size_t i = 0; i < nf; ++i) dst[k * nf + i] = src[k * nf + (size_t)order[i]];
    };
    perm1(d->face_p, fo.faceP);
    perm1(d->face_n, fo.faceN);
    perm1(d->face_ghost, fo.ghost);
    permD(d->S, fo.S);
    permD(d->d, fo.dv);
    perm1(d->w, fo.w);
    perm1(d->smag, fo.smag);
    perm1(d->dmag_inv, fo.dinv);
    permD(d->dnorm, fo.dnorm);
    perm1(d->delta_mag, fo.dmag);
    permD(d->K, fo.K);
    const size_t ne = (size_t)d->cell_face_offsets[d->n_cells];
    fo.cellFaces.resize(ne);
    for (size_t e = 0; e < ne; ++e) fo.cellFaces[e] = pos[(size_t)d->cell_faces[e]];
    fo.desc = *d;
    fo.desc.face_p = fo.faceP.data();
    fo.desc.face_n = fo.faceN.data();
    fo.desc.face_ghost = fo.ghost.data();
    fo.desc.S = fo.S.data();
    fo.desc.d = fo.dv.data();
    fo.desc.w = fo.w.data();
    fo.desc.smag = fo.smag.data();
    fo.desc.dmag_inv = fo.dinv.data();
    fo.desc.dnorm = fo.dnorm.data();
    fo.desc.delta_mag = fo.dmag.data();
    fo.desc.K = fo.K.data();
    fo.desc.cell_faces = fo.cellFaces.data();
}

// Creates a solver; `stream` (not owned) is shared by the partitions of a
// decomposed case, which alone may carry processor-face halos.
int createSolver(const lfm_solver_desc* d, const lfm_solver_opts* opts, cudaStream_t stream, lfm_solver** out) {
    if (!out) return lfm::setError(LFM_ERR_INVALID, "null output handle");
    *out = nullptr;
    int rc = lfm::setup::validateDesc(d);
    if (rc) return rc;
    FaceOrder faceOrder;
    if (faceOrderBySlot(d)) {
        orderFacesBySlot(d, faceOrder);
        d = &faceOrder.desc;
    }
    if (d->n_halos > 0 && !stream)
        return lfm::setError(LFM_ERR_INVALID, "a partition with processor-face halos runs in an lfm_partitioned");
    lfm_solver* s = new lfm_solver;
    s->precision = opts ? opts->precision : LFM_FP64;
    s->device = opts ? opts->device : 0;
    if (s->precision != LFM_FP64 && s->precision != LFM_FP32_BULK) {
        delete s;
        return lfm::setError(LFM_ERR_INVALID, "unknown precision");
    }
    auto fail = [&](int code) {
        lfm_solver_destroy(s);
        return code;
    };
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) {
        delete s;
        return cudaFail(e, "cudaSetDevice");
    }
    if (stream) {
        s->stream = stream;
        s->ownStream = false;
    } else if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        delete s;
        return cudaFail(e, "cudaStreamCreate");
    }
    cudaEventCreate(&s->ev0);
    cudaEventCreate(&s->ev1);
    s->D = d->dim;
    s->nq = d->nq;
    s->nc = (int)d->n_cells;
    s->ng = (int)d->n_ghosts;
    s->nf = (int)d->n_faces;
    s->nh = (int)d->n_halos;
    s->nt = s->nc + s->ng + s->nh;
    s->scheme = d->solver;
    s->rkOrder = d->rk_order;
    s->rkA.assign(d->rkA, d->rkA + d->rk_order);
    s->rkB.assign(d->rkB, d->rkB + d->rk_order);
    s->needGrad = lfm::setup::needGrad(d);
    s->needVis = lfm::setup::needVis(d);
    s->residuals = d->residuals != 0;

    const size_t nq = (size_t)s->nq, nc = (size_t)s->nc, nt = (size_t)s->nt, nf = (size_t)s->nf;
    if ((rc = devAlloc(s, &s->q, nq * nt))) return fail(rc);
    if ((rc = devAlloc(s, &s->res, s->residuals ? nq * nc : 1))) return fail(rc);
    const size_t nPartial = (nc + 255) / 256 + 1;
    if ((rc = devAlloc(s, &s->partial, nPartial))) return fail(rc);
    if ((rc = devAlloc(s, &s->scalar, 16))) return fail(rc);
    if ((rc = devAlloc(s, &s->flag, 1))) return fail(rc);
    if ((rc = upload(s, &s->volInv, d->vol_inv, nc))) return fail(rc);

    // connectivity as 32-bit indices
    std::vector<int> fP = toInt(d->face_p, nf), fN = toInt(d->face_n, nf);
    std::vector<int> cfOff = toInt(d->cell_face_offsets, nc + 1);
    const size_t ne = (size_t)d->cell_face_offsets[nc];
    std::vector<int> cfList(ne), cfNbr(ne);
    for (size_t k = 0; k < ne; ++k) {
        const int64_t f = d->cell_faces[k];
        cfList[k] = d->cell_face_sign[k] > 0 ? (int)f : ~(int)f;
        cfNbr[k] = (int)(d->cell_face_sign[k] > 0 ? d->face_n[f] : d->face_p[f]);
    }
    std::vector<int> gCell = toInt(d->ghost_cell, (size_t)s->ng), gKind((size_t)s->ng), gFace((size_t)s->ng, 0);
    for (int g = 0; g < s->ng; ++g) gKind[(size_t)g] = d->ghost_kind[g];
    for (int f = 0; f < s->nf; ++f)   // ghosts only (halos follow them)
        if (fN[(size_t)f] >= s->nc && fN[(size_t)f] < s->nc + s->ng) gFace[(size_t)(fN[(size_t)f] - s->nc)] = f;
    std::vector<int> sOff = toInt(d->cell_s_offsets, nc + 1);
    int *dP, *dN, *dOff, *dList, *dNbr, *dGC, *dGK, *dGF;
    uint8_t* dG;
    if ((rc = upload(s, &dP, fP.data(), nf))) return fail(rc);
    if ((rc = upload(s, &dN, fN.data(), nf))) return fail(rc);
    if ((rc = upload(s, &dG, d->face_ghost, nf))) return fail(rc);
    if ((rc = upload(s, &dOff, cfOff.data(), nc + 1))) return fail(rc);
    if ((rc = upload(s, &dList, cfList.data(), ne))) return fail(rc);
    if ((rc = upload(s, &dNbr, cfNbr.data(), ne))) return fail(rc);
    if ((rc = upload(s, &dGC, gCell.data(), (size_t)s->ng))) return fail(rc);
    if ((rc = upload(s, &dGK, gKind.data(), (size_t)s->ng))) return fail(rc);
    if ((rc = upload(s, &dGF, gFace.data(), (size_t)s->ng))) return fail(rc);
    if ((rc = upload(s, &s->sOff, sOff.data(), nc + 1))) return fail(rc);
    if ((rc = upload(s, &s->cellS, d->cell_s, (size_t)d->cell_s_offsets[nc] * (size_t)s->D))) return fail(rc);
    if (s->precision == LFM_FP32_BULK)
        rc = buildArgs<float>(s, d, s->a32, dP, dN, dG, dOff, dList, dNbr, dGC, dGK, dGF);
    else
        rc = buildArgs<double>(s, d, s->a64, dP, dN, dG, dOff, dList, dNbr, dGC, dGK, dGF);
    if (rc) return fail(rc);
    // fused tile stages: FP32-bulk without halos, when a block's tile fits
    lfm::TileSet tiles;
    bool tiled = false;
    if (s->precision == LFM_FP32_BULK && s->nh == 0 && !d->smag_c) {
        const int tc = tileCellsOption();
        if (tc > 0) {
            try {
                tiles = lfm::buildTiles(d, tc, s->D == 2 ? kTileMaxLocal2D : kTileMaxLocal3D);
                tiled = lfm::dev::tile_smem_bytes(s->D, tiles.maxL, tiles.maxLF, tileHaveV(s), tileHaveGrad(s)) <=
                            kMaxTileSmem &&
                        (double)tiles.localCells <= kMaxTileStaging * (double)s->nc;
            } catch (const std::exception&) {
                tiled = false;
            }
        }
    }
    // the tile stages need the update to write the ghosts; the FP64 update
    // always writes them (its kernel is bound by the FP64 pipe, not by the
    // registers the ghost branch adds)
    if (s->precision == LFM_FP64 ||
        tiled || s->nc <= (s->D == 2 ? kFuseGhostCells2D : kFuseGhostCells3D)) {
        // cells with boundary faces: their update writes the ghosts' next state
        std::vector<uint8_t> cg(nc, 0);
        for (size_t f = 0; f < nf; ++f)
            if (fN[f] >= s->nc && fN[f] < s->nc + s->ng) cg[(size_t)fP[f]] = 1;
        uint8_t* dCG = nullptr;
        if ((rc = upload(s, &dCG, cg.data(), nc))) return fail(rc);
        if (s->precision == LFM_FP32_BULK) s->a32.cellGhosts = dCG;
        else s->a64.cellGhosts = dCG;
    }
    if (s->precision == LFM_FP32_BULK && !tiled && (s->D == 3 || s->nc > kFuseGhostCells2D)) {
        // the update's fixed-width cell -> face table, when every cell fits it:
        // cases whose gathers come from HBM (3D; 2D beyond 1M cells, 0.263 ->
        // 0.255 ms per step on a 1.57M-cell cylinder); a 2D case that L2 holds
        // loses more L2 hits to the extra table than the shorter gather saves
        const size_t W = (size_t)(s->D == 2 ? lfm::dev::kEllWidth<2> : lfm::dev::kEllWidth<3>);
        bool fits = true;
        for (size_t c = 0; c < nc && fits; ++c) fits = (size_t)(cfOff[c + 1] - cfOff[c]) <= W;
        if (fits) {
            std::vector<int> ell(W * nc, lfm::dev::kEllPad);
            for (size_t c = 0; c < nc; ++c)
                for (int e = cfOff[c]; e < cfOff[c + 1]; ++e) ell[(size_t)(e - cfOff[c]) * nc + c] = cfList[(size_t)e];
            int* dEll = nullptr;
            if ((rc = upload(s, &dEll, ell.data(), W * nc))) return fail(rc);
            s->a32.cfEll = dEll;
        }
    }
    {   // ghost face geometry in FP64 and patch ids (post-processing)
        const size_t ng = (size_t)s->ng, D = (size_t)s->D;
        std::vector<double> gs(D * ng), gd(D * ng);
        for (size_t g = 0; g < ng; ++g)
            for (size_t k = 0; k < D; ++k) {
                gs[k * ng + g] = d->S[k * nf + (size_t)gFace[g]];
                gd[k * ng + g] = d->d[k * nf + (size_t)gFace[g]];
            }
        if ((rc = upload(s, &s->gS, gs.data(), D * ng))) return fail(rc);
        if ((rc = upload(s, &s->gD, gd.data(), D * ng))) return fail(rc);
        if (d->ghost_patch) {
            std::vector<int> gp(ng);
            for (size_t g = 0; g < ng; ++g) gp[g] = (int)d->ghost_patch[g];
            if ((rc = upload(s, &s->gPatch, gp.data(), ng))) return fail(rc);
        }
    }
    if (tiled) {
        lfm::TileDesc* dT = nullptr;
        int* dI = nullptr;
        float* dF = nullptr;
        uint8_t* dB = nullptr;
        if ((rc = upload(s, &dT, tiles.tiles.data(), tiles.tiles.size()))) return fail(rc);
        if ((rc = upload(s, &dI, tiles.ints.data(), tiles.ints.size()))) return fail(rc);
        if ((rc = upload(s, &dF, tiles.floats.data(), tiles.floats.size()))) return fail(rc);
        if ((rc = upload(s, &dB, tiles.bytes.data(), tiles.bytes.size()))) return fail(rc);
        if ((rc = devAlloc(s, &s->prim1, (size_t)lfm::dev::primRows<float>(s->D) * nt))) return fail(rc);
        s->tile.tiles = dT;
        s->tile.ints = dI;
        s->tile.floats = dF;
        s->tile.bytes = dB;
        s->tile.nTiles = (int)tiles.tiles.size();
        s->tile.smemBytes = lfm::dev::tile_smem_bytes(s->D, tiles.maxL, tiles.maxLF, tileHaveV(s), tileHaveGrad(s));
        s->tile.needGrad = s->needGrad ? 1 : 0;
        s->tile.needVis = s->needVis ? 1 : 0;
        s->tile.haveV = tileHaveV(s) ? 1 : 0;
        s->tile.haveGrad = tileHaveGrad(s) ? 1 : 0;
        s->tile.block = tiles.tileCells <= 128 ? 128 : 256;
        s->tiled = true;
    }
    // fused flux + update stages: FP32-bulk single cases whose update writes
    // the ghosts (no processor halos, laminar, no tile stages)
    if (s->precision == LFM_FP32_BULK && !tiled && s->nh == 0 && !d->smag_c && s->a32.cellGhosts &&
        fluxUpdateOption(s)) {
        if ((rc = devAlloc(s, &s->prim1, (size_t)lfm::dev::primRows<float>(s->D) * nt))) return fail(rc);
        s->fluxUpdate = true;
    }
    // flux kernel variants: FP32-bulk M1 / M2 laminar cases with separate flux
    // and update kernels; the cell-centred one where the faces are stored by
    // owner (the description's order)
    s->fluxVariants = s->precision == LFM_FP32_BULK && !tiled && !s->fluxUpdate && !d->smag_c &&
                      lfm::dev::flux_staging_supported(s->scheme, false);
    if (s->fluxVariants) {
        bool byOwner = true;
        for (size_t f = 1; f < nf && byOwner; ++f) byOwner = fP[f] >= fP[f - 1];
        if (byOwner) {
            std::vector<int> own(nc + 1, 0);
            for (size_t f = 0; f < nf; ++f) ++own[(size_t)fP[f] + 1];
            for (size_t c = 0; c < nc; ++c) own[c + 1] += own[c];
            if ((rc = upload(s, &s->fOwnDev, own.data(), nc + 1))) return fail(rc);
            if (fluxCellOption(s)) s->a32.fOwn = s->fOwnDev;
        }
    }
    if (s->fluxVariants) {
        lfm::dev::FluxStaging fs = fluxStagingOption(s);
        if (fs.stages > 0) {
            if ((e = lfm::dev::configure_flux_staging(s->D, s->scheme, s->nf, fs)) != cudaSuccess)
                return fail(cudaFail(e, "configure_flux_staging"));
            s->fluxStaging = fs;
        }
    }
    if (s->precision == LFM_FP32_BULK) {
        for (int v = 0; v < s->nq; ++v) s->qRef[v] = s->a32.qRef[v];
        if ((rc = devAlloc(s, &s->stage, nq * nc))) return fail(rc);
    }
    if ((e = cudaHostAlloc(reinterpret_cast<void**>(&s->flagHost), sizeof(int), cudaHostAllocDefault)) != cudaSuccess)
        return fail(cudaFail(e, "cudaHostAlloc"));
    *s->flagHost = 0;
    if (d->q0) {
        if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) return fail(cudaFail(e, "create"));
        if ((rc = lfm_solver_set_state(s, d->q0))) return fail(rc);
    }
    if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) return fail(cudaFail(e, "create"));
    *out = s;
    return LFM_OK;
}

}  // namespace

extern "C" int lfm_solver_create(const lfm_solver_desc* d, const lfm_solver_opts* opts, lfm_solver** out) {
    return createSolver(d, opts, nullptr, out);
}

extern "C" void lfm_solver_destroy(lfm_solver* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    if (s->graphOdd) cudaGraphExecDestroy(s->graphOdd);
    if (s->advGraph) cudaGraphExecDestroy(s->advGraph);
    if (s->flagHost) cudaFreeHost(s->flagHost);
    for (void* p : s->allocations) cudaFree(p);
    if (s->scrub) cudaFree(s->scrub);
    if (s->dPatches) cudaFree(s->dPatches);
    if (s->dForces) cudaFree(s->dForces);
    if (s->probeCells) cudaFree(s->probeCells);
    if (s->probeHist) cudaFree(s->probeHist);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->stream && s->ownStream) cudaStreamDestroy(s->stream);
    delete s;
}

namespace {

// The state upload of lfm_solver_set_state, enqueued on the solver stream.
int enqueueSetState(lfm_solver* s, const double* q) {
    // a new state starts with a clear non-finite flag
    LFM_CUDA(cudaMemsetAsync(s->flag, 0, sizeof(int), s->stream));
    const size_t nc = (size_t)s->nc;
    if (s->precision == LFM_FP32_BULK) {   // stored as q - q_ref
        LFM_CUDA(cudaMemcpyAsync(s->stage, q, (size_t)s->nq * nc * sizeof(double), cudaMemcpyHostToDevice,
                                 s->stream));
        // q' with the cells' primitives (and the ghosts' the update keeps) in
        // one pass: the per-stage preparation covers the other ghosts and halos
        lfm::dev::launch_set_state32(s->a32, s->stage, s->nc, s->stream);
        LFM_CUDA(cudaGetLastError());
    } else {   // rows of nc values into rows of nt
        LFM_CUDA(cudaMemcpy2DAsync(s->q, (size_t)s->nt * sizeof(double), q, nc * sizeof(double),
                                   nc * sizeof(double), (size_t)s->nq, cudaMemcpyHostToDevice, s->stream));
    }
    s->primsValid = s->precision == LFM_FP32_BULK;   // FP64: rebuilt by ensurePrims
    s->primParity = 0;
    s->ghostRowsValid = false;
    return LFM_OK;
}

// The state download of lfm_solver_get_state, enqueued on the solver stream.
int enqueueGetState(lfm_solver* s, double* q) {
    if (s->precision == LFM_FP32_BULK) {   // stored as q - q_ref
        lfm::dev::QOffset qo;
        for (int v = 0; v < 5; ++v) qo.v[v] = s->qRef[v];
        lfm::dev::launch_offset_rows(s->stage, s->nc, s->q, s->nt, s->nc, s->nq, qo, 1.0, s->stream);
        LFM_CUDA(cudaGetLastError());
        LFM_CUDA(cudaMemcpyAsync(q, s->stage, (size_t)s->nq * s->nc * sizeof(double), cudaMemcpyDeviceToHost,
                                 s->stream));
    } else {
        LFM_CUDA(cudaMemcpy2DAsync(q, (size_t)s->nc * sizeof(double), s->q, (size_t)s->nt * sizeof(double),
                                   (size_t)s->nc * sizeof(double), (size_t)s->nq, cudaMemcpyDeviceToHost,
                                   s->stream));
    }
    return LFM_OK;
}

}  // namespace

extern "C" int lfm_solver_set_state(lfm_solver* s, const double* q) {
    if (!s || !q) return lfm::setError(LFM_ERR_INVALID, "null argument");
    LFM_CUDA(cudaSetDevice(s->device));
    int rc = enqueueSetState(s, q);
    if (rc) return rc;
    LFM_CUDA(cudaStreamSynchronize(s->stream));
    return LFM_OK;
}

extern "C" int lfm_solver_get_state(lfm_solver* s, double* q) {
    if (!s || !q) return lfm::setError(LFM_ERR_INVALID, "null argument");
    LFM_CUDA(cudaSetDevice(s->device));
    int rc = enqueueGetState(s, q);
    if (rc) return rc;
    LFM_CUDA(cudaStreamSynchronize(s->stream));
    return LFM_OK;
}

namespace {

bool pageLocked(const void* p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

// The whole advance between page-locked host states as one graph launch
// (device work only; the host-side state flags are set as the enqueued path
// leaves them). Captured once per (q_in, q_out, nsteps, dt).
int advanceGraph(lfm_solver* s, const double* qIn, int nsteps, double dt, double* qOut) {
    if (!(s->advGraph && s->advIn == qIn && s->advOut == qOut && s->advSteps == nsteps && s->advDt == dt)) {
        if (s->advGraph) cudaGraphExecDestroy(s->advGraph);
        s->advGraph = nullptr;
        cudaGraph_t g = nullptr;
        LFM_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueueSetState(s, qIn);
        if (!rc) rc = ensurePrims(s);
        // a new state starts in primitive buffer 0; alternating stages move
        // the current primitives to the other buffer after an odd stage count
        int parity = 0;
        for (int k = 0; k < nsteps && !rc; ++k) {
            launchStep(s, dt, parity);
            if (alternating(s)) parity ^= (s->rkOrder & 1);
        }
        if (!rc) rc = enqueueGetState(s, qOut);
        cudaError_t ce = cudaMemcpyAsync(s->flagHost, s->flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream);
        cudaError_t e = cudaStreamEndCapture(s->stream, &g);
        if (rc || ce != cudaSuccess || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return rc ? rc : cudaFail(ce != cudaSuccess ? ce : e, "advance capture");
        }
        e = cudaGraphInstantiate(&s->advGraph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cudaFail(e, "cudaGraphInstantiate");
        s->advIn = qIn;
        s->advOut = qOut;
        s->advSteps = nsteps;
        s->advDt = dt;
    }
    LFM_CUDA(cudaGraphLaunch(s->advGraph, s->stream));
    // the flags the enqueued path leaves: a new state, its primitives, stages run
    s->primParity = alternating(s) ? ((nsteps * s->rkOrder) & 1) : 0;
    s->primsValid = true;
    s->ghostRowsValid = true;
    s->lastStageB = s->rkB.empty() ? 0.0 : s->rkB.back();
    LFM_CUDA(cudaStreamSynchronize(s->stream));
    LFM_CUDA(cudaGetLastError());
    if (*s->flagHost) return lfm::setError(LFM_ERR_NUMERIC, "non-finite conserved state");
    return LFM_OK;
}

}  // namespace

extern "C" int lfm_solver_advance(lfm_solver* s, const double* q_in, int nsteps, double dt, double* q_out) {
    if (!s || nsteps < 0) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    LFM_CUDA(cudaSetDevice(s->device));
    int rc = LFM_OK;
    if (q_in && q_out && nsteps > 0 && s->rkOrder > 0 && pageLocked(q_in) && pageLocked(q_out))
        return advanceGraph(s, q_in, nsteps, dt, q_out);
    if (q_in && (rc = enqueueSetState(s, q_in))) return rc;
    if (nsteps > 0 && (rc = lfm_solver_step(s, nsteps, dt))) return rc;
    if (q_out && (rc = enqueueGetState(s, q_out))) return rc;
    return lfm_solver_sync(s);
}

extern "C" int lfm_solver_stage(lfm_solver* s, int rk, double dt) {
    if (!s) return lfm::setError(LFM_ERR_INVALID, "null solver");
    if (rk < 0 || rk >= s->rkOrder) return lfm::setError(LFM_ERR_INVALID, "stage index out of range");
    LFM_CUDA(cudaSetDevice(s->device));
    untile(s);
    int rc = ensurePrims(s);
    if (rc) return rc;
    s->lastStageB = s->rkB[(size_t)rk];
    const StageConfig c = stageConfig(s, rk, dt);
    if (s->precision == LFM_FP32_BULK)
        lfm::dev::launch_stage<float>(s->a32, c, s->stream);
    else
        lfm::dev::launch_stage<double>(s->a64, c, s->stream);
    LFM_CUDA(cudaGetLastError());
    return LFM_OK;
}

extern "C" int lfm_solver_step(lfm_solver* s, int nsteps, double dt) {
    if (!s || nsteps < 0) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    if (nsteps == 0) return LFM_OK;
    LFM_CUDA(cudaSetDevice(s->device));
    if (s->rkOrder == 0) {   // no stage: a time step only clears the residual (prepare_for_timestep)
        if (s->residuals) LFM_CUDA(cudaMemsetAsync(s->res, 0, sizeof(double) * (size_t)s->nq * s->nc, s->stream));
        return LFM_OK;
    }
    int rc = ensureGraph(s, dt);
    if (rc) return rc;
    if ((rc = ensurePrims(s))) return rc;
    for (int k = 0; k < nsteps; ++k) LFM_CUDA(launchStepGraph(s));
    return LFM_OK;
}

extern "C" int lfm_solver_step_timed(lfm_solver* s, int nsteps, double dt, float* ms) {
    if (!s || !ms) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    LFM_CUDA(cudaSetDevice(s->device));
    int rc = s->rkOrder > 0 ? ensureGraph(s, dt) : LFM_OK;
    if (rc) return rc;
    LFM_CUDA(cudaEventRecord(s->ev0, s->stream));
    rc = lfm_solver_step(s, nsteps, dt);
    if (rc) return rc;
    LFM_CUDA(cudaEventRecord(s->ev1, s->stream));
    LFM_CUDA(cudaEventSynchronize(s->ev1));
    LFM_CUDA(cudaEventElapsedTime(ms, s->ev0, s->ev1));
    return LFM_OK;
}

static int reduceScalar(lfm_solver* s, double dt, int mode, double maxCo, double* out) {
    LFM_CUDA(cudaSetDevice(s->device));
    lfm::dev::QOffset qo;
    for (int v = 0; v < 5; ++v) qo.v[v] = s->qRef[v];
    lfm::dev::launch_cfl(s->D, s->q, qo, s->nt, s->nc, s->volInv, s->sOff, s->cellS, dt, mode, maxCo, s->partial,
                         s->scalar, s->stream);
    LFM_CUDA(cudaGetLastError());
    LFM_CUDA(cudaMemcpyAsync(out, s->scalar, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    LFM_CUDA(cudaStreamSynchronize(s->stream));
    return LFM_OK;
}

extern "C" int lfm_solver_cfl(lfm_solver* s, double dt, double* cfl) {
    if (!s || !cfl) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    return reduceScalar(s, dt, 0, 0.0, cfl);
}

extern "C" int lfm_solver_min_dt(lfm_solver* s, double max_co, double* dt) {
    if (!s || !dt) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    return reduceScalar(s, 0.0, 1, max_co, dt);
}

extern "C" int lfm_solver_residual(lfm_solver* s, double* res) {
    if (!s || !res) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    if (!s->residuals) return lfm::setError(LFM_ERR_INVALID, "the case does not record residuals");
    LFM_CUDA(cudaSetDevice(s->device));
    for (int v = 0; v < s->nq; ++v)
        lfm::dev::launch_res_sum(s->res + (size_t)v * s->nc, s->nc, s->partial, s->scalar + v, s->stream);
    LFM_CUDA(cudaGetLastError());
    LFM_CUDA(cudaMemcpyAsync(res, s->scalar, sizeof(double) * (size_t)s->nq, cudaMemcpyDeviceToHost, s->stream));
    LFM_CUDA(cudaStreamSynchronize(s->stream));
    return LFM_OK;
}

extern "C" int lfm_solver_cell_residual(lfm_solver* s, double* res) {
    if (!s || !res) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    if (!s->residuals) return lfm::setError(LFM_ERR_INVALID, "the case does not record residuals");
    LFM_CUDA(cudaSetDevice(s->device));
    LFM_CUDA(cudaMemcpyAsync(res, s->res, sizeof(double) * (size_t)s->nq * (size_t)s->nc, cudaMemcpyDeviceToHost,
                             s->stream));
    LFM_CUDA(cudaStreamSynchronize(s->stream));
    return LFM_OK;
}

// ---------------------------------------------------------------------------
// Residual without allocation: scratch in a static device array.
// ---------------------------------------------------------------------------
namespace {

__device__ __align__(256) unsigned char g_noallocScratch[LFM_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_noallocMutex;
void* g_noallocAddr[kMaxDevices] = {};

// Device address of the scratch array on `device` (current), looked up once.
int noallocScratch(int device, unsigned char** out) {
    if (device < 0 || device >= kMaxDevices) return lfm::setError(LFM_ERR_UNSUPPORTED, "device ordinal too large");
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (!g_noallocAddr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess || !p) return cudaFail(e, "cudaGetSymbolAddress(g_noallocScratch)");
        g_noallocAddr[device] = p;
    }
    *out = static_cast<unsigned char*>(g_noallocAddr[device]);
    return LFM_OK;
}

template <typename T, int D>
__global__ void __launch_bounds__(256) k_gather_residual(const T* flux, int nf, int nc, const int* cfOff,
                                                         const int* cfList, double* res) {
    const int c = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (c >= nc) return;
    constexpr int NQ = D + 2;
    T sum[NQ];
#pragma unroll
    for (int v = 0; v < NQ; ++v) sum[v] = T(0);
    for (int e = cfOff[c]; e < cfOff[c + 1]; ++e) {
        const int code = cfList[e];
        if (code >= 0) {
#pragma unroll
            for (int v = 0; v < NQ; ++v) sum[v] += flux[(size_t)v * nf + code];
        } else {
#pragma unroll
            for (int v = 0; v < NQ; ++v) sum[v] -= flux[(size_t)v * nf + ~code];
        }
    }
#pragma unroll
    for (int v = 0; v < NQ; ++v) res[(size_t)v * nc + c] = (double)sum[v];
}

template <typename T>
int residualNoalloc(const lfm_solver* s, const Args<T>& base, const double* q, int64_t qStride, double* res,
                    cudaStream_t st) {
    const size_t nt = (size_t)s->nt, nf = (size_t)s->nf, D = (size_t)s->D, nq = (size_t)s->nq;
    const bool ausm = s->scheme == LFM_SOLVER_M2AUSM;
    auto round = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t bq = round(nq * nt * sizeof(double));
    const size_t bPrim = round((size_t)lfm::dev::primRows<T>(s->D) * nt * sizeof(T));
    const size_t bV = round((D * D + 2 * D + (base.smagC ? D * D : 0)) * nt * sizeof(T));
    const size_t bGrad = ausm ? round((2 * D + D * D) * nt * sizeof(T)) : 0;
    const size_t bFlux = round(nq * nf * sizeof(T));
    const size_t need = bq + bPrim + bV + bGrad + bFlux;
    if (need > LFM_NOALLOC_SCRATCH_BYTES)
        return lfm::setError(LFM_ERR_UNSUPPORTED, "the case needs " + std::to_string(need) +
                                                      " bytes of scratch; lfm_solver_residual_noalloc holds " +
                                                      std::to_string((size_t)LFM_NOALLOC_SCRATCH_BYTES));
    unsigned char* scratch = nullptr;
    int rc = noallocScratch(s->device, &scratch);
    if (rc) return rc;
    Args<T> a = base;
    a.q = reinterpret_cast<double*>(scratch);
    a.prim = reinterpret_cast<T*>(scratch + bq);
    a.primW = a.prim;
    a.V = reinterpret_cast<T*>(scratch + bq + bPrim);
    a.grad = ausm ? reinterpret_cast<T*>(scratch + bq + bPrim + bV) : base.grad;
    a.flux = reinterpret_cast<T*>(scratch + bq + bPrim + bV + bGrad);
    a.dq = nullptr;
    a.res = nullptr;
    // The array keeps the previous call's contents: the viscous terms and
    // gradients of the ghosts are read as zeros, so clear both blocks.
    LFM_CUDA(cudaMemsetAsync(a.V, 0, bV, st));
    if (ausm) LFM_CUDA(cudaMemsetAsync(a.grad, 0, bGrad, st));
    if constexpr (sizeof(T) == sizeof(float)) {
        // the FP32-bulk kernels read the state as q - q_ref
        lfm::dev::launch_to_perturbation(a, q, qStride, st);
    } else {
        // rows of nc values (stride q_stride) into rows of nt, one strided copy
        LFM_CUDA(cudaMemcpy2DAsync(a.q, nt * sizeof(double), q, (size_t)qStride * sizeof(double),
                                   (size_t)s->nc * sizeof(double), nq, cudaMemcpyDeviceToDevice, st));
    }
    StageConfig c;
    c.scheme = s->scheme;
    c.needGrad = s->needGrad;
    c.needVis = s->needVis;
    for (int k = 0; k < 4; ++k) lfm::dev::launch_kernel<T>(a, c, k, st);   // prep, grad, vis, flux
    const unsigned nb = (unsigned)((s->nc + 255) / 256);
    if (s->D == 2)
        k_gather_residual<T, 2><<<nb, 256, 0, st>>>(a.flux, s->nf, s->nc, a.cfOff, a.cfList, res);
    else
        k_gather_residual<T, 3><<<nb, 256, 0, st>>>(a.flux, s->nf, s->nc, a.cfOff, a.cfList, res);
    LFM_CUDA(cudaGetLastError());
    return LFM_OK;
}

}  // namespace

extern "C" int lfm_solver_residual_noalloc(const lfm_solver* s, const double* q, int64_t q_stride, double* res,
                                           void* stream) {
    if (!s || !q || !res) return lfm::setError(LFM_ERR_INVALID, "lfm_solver_residual_noalloc: null argument");
    if (q_stride < s->nc) return lfm::setError(LFM_ERR_INVALID, "q_stride is smaller than the cell count");
    // A partition of a decomposed case reads processor-face halo states that
    // its partitioned solver copies in before each stage; a caller's state
    // here covers the partition's own cells only, so those rows would be stale
    // (or zero) in the scratch array.
    if (s->nh > 0)
        return lfm::setError(LFM_ERR_UNSUPPORTED,
                             "lfm_solver_residual_noalloc: partitions with processor-face halos are not supported");
    LFM_CUDA(cudaSetDevice(s->device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (s->precision == LFM_FP32_BULK) return residualNoalloc<float>(s, s->a32, q, q_stride, res, st);
    return residualNoalloc<double>(s, s->a64, q, q_stride, res, st);
}

// ---------------------------------------------------------------------------
// Post-processing (post_kernels.cu).
// ---------------------------------------------------------------------------
namespace {

lfm::dev::QOffset stateOffset(const lfm_solver* s) {
    lfm::dev::QOffset qo;
    for (int v = 0; v < 5; ++v) qo.v[v] = s->precision == LFM_FP32_BULK ? s->qRef[v] : 0.0;
    return qo;
}

double gammaMinusOne(const lfm_solver* s) { return s->precision == LFM_FP32_BULK ? s->a32.gm1 : s->a64.gm1; }
double pInfOf(const lfm_solver* s) { return s->precision == LFM_FP32_BULK ? s->a32.pInf : s->a64.pInf; }

}  // namespace

extern "C" int lfm_solver_stats_reset(lfm_solver* s) {
    if (!s) return lfm::setError(LFM_ERR_INVALID, "null solver");
    LFM_CUDA(cudaSetDevice(s->device));
    int rc;
    if (!s->statAvg && ((rc = devAlloc(s, &s->statAvg, (size_t)s->nc)) || (rc = devAlloc(s, &s->statRms, (size_t)s->nc))))
        return rc;
    LFM_CUDA(cudaMemsetAsync(s->statAvg, 0, (size_t)s->nc * sizeof(double), s->stream));
    LFM_CUDA(cudaMemsetAsync(s->statRms, 0, (size_t)s->nc * sizeof(double), s->stream));
    return LFM_OK;
}

extern "C" int lfm_solver_stats_accumulate(lfm_solver* s, int n) {
    if (!s) return lfm::setError(LFM_ERR_INVALID, "null solver");
    if (!s->statAvg) return lfm::setError(LFM_ERR_INVALID, "lfm_solver_stats_reset was not called");
    if (n < 1) return LFM_OK;
    LFM_CUDA(cudaSetDevice(s->device));
    lfm::dev::launch_stats(s->D, s->q, s->nt, stateOffset(s), s->nc, gammaMinusOne(s), n, s->statAvg, s->statRms,
                           s->stream);
    LFM_CUDA(cudaGetLastError());
    return LFM_OK;
}

extern "C" int lfm_solver_stats_get(lfm_solver* s, int n, double* p_avg, double* p_rms) {
    if (!s || !p_avg || !p_rms || n < 1) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    if (!s->statAvg) return lfm::setError(LFM_ERR_INVALID, "lfm_solver_stats_reset was not called");
    LFM_CUDA(cudaSetDevice(s->device));
    const size_t nc = (size_t)s->nc;
    LFM_CUDA(cudaMemcpyAsync(p_avg, s->statAvg, nc * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    LFM_CUDA(cudaMemcpyAsync(p_rms, s->statRms, nc * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    LFM_CUDA(cudaStreamSynchronize(s->stream));
    // updateAverageField: factor 1/n, square root of the RMS sum
    // (updateScalarField / updateScalarFieldSqrt of the mesh reader)
    const double f = 1.0 / n;
    for (size_t c = 0; c < nc; ++c) {
        p_avg[c] = p_avg[c] * f;
        p_rms[c] = std::sqrt(p_rms[c] * f);
    }
    return LFM_OK;
}

extern "C" int lfm_solver_forces(lfm_solver* s, int n_patches, const int32_t* patches, double* f_pressure,
                                 double* f_viscous) {
    if (!s || n_patches < 0 || (n_patches > 0 && (!patches || !f_pressure || !f_viscous)))
        return lfm::setError(LFM_ERR_INVALID, "bad argument");
    if (!s->gPatch && s->ng > 0)
        return lfm::setError(LFM_ERR_INVALID, "the solver description has no ghost_patch: forces unavailable");
    if (n_patches == 0) return LFM_OK;
    LFM_CUDA(cudaSetDevice(s->device));
    int rc;
    if (!s->forceTerms && s->ng > 0 &&
        (rc = devAlloc(s, &s->forceTerms, (size_t)(s->D + s->D * s->D) * (size_t)s->ng)))
        return rc;
    if (n_patches > s->patchCap) {
        if (s->dPatches) cudaFree(s->dPatches);
        if (s->dForces) cudaFree(s->dForces);
        s->dPatches = nullptr;
        s->dForces = nullptr;
        s->patchCap = 0;
        LFM_CUDA(cudaMalloc(&s->dPatches, (size_t)n_patches * sizeof(int)));
        LFM_CUDA(cudaMalloc(&s->dForces, 2 * (size_t)n_patches * (size_t)s->D * sizeof(double)));
        s->patchCap = n_patches;
    }
    const size_t nv = (size_t)n_patches * (size_t)s->D;
    std::vector<int> pl(patches, patches + n_patches);
    LFM_CUDA(cudaMemcpyAsync(s->dPatches, pl.data(), pl.size() * sizeof(int), cudaMemcpyHostToDevice, s->stream));
    LFM_CUDA(cudaMemsetAsync(s->dForces, 0, 2 * nv * sizeof(double), s->stream));
    // ghost states of the last stage's start, as the reference's ghost cells
    // hold after a step: recovered from the last update (the update writes the
    // ghosts of the next stage's state); the current state's before any stage
    const int mode = !s->ghostRowsValid ? lfm::dev::kGhostFresh : lfm::dev::kGhostUndo;
    if (s->precision == LFM_FP32_BULK)
        lfm::dev::launch_forces<float>(s->a32, stateOffset(s), s->gS, s->gD, s->gPatch, mode, s->lastStageB,
                                       s->dPatches, n_patches, s->forceTerms, s->dForces, s->dForces + nv, s->stream);
    else
        lfm::dev::launch_forces<double>(s->a64, stateOffset(s), s->gS, s->gD, s->gPatch, mode, s->lastStageB,
                                        s->dPatches, n_patches, s->forceTerms, s->dForces, s->dForces + nv,
                                        s->stream);
    LFM_CUDA(cudaGetLastError());
    LFM_CUDA(cudaMemcpyAsync(f_pressure, s->dForces, nv * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    LFM_CUDA(cudaMemcpyAsync(f_viscous, s->dForces + nv, nv * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    LFM_CUDA(cudaStreamSynchronize(s->stream));
    return LFM_OK;
}

extern "C" int lfm_solver_probes_set(lfm_solver* s, int n, const int64_t* cells, int capacity) {
    if (!s || n < 0 || capacity < 0 || (n > 0 && !cells)) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    for (int i = 0; i < n; ++i)
        if (cells[i] < 0 || cells[i] >= s->nc) return lfm::setError(LFM_ERR_INVALID, "probe cell out of range");
    LFM_CUDA(cudaSetDevice(s->device));
    LFM_CUDA(cudaStreamSynchronize(s->stream));
    if (s->probeCells) cudaFree(s->probeCells);
    if (s->probeHist) cudaFree(s->probeHist);
    s->probeCells = nullptr;
    s->probeHist = nullptr;
    s->nProbes = s->probeCap = s->probeRecords = 0;
    if (n == 0) return LFM_OK;
    std::vector<int> c32(cells, cells + n);
    LFM_CUDA(cudaMalloc(&s->probeCells, (size_t)n * sizeof(int)));
    LFM_CUDA(cudaMalloc(&s->probeHist, (size_t)n * (size_t)std::max(capacity, 1) * sizeof(double)));
    LFM_CUDA(cudaMemcpy(s->probeCells, c32.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice));
    s->nProbes = n;
    s->probeCap = capacity;
    return LFM_OK;
}

extern "C" int lfm_solver_probes_record(lfm_solver* s) {
    if (!s) return lfm::setError(LFM_ERR_INVALID, "null solver");
    if (s->nProbes == 0) return lfm::setError(LFM_ERR_INVALID, "no probes set");
    if (s->probeRecords >= s->probeCap) return lfm::setError(LFM_ERR_NOMEM, "probe history is full");
    LFM_CUDA(cudaSetDevice(s->device));
    lfm::dev::launch_probe(s->D, s->q, s->nt, stateOffset(s), s->probeCells, s->nProbes, gammaMinusOne(s), pInfOf(s),
                           s->probeHist + (size_t)s->probeRecords * (size_t)s->nProbes, s->stream);
    LFM_CUDA(cudaGetLastError());
    ++s->probeRecords;
    return LFM_OK;
}

extern "C" int lfm_solver_probes_read(lfm_solver* s, double* out, int* n_records) {
    if (!s || !n_records) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    LFM_CUDA(cudaSetDevice(s->device));
    *n_records = s->probeRecords;
    if (s->probeRecords > 0) {
        if (!out) return lfm::setError(LFM_ERR_INVALID, "null output");
        LFM_CUDA(cudaMemcpyAsync(out, s->probeHist, (size_t)s->probeRecords * (size_t)s->nProbes * sizeof(double),
                                 cudaMemcpyDeviceToHost, s->stream));
    }
    LFM_CUDA(cudaStreamSynchronize(s->stream));
    return LFM_OK;
}

extern "C" int lfm_solver_sync(lfm_solver* s) {
    if (!s) return lfm::setError(LFM_ERR_INVALID, "null solver");
    LFM_CUDA(cudaSetDevice(s->device));
    LFM_CUDA(cudaMemcpyAsync(s->flagHost, s->flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    LFM_CUDA(cudaStreamSynchronize(s->stream));
    LFM_CUDA(cudaGetLastError());
    if (*s->flagHost) return lfm::setError(LFM_ERR_NUMERIC, "non-finite conserved state");
    return LFM_OK;
}

extern "C" int lfm_solver_flush_l2(lfm_solver* s, size_t bytes) {
    if (!s) return lfm::setError(LFM_ERR_INVALID, "null solver");
    LFM_CUDA(cudaSetDevice(s->device));
    if (bytes > s->scrubBytes) {
        if (s->scrub) cudaFree(s->scrub);
        s->scrub = nullptr;
        s->scrubBytes = 0;
        LFM_CUDA(cudaMalloc(&s->scrub, bytes));
        s->scrubBytes = bytes;
    }
    LFM_CUDA(cudaMemsetAsync(s->scrub, 0x5a, bytes, s->stream));
    return LFM_OK;
}

extern "C" int lfm_solver_bench(lfm_solver* s, int nsteps, double dt, size_t flush_bytes, float* ms) {
    if (!s || !ms || nsteps <= 0) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    LFM_CUDA(cudaSetDevice(s->device));
    int rc = ensureGraph(s, dt);
    if (rc) return rc;
    if ((rc = ensurePrims(s))) return rc;
    if (flush_bytes > s->scrubBytes) {
        if (s->scrub) cudaFree(s->scrub);
        s->scrub = nullptr;
        s->scrubBytes = 0;
        LFM_CUDA(cudaMalloc(&s->scrub, flush_bytes));
        s->scrubBytes = flush_bytes;
    }
    std::vector<cudaEvent_t> ev(2 * (size_t)nsteps);
    for (auto& x : ev) LFM_CUDA(cudaEventCreate(&x));
    for (int k = 0; k < nsteps; ++k) {
        if (flush_bytes) LFM_CUDA(cudaMemsetAsync(s->scrub, 0x5a + (k & 1), flush_bytes, s->stream));
        LFM_CUDA(cudaEventRecord(ev[2 * (size_t)k], s->stream));
        LFM_CUDA(launchStepGraph(s));
        LFM_CUDA(cudaEventRecord(ev[2 * (size_t)k + 1], s->stream));
    }
    LFM_CUDA(cudaStreamSynchronize(s->stream));
    for (int k = 0; k < nsteps; ++k) LFM_CUDA(cudaEventElapsedTime(&ms[k], ev[2 * (size_t)k], ev[2 * (size_t)k + 1]));
    for (auto& x : ev) cudaEventDestroy(x);
    return LFM_OK;
}

extern "C" int lfm_solver_launches_per_step(const lfm_solver* s, int* launches) {
    if (!s || !launches) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    // preparation: the update writes the cells' and (cellGhosts) the ghosts'
    // primitives, so only halos remain
    const bool fused = s->precision == LFM_FP32_BULK ? s->a32.cellGhosts != nullptr : s->a64.cellGhosts != nullptr;
    const bool prep = !fused || s->nh > 0;
    *launches = s->tiled ? s->rkOrder
                         : s->rkOrder * ((prep ? 1 : 0) + (s->fluxUpdate ? 1 : 2) + (s->needGrad ? 1 : 0) +
                                         (s->needVis ? 1 : 0));
    return LFM_OK;
}

extern "C" const char* lfm_solver_kernel_name(int i) { return lfm::dev::kernelName(i); }

// Per-kernel times of a time step, by prefix differences: the step's kernel
// launches in order are L1..LM; for every m the graph of L1..Lm runs a few
// times, each after the L2 scrub of the benchmark loop (when one exists),
// timed with events on the stream around the graph launch, and T(m) is the
// median. Launch Lm is charged T(m) - T(m-1) (T(0): the empty event pair),
// so each kernel is timed where it runs in the step - after the same
// kernels, with the L2 contents they leave - and the charges add up to the
// step's own time T(M). With tile stages the whole stage is one kernel and
// the step's time goes to slot kKernelsPerStage ("k_tile_stage").
namespace {

struct Launch {
    int stage, slot;
};

// Median over reps of the time of `body` enqueued after an L2 scrub.
template <typename F>
cudaError_t medianTime(lfm_solver* s, int reps, cudaEvent_t e0, cudaEvent_t e1, F body, float* out) {
    std::vector<float> t;
    cudaError_t e = cudaSuccess;
    for (int r = 0; r < reps && e == cudaSuccess; ++r) {
        if (s->scrub) e = cudaMemsetAsync(s->scrub, 0x5a + (r & 1), s->scrubBytes, s->stream);
        if (e == cudaSuccess) e = cudaEventRecord(e0, s->stream);
        if (e == cudaSuccess) e = body();
        if (e == cudaSuccess) e = cudaEventRecord(e1, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        t.push_back(ms);
    }
    if (e != cudaSuccess) return e;
    std::sort(t.begin(), t.end());
    *out = t[t.size() / 2];
    return cudaSuccess;
}

void launchOne(lfm_solver* s, const Launch& l, double dt) {
    const StageConfig c = stageConfig(s, l.stage, dt);
    if (s->fluxUpdate) {   // buffers of a step that starts from buffer 0
        float* buf[2] = {s->a32.prim, s->prim1};
        Args<float> g = s->a32;
        g.prim = buf[l.stage & 1];
        g.primW = buf[(l.stage & 1) ^ 1];
        if (l.slot == lfm::dev::kSlotFluxUpdate) lfm::dev::launch_fluxupdate32(g, c, s->stream);
        else if (l.slot < 3) lfm::dev::launch_kernel<float>(g, c, l.slot, s->stream);
        return;
    }
    if (s->precision == LFM_FP32_BULK)
        lfm::dev::launch_kernel<float>(s->a32, c, l.slot, s->stream);
    else
        lfm::dev::launch_kernel<double>(s->a64, c, l.slot, s->stream);
}

// Graph of the launches [0, m) of `seq` (nullptr when m == 0).
cudaError_t prefixGraph(lfm_solver* s, const std::vector<Launch>& seq, size_t m, double dt, cudaGraphExec_t* out) {
    *out = nullptr;
    if (m == 0) return cudaSuccess;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    for (size_t k = 0; k < m; ++k) launchOne(s, seq[k], dt);
    e = cudaStreamEndCapture(s->stream, &g);
    if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
    if (g) cudaGraphDestroy(g);
    return e;
}

}  // namespace

extern "C" int lfm_solver_profile_step(lfm_solver* s, double dt, int n, float* ms) {
    if (!s || !ms || n < lfm::dev::kKernelSlots) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    LFM_CUDA(cudaSetDevice(s->device));
    for (int k = 0; k < n; ++k) ms[k] = 0.f;
    if (s->rkOrder == 0) return LFM_OK;   // no stage, no kernel
    int rc = ensurePrims(s);
    if (rc) return rc;
    constexpr int kReps = 7;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    LFM_CUDA(cudaEventCreate(&e0));
    LFM_CUDA(cudaEventCreate(&e1));
    cudaError_t e = cudaSuccess;
    float t0 = 0.f;
    e = medianTime(s, kReps, e0, e1, [] { return cudaSuccess; }, &t0);
    if (s->tiled) {
        // whole steps (the primitive buffers alternate between the stages)
        if (e == cudaSuccess && !(rc = ensureGraph(s, dt))) {
            float t = 0.f;
            e = medianTime(s, kReps, e0, e1, [s] { return launchStepGraph(s); }, &t);
            ms[lfm::dev::kSlotTileStage] = std::max(0.f, t - t0);
        }
    } else if (e == cudaSuccess) {
        // the launches of one step: a (stage, slot) pair counts when its
        // capture holds a kernel
        std::vector<Launch> seq;
        std::vector<int> slots;
        for (int w = 0; w < lfm::dev::kKernelsPerStage; ++w)
            if (!s->fluxUpdate || w < 3) slots.push_back(w);
        if (s->fluxUpdate) slots.push_back(lfm::dev::kSlotFluxUpdate);
        for (int k = 0; k < s->rkOrder && e == cudaSuccess; ++k)
            for (int w : slots) {
                if (e != cudaSuccess) break;
                cudaGraph_t g = nullptr;
                e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
                if (e != cudaSuccess) break;
                launchOne(s, Launch{k, w}, dt);
                e = cudaStreamEndCapture(s->stream, &g);
                size_t nodes = 0;
                if (e == cudaSuccess) e = cudaGraphGetNodes(g, nullptr, &nodes);
                if (g) cudaGraphDestroy(g);
                if (e == cudaSuccess && nodes > 0) seq.push_back(Launch{k, w});
            }
        float prev = t0;
        for (size_t m = 1; m <= seq.size() && e == cudaSuccess; ++m) {
            cudaGraphExec_t ge = nullptr;
            e = prefixGraph(s, seq, m, dt, &ge);
            float t = 0.f;
            if (e == cudaSuccess) e = medianTime(s, kReps, e0, e1, [s, ge] { return cudaGraphLaunch(ge, s->stream); }, &t);
            if (ge) cudaGraphExecDestroy(ge);
            ms[seq[m - 1].slot] += t - prev;
            prev = t;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (alternating(s)) {   // partial steps leave the primitives in either buffer
        s->primsValid = false;
        s->primParity = 0;
    }
    if (rc) return rc;
    if (e != cudaSuccess) return cudaFail(e, "profile step");
    return LFM_OK;
}

// ---------------------------------------------------------------------------
// Decomposed cases: every partition on the same GPU (lfm_partitioned_*).
//
// The reference runs one partition per MPI rank and exchanges halo cells
// after each stage's update (conserved state) and after calc_VIS (viscous
// terms) (src/mesh_solver.cpp:500-672). Here every partition is a solver on
// one shared stream, and the exchange is a gather kernel per partition that
// copies the source cells into the halo slots: state before each stage's
// preparation, viscous terms between the viscous pass and the fluxes.
// Gradients are not exchanged (the reference exchanges none: its halos'
// gradients stay zero, and M2AUSM with minmod reads zero gradients there).
// ---------------------------------------------------------------------------
struct lfm_partitioned {
    int device = 0;
    int precision = LFM_FP64;
    cudaStream_t stream = nullptr;
    std::vector<lfm_solver*> parts;
    std::vector<int*> haloPart, haloCell;   // device lists per partition
    double** dQ = nullptr;                  // per-partition state base pointers
    void** dV = nullptr;                    // per-partition viscous-term base pointers
    int* dNt = nullptr;                     // per-partition row strides
    cudaGraphExec_t graph = nullptr;
    double graphDt = 0;
};

namespace {

template <typename T>
void partitionedStages(lfm_partitioned* P, double dt) {
    const size_t np = P->parts.size();
    auto args = [&](size_t p) -> const Args<T>& {
        if constexpr (sizeof(T) == sizeof(float)) return P->parts[p]->a32;
        else return P->parts[p]->a64;
    };
    lfm_solver* s0 = P->parts[0];
    for (int k = 0; k < s0->rkOrder; ++k) {
        const StageConfig c = stageConfig(s0, k, dt);
        for (size_t p = 0; p < np; ++p) {
            const lfm_solver* s = P->parts[p];
            lfm::dev::launch_halo_gather<double>(s->q, s->nt, s->nc + s->ng, s->nq, s->nh, P->haloPart[p],
                                                 P->haloCell[p], P->dQ, P->dNt, P->stream);
        }
        for (int w = 0; w < 3; ++w)   // preparation, gradients, viscous terms
            for (size_t p = 0; p < np; ++p) lfm::dev::launch_kernel<T>(args(p), c, w, P->stream);
        if (s0->needVis)
            for (size_t p = 0; p < np; ++p) {
                const lfm_solver* s = P->parts[p];
                const int rows = s->D * s->D + 2 * s->D + (args(p).smagC ? s->D * s->D : 0);
                lfm::dev::launch_halo_gather<T>(args(p).V, s->nt, s->nc + s->ng, rows, s->nh, P->haloPart[p],
                                                P->haloCell[p], reinterpret_cast<T* const*>(P->dV), P->dNt,
                                                P->stream);
            }
        for (int w = 3; w < 5; ++w)   // fluxes, update
            for (size_t p = 0; p < np; ++p) lfm::dev::launch_kernel<T>(args(p), c, w, P->stream);
    }
}

int partitionedGraph(lfm_partitioned* P, double dt) {
    if (P->graph && P->graphDt == dt) return LFM_OK;
    if (P->graph) {
        cudaGraphExecDestroy(P->graph);
        P->graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    LFM_CUDA(cudaStreamBeginCapture(P->stream, cudaStreamCaptureModeThreadLocal));
    if (P->precision == LFM_FP32_BULK)
        partitionedStages<float>(P, dt);
    else
        partitionedStages<double>(P, dt);
    cudaError_t e = cudaStreamEndCapture(P->stream, &g);
    if (e != cudaSuccess) return cudaFail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&P->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cudaFail(e, "cudaGraphInstantiate");
    P->graphDt = dt;
    return LFM_OK;
}

int checkPart(const lfm_partitioned* P, int part) {
    if (!P) return lfm::setError(LFM_ERR_INVALID, "null partitioned solver");
    if (part < 0 || part >= (int)P->parts.size())
        return lfm::setError(LFM_ERR_INVALID, "no partition " + std::to_string(part));
    return LFM_OK;
}

}  // namespace

extern "C" void lfm_partitioned_destroy(lfm_partitioned* P) {
    if (!P) return;
    cudaSetDevice(P->device);
    if (P->stream) cudaStreamSynchronize(P->stream);
    if (P->graph) cudaGraphExecDestroy(P->graph);
    for (lfm_solver* s : P->parts) lfm_solver_destroy(s);
    for (int* p : P->haloPart) cudaFree(p);
    for (int* p : P->haloCell) cudaFree(p);
    cudaFree(P->dQ);
    cudaFree(P->dV);
    cudaFree(P->dNt);
    if (P->stream) cudaStreamDestroy(P->stream);
    delete P;
}

extern "C" int lfm_partitioned_create(const lfm_solver_desc* const* descs, int nparts, const lfm_solver_opts* opts,
                                      lfm_partitioned** out) {
    if (!descs || !out || nparts < 1) return lfm::setError(LFM_ERR_INVALID, "lfm_partitioned_create: bad argument");
    *out = nullptr;
    for (int p = 0; p < nparts; ++p) {
        int rc = lfm::setup::validateDesc(descs[p]);
        if (rc) return rc;
        const lfm_solver_desc* d = descs[p];
        const lfm_solver_desc* d0 = descs[0];
        if (d->dim != d0->dim || d->solver != d0->solver || d->rk_order != d0->rk_order || d->mu != d0->mu ||
            d->minmod != d0->minmod)
            return lfm::setError(LFM_ERR_INVALID, "partitions of one case must share dim, scheme, rk_order and mu");
        for (int64_t h = 0; h < d->n_halos; ++h) {
            const int64_t q = d->halo_src_part[h];
            if (q < 0 || q >= nparts || d->halo_src_cell[h] < 0 || d->halo_src_cell[h] >= descs[q]->n_cells)
                return lfm::setError(LFM_ERR_INVALID, "halo " + std::to_string(h) + " of partition " +
                                                          std::to_string(p) + " has no valid source cell");
        }
    }
    lfm_partitioned* P = new lfm_partitioned;
    P->device = opts ? opts->device : 0;
    P->precision = opts ? opts->precision : LFM_FP64;
    auto fail = [&](int rc) {
        lfm_partitioned_destroy(P);
        return rc;
    };
    cudaError_t e = cudaSetDevice(P->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(cudaFail(e, "partitioned stream"));
    for (int p = 0; p < nparts; ++p) {
        lfm_solver* s = nullptr;
        int rc = createSolver(descs[p], opts, P->stream, &s);
        if (rc) return fail(rc);
        P->parts.push_back(s);
        std::vector<int> hp((size_t)s->nh), hc((size_t)s->nh);
        for (int h = 0; h < s->nh; ++h) {
            hp[(size_t)h] = (int)descs[p]->halo_src_part[h];
            hc[(size_t)h] = (int)descs[p]->halo_src_cell[h];
        }
        int *dp = nullptr, *dc = nullptr;
        const size_t n = std::max<size_t>(1, hp.size());
        if ((e = cudaMalloc(&dp, n * sizeof(int))) != cudaSuccess || (e = cudaMalloc(&dc, n * sizeof(int))) != cudaSuccess)
            return fail(cudaFail(e, "halo lists"));
        P->haloPart.push_back(dp);
        P->haloCell.push_back(dc);
        if (!hp.empty() &&
            ((e = cudaMemcpy(dp, hp.data(), hp.size() * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess ||
             (e = cudaMemcpy(dc, hc.data(), hc.size() * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess))
            return fail(cudaFail(e, "halo lists"));
    }
    std::vector<double*> q((size_t)nparts);
    std::vector<void*> v((size_t)nparts);
    std::vector<int> nt((size_t)nparts);
    for (int p = 0; p < nparts; ++p) {
        const lfm_solver* s = P->parts[(size_t)p];
        q[(size_t)p] = s->q;
        v[(size_t)p] = P->precision == LFM_FP32_BULK ? (void*)s->a32.V : (void*)s->a64.V;
        nt[(size_t)p] = s->nt;
    }
    if ((e = cudaMalloc(&P->dQ, nparts * sizeof(double*))) != cudaSuccess ||
        (e = cudaMalloc(&P->dV, nparts * sizeof(void*))) != cudaSuccess ||
        (e = cudaMalloc(&P->dNt, nparts * sizeof(int))) != cudaSuccess ||
        (e = cudaMemcpy(P->dQ, q.data(), nparts * sizeof(double*), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(P->dV, v.data(), nparts * sizeof(void*), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(P->dNt, nt.data(), nparts * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(cudaFail(e, "partition tables"));
    *out = P;
    return LFM_OK;
}

extern "C" int lfm_partitioned_set_state(lfm_partitioned* P, int part, const double* q) {
    int rc = checkPart(P, part);
    return rc ? rc : lfm_solver_set_state(P->parts[(size_t)part], q);
}

extern "C" int lfm_partitioned_get_state(lfm_partitioned* P, int part, double* q) {
    int rc = checkPart(P, part);
    return rc ? rc : lfm_solver_get_state(P->parts[(size_t)part], q);
}

extern "C" int lfm_partitioned_step(lfm_partitioned* P, int nsteps, double dt) {
    if (!P || nsteps < 0) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    if (nsteps == 0) return LFM_OK;
    LFM_CUDA(cudaSetDevice(P->device));
    int rc = partitionedGraph(P, dt);
    if (rc) return rc;
    for (lfm_solver* s : P->parts)
        if ((rc = ensurePrims(s))) return rc;
    for (int k = 0; k < nsteps; ++k) LFM_CUDA(cudaGraphLaunch(P->graph, P->stream));
    return LFM_OK;
}

extern "C" int lfm_partitioned_solver(lfm_partitioned* P, int part, lfm_solver** out) {
    int rc = checkPart(P, part);
    if (rc) return rc;
    if (!out) return lfm::setError(LFM_ERR_INVALID, "null output handle");
    *out = P->parts[(size_t)part];
    return LFM_OK;
}

extern "C" int lfm_partitioned_sync(lfm_partitioned* P) {
    if (!P) return lfm::setError(LFM_ERR_INVALID, "null partitioned solver");
    for (lfm_solver* s : P->parts) {
        int rc = lfm_solver_sync(s);
        if (rc) return rc;
    }
    return LFM_OK;
}

// ---------------------------------------------------------------------------
// Flux kernel tuning (FP32-bulk): the face-per-thread kernel, the cell-centred
// kernel and the staged kernels at each staging depth give the same bits;
// lfm_solver_autotune times them on the solver's own case and keeps the
// fastest.
// ---------------------------------------------------------------------------
namespace {

void dropGraphs(lfm_solver* s) {
    if (s->graph) cudaGraphExecDestroy(s->graph);
    if (s->graphOdd) cudaGraphExecDestroy(s->graphOdd);
    if (s->advGraph) cudaGraphExecDestroy(s->advGraph);
    s->graph = s->graphOdd = s->advGraph = nullptr;
    s->graphDt = 0;
    s->advIn = nullptr;
    s->advOut = nullptr;
}

lfm_solver_tuning currentTuning(const lfm_solver* s) {
    lfm_solver_tuning t{};
    if (s->fluxStaging.stages > 0) {
        t.flux_kernel = LFM_FLUX_STAGED;
        t.staging_depth = s->fluxStaging.stages;
        t.staging_faces = s->fluxStaging.faces;
    } else {
        t.flux_kernel = s->a32.fOwn ? LFM_FLUX_CELL : LFM_FLUX_FACE;
    }
    t.ms_per_step = 0.0f;
    return t;
}

int applyTuning(lfm_solver* s, const lfm_solver_tuning& t) {
    if (t.flux_kernel == LFM_FLUX_FACE || t.flux_kernel == LFM_FLUX_CELL) {
        if (t.flux_kernel == LFM_FLUX_CELL && !s->fOwnDev)
            return lfm::setError(LFM_ERR_UNSUPPORTED, "cell-centred flux: faces not stored by owner");
        s->a32.fOwn = t.flux_kernel == LFM_FLUX_CELL ? s->fOwnDev : nullptr;
        s->fluxStaging = lfm::dev::FluxStaging{};
    } else if (t.flux_kernel == LFM_FLUX_STAGED) {
        lfm::dev::FluxStaging fs;
        fs.stages = t.staging_depth;
        fs.faces = t.staging_faces;
        if (fs.stages < 1 || fs.stages > 4) return lfm::setError(LFM_ERR_INVALID, "staging depth must be 1..4");
        const cudaError_t e = lfm::dev::configure_flux_staging(s->D, s->scheme, s->nf, fs);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return lfm::setError(LFM_ERR_INVALID, std::string("staged flux configuration refused: ") +
                                                      cudaGetErrorString(e));
        }
        s->fluxStaging = fs;
        s->a32.fOwn = nullptr;
    } else {
        return lfm::setError(LFM_ERR_INVALID, "unknown flux kernel");
    }
    dropGraphs(s);
    return LFM_OK;
}

}  // namespace

extern "C" int lfm_solver_get_tuning(const lfm_solver* s, lfm_solver_tuning* t) {
    if (!s || !t) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    *t = currentTuning(s);
    return LFM_OK;
}

extern "C" int lfm_solver_set_tuning(lfm_solver* s, const lfm_solver_tuning* t) {
    if (!s || !t) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    if (!s->fluxVariants) {
        if (t->flux_kernel == LFM_FLUX_FACE) return LFM_OK;
        return lfm::setError(LFM_ERR_UNSUPPORTED, "flux kernel variants: FP32-bulk M1 / M2 laminar solvers with "
                                                  "separate flux and update kernels only");
    }
    LFM_CUDA(cudaSetDevice(s->device));
    LFM_CUDA(cudaStreamSynchronize(s->stream));
    return applyTuning(s, *t);
}

extern "C" int lfm_solver_autotune(lfm_solver* s, double dt, int trial_steps, size_t flush_bytes,
                                   lfm_solver_tuning* chosen, lfm_solver_tuning* tried, int capacity,
                                   int* n_tried) {
    if (!s || trial_steps <= 0 || !(dt > 0) || capacity < 0) return lfm::setError(LFM_ERR_INVALID, "bad argument");
    if (n_tried) *n_tried = 0;
    LFM_CUDA(cudaSetDevice(s->device));
    std::vector<lfm_solver_tuning> cand;
    cand.push_back(currentTuning(s));
    if (s->fluxVariants) {
        cand.clear();
        cand.push_back(lfm_solver_tuning{LFM_FLUX_FACE, 0, 0, 0.0f});
        if (s->fOwnDev) cand.push_back(lfm_solver_tuning{LFM_FLUX_CELL, 0, 0, 0.0f});
        cand.push_back(lfm_solver_tuning{LFM_FLUX_STAGED, 1, 256, 0.0f});
        const int shapes[][2] = {{2, 64}, {2, 128}, {2, 256}, {3, 64}, {3, 128}, {4, 64}};
        for (const auto& sh : shapes) cand.push_back(lfm_solver_tuning{LFM_FLUX_STAGED, sh[0], sh[1], 0.0f});
    }
    const lfm_solver_tuning before = currentTuning(s);
    // the stored state and primitives, copied on the device (the FP32-bulk
    // state is q - q_ref: a round trip through the absolute state would not
    // keep its bits)
    LFM_CUDA(cudaStreamSynchronize(s->stream));
    int rc = ensurePrims(s);
    if (rc) return rc;
    const size_t qBytes = (size_t)s->nq * (size_t)s->nt * sizeof(double);
    const size_t pBytes = s->precision == LFM_FP32_BULK
                              ? (size_t)lfm::dev::primRows<float>(s->D) * (size_t)s->nt * sizeof(float) : 0;
    void* saved = nullptr;
    LFM_CUDA(cudaMalloc(&saved, qBytes + pBytes));
    char* sq = static_cast<char*>(saved);
    auto restore = [&]() -> int {
        LFM_CUDA(cudaMemsetAsync(s->flag, 0, sizeof(int), s->stream));
        LFM_CUDA(cudaMemcpyAsync(s->q, sq, qBytes, cudaMemcpyDeviceToDevice, s->stream));
        if (pBytes) LFM_CUDA(cudaMemcpyAsync(s->a32.prim, sq + qBytes, pBytes, cudaMemcpyDeviceToDevice, s->stream));
        s->primsValid = pBytes != 0;   // FP64: rebuilt by ensurePrims
        s->primParity = 0;
        LFM_CUDA(cudaStreamSynchronize(s->stream));
        return LFM_OK;
    };
    cudaError_t ce = cudaMemcpyAsync(sq, s->q, qBytes, cudaMemcpyDeviceToDevice, s->stream);
    if (ce == cudaSuccess && pBytes)
        ce = cudaMemcpyAsync(sq + qBytes, s->a32.prim, pBytes, cudaMemcpyDeviceToDevice, s->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s->stream);
    if (ce != cudaSuccess) {
        cudaFree(saved);
        return cudaFail(ce, "autotune state copy");
    }
    std::vector<float> ms((size_t)trial_steps);
    int best = -1;
    for (size_t k = 0; k < cand.size(); ++k) {
        if (s->fluxVariants && applyTuning(s, cand[k]) != LFM_OK) continue;   // refused shapes are skipped
        if ((rc = restore())) break;
        float warm = 0.0f;
        if ((rc = lfm_solver_bench(s, 1, dt, flush_bytes, &warm))) break;   // captures the step graph
        if ((rc = restore())) break;
        if ((rc = lfm_solver_bench(s, trial_steps, dt, flush_bytes, ms.data()))) break;
        std::vector<float> sorted(ms);
        std::sort(sorted.begin(), sorted.end());
        cand[k].ms_per_step = sorted[sorted.size() / 2];
        if (best < 0 || cand[k].ms_per_step < cand[(size_t)best].ms_per_step) best = (int)k;
        if (n_tried) {
            if (tried && *n_tried < capacity) tried[*n_tried] = cand[k];
            ++*n_tried;
        }
    }
    const lfm_solver_tuning pick = best >= 0 ? cand[(size_t)best] : before;
    if (s->fluxVariants) {
        const int rc2 = applyTuning(s, pick);
        if (!rc) rc = rc2;
    }
    const int rc3 = restore();
    if (!rc) rc = rc3;
    cudaFree(saved);
    if (!rc && best < 0) rc = lfm::setError(LFM_ERR_INVALID, "no flux kernel configuration could be timed");
    if (chosen) *chosen = pick;
    return rc;
}
