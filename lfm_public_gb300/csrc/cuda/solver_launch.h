// Host-side launch interface of the time-step kernels.
#pragma once

#include <cuda_runtime.h>

#include "solver_kernels.cuh"
#include "tile_desc.h"

namespace lfm {
namespace dev {

// Staged FP32-bulk flux kernel (flux_staged_fp32.cu): faces per block (one
// chunk), shared-memory buffers per thread (the staging depth, 0 = the plain
// flux kernel), and the persistent grid and dynamic shared memory set by
// configure_flux_staging.
struct FluxStaging {
    int stages = 0;
    int faces = 128;
    int grid = 0;
    size_t smem = 0;
};

// What one RK stage runs (src/mesh_solver.cpp:500-672).
struct StageConfig {
    int scheme = 0;       // kSchemeM1 / M2 / AUSM
    bool needGrad = false;
    bool needVis = true;
    double A = 0, B = 1;  // low-storage RK coefficients of this stage
    double dt = 0;
    int first = 0;        // stage 0: dq starts from zero (prepare_for_timestep)
    int withRes = 0;      // record the stage-0 residual
    // FP32-bulk: the update writes the next stage's cell primitives, so the
    // preparation pass covers the ghosts only unless the cell primitives are
    // stale (a new state was set).
    bool fullPrep = true;
    // FP32-bulk flux: the staged kernel when stages > 0
    FluxStaging fluxStaging;
};

template <typename T>
void launch_stage(const Args<T>& a, const StageConfig& s, cudaStream_t st);
template <typename T>
void launch_kernel(const Args<T>& a, const StageConfig& s, int which, cudaStream_t st);
template <>
void launch_stage<float>(const Args<float>& a, const StageConfig& s, cudaStream_t st);
template <>
void launch_kernel<float>(const Args<float>& a, const StageConfig& s, int which, cudaStream_t st);
// FP32-bulk kernels (perturbation form).
void launch_kernel_fp32(const Args<float>& a, const StageConfig& s, int which, cudaStream_t st);
// FP32-bulk fused flux + update of every cell (laminar, a.cellGhosts set): the
// face rhs evaluated by the cells themselves; the next stage's primitives go
// to a.primW, which must not be a.prim.
void launch_fluxupdate32(const Args<float>& a, const StageConfig& s, cudaStream_t st);
// Staged flux kernel: for M1 / M2 without the LES terms; configure sets the
// kernel's shared-memory limit (outside graph capture) and fs.grid, fs.smem.
bool flux_staging_supported(int scheme, bool les);
cudaError_t configure_flux_staging(int D, int scheme, int nf, FluxStaging& fs);
void launch_flux32_staged(const Args<float>& a, const StageConfig& s, cudaStream_t st);
// q' = q - q_ref for the cells of an FP32-bulk solver from an absolute state
// [nq][stride] on the device.
void launch_to_perturbation(const Args<float>& a, const double* q, int64_t stride, cudaStream_t st);
// A new FP32-bulk state from an absolute one: q', the cells' primitives and
// (with a.cellGhosts) their boundary ghosts' states and primitives.
void launch_set_state32(const Args<float>& a, const double* q, int64_t stride, cudaStream_t st);

// Rows of the per-cell primitive array: FP64 keeps 1/rho, u[D], R psi, c;
// the FP32 perturbation form keeps rho', m'[D], u'[D], R psi', c.
template <typename T>
constexpr int primRows(int D) {
    return sizeof(T) == sizeof(double) ? D + 3 : 2 * D + 3;
}
// Offset added to the stored state before use (the FP32-bulk form stores
// q - q_ref; zero for the FP64 path).
struct QOffset {
    double v[5];
};
// mode 0: max CFL, mode 1: min dt
void launch_cfl(int D, const double* q, QOffset qo, int nt, int nc, const double* volInv, const int* sOff, const double* cellS,
                double dt, int mode, double maxCo, double* partial, double* out, cudaStream_t st);
void launch_res_sum(const double* res, int nc, double* partial, double* out, cudaStream_t st);
void launch_set_flag(int* flag, int v, cudaStream_t st);
// dst[v][c] = src[v][c] + sign * off.v[v], v < nq, c < n (row strides in elements).
void launch_offset_rows(double* dst, int64_t dstStride, const double* src, int64_t srcStride, int n, int nq,
                        QOffset off, double sign, cudaStream_t st);
// Halo slots [first, first + nh) of dst (row stride dstNt) take `rows` values
// of cell srcCell[h] of partition srcPart[h] (base srcBase[p], stride srcNt[p]).
template <typename X>
void launch_halo_gather(X* dst, int dstNt, int first, int rows, int nh, const int* srcPart, const int* srcCell,
                        X* const* srcBase, const int* srcNt, cudaStream_t st);

// Post-processing (post_kernels.cu).
void launch_stats(int D, const double* q, int64_t nt, QOffset qo, int nc, double gm1, int n, double* avg,
                  double* rms, cudaStream_t st);
void launch_probe(int D, const double* q, int64_t nt, QOffset qo, const int* cells, int n, double gm1, double pInf,
                  double* out, cudaStream_t st);
enum { kGhostStored = 0, kGhostFresh = 1, kGhostUndo = 2 };
template <typename T>
void launch_forces(const Args<T>& a, QOffset qo, const double* gS, const double* gD, const int* gPatch, int mode,
                   double Blast, const int* patches, int nPatches, double* terms, double* fp, double* fv,
                   cudaStream_t st);

// Fused FP32-bulk stage over tiles (tile_kernels.cu).
struct TileArgs {
    const TileDesc* tiles;
    const int* ints;
    const float* floats;
    const uint8_t* bytes;
    const float* primIn;   // primitives at the stage start (the update writes the other buffer)
    int nTiles;
    int block;             // threads of a block
    size_t smemBytes;      // dynamic shared memory of a block
    int needGrad, needVis; // passes to run
    int haveV, haveGrad;   // arrays the fluxes read (zero where not computed)
};
size_t tile_smem_bytes(int D, int maxL, int maxLF, bool haveV, bool haveGrad);
// g: the solver's arguments with prim = the output primitive buffer.
cudaError_t launch_tile_stage(const Args<float>& g, const TileArgs& t, const StageConfig& s, cudaStream_t st);

constexpr int kKernelsPerStage = 5;  // prep, grad, vis, flux, update
// Timing slots of lfm_solver_profile_step: the five kernels, then the fused
// tile stage (which does the work of the five), then the fused flux + update
// (which does the work of the last two).
constexpr int kKernelSlots = 7;
constexpr int kSlotTileStage = 5;
constexpr int kSlotFluxUpdate = 6;
inline const char* kernelName(int i) {
    static const char* names[] = {"k_prep", "k_grad", "k_vis", "k_flux", "k_update", "k_tile_stage",
                                  "k_flux_update"};
    return (i >= 0 && i < kKernelSlots) ? names[i] : "";
}

}  // namespace dev
}  // namespace lfm
