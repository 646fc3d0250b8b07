// Batched multi-case time step: many independent cases (uneven cell counts,
// mixed schemes and dimensions) advanced by one persistent kernel per RK stage.
//
// Every case lives in its own block of a device arena, with the FP32-bulk
// arrays of a single-case solver (Args<float>). A stage is four phases over
// all cases -- ghost states and primitives (of every cell too, right after a
// case's state was set); gradients and viscous terms; face fluxes; gather, RK
// update and the cells' next primitives -- separated by grid-wide barriers. Work
// is a flat list of tiles per phase (a tile is a run of consecutive cells or
// faces of one case); each block takes an equal contiguous range of it, so
// uneven cases load-balance at tile granularity. The tile lists and case table are read
// from device memory at run time: cases join and leave between time steps
// without recapturing the CUDA graph of a step.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "solver_kernels.cuh"

namespace lfm {
namespace dev {

constexpr int kBatchMaxStages = 8;
constexpr int kBatchPhases = 4;   // prep, grad+vis, flux, update

// One case of a batch: its kernel arguments (device pointers into its arena
// block), time step and RK coefficients.
struct __align__(16) BatchCase {
    Args<float> a;
    double dt;
    float dt32;
    double rkA[kBatchMaxStages], rkB[kBatchMaxStages];
    int scheme, needGrad, needVis, residuals;
};

// A run of `count` consecutive items (cells, ghosts or faces) of case `slot`.
struct __align__(16) BatchTile {
    int slot, start, count, pad;
};

// Zeroed before every time step: the grid-barrier arrival counter of each stage.
struct BatchCtl {
    unsigned barrier[kBatchMaxStages];
};

struct BatchArgs {
    const BatchCase* cases;
    const BatchTile* tiles[kBatchPhases];
    const int* nTiles;          // [kBatchPhases]
    BatchCtl* ctl;
    int* error;                 // set when a grid barrier gives up waiting
    int itemsPerThread;
    unsigned barrierExtra;      // arrivals every barrier waits for beyond the grid's (test aid; 0)
};

// Kernel variants, chosen from the cases in the batch: compiling out what no
// case needs lowers the kernel's register count and raises its occupancy.
constexpr int kBatchVariant2DInviscid = 0;   // 2D, M1/M2, mu = 0
constexpr int kBatchVariant2D = 1;           // 2D, any scheme, viscous
constexpr int kBatchVariantGeneral = 2;      // 2D and 3D, any scheme, viscous

// Launches stage `stage` of every case as one persistent (cooperative when
// `cooperative`) kernel of `grid` blocks of `block` threads (128, 256 or 512).
cudaError_t launch_batch_stage(const BatchArgs& b, int stage, int block, int variant, int grid, bool cooperative,
                               cudaStream_t st);
// Resident blocks per SM of the stage kernel at `block` threads.
int batch_blocks_per_sm(int block, int variant);
// Stage `stage` as one kernel per phase (grid-stride over each phase's
// tiles, kernel boundaries in place of the grid barriers); each kernel's grid
// is bps (0 = all that fit) resident blocks per SM x sms.
cudaError_t launch_batch_phased(const BatchArgs& b, int stage, int block, int variant, int bps, int sms,
                                cudaStream_t st);

}  // namespace dev
}  // namespace lfm
