// Persistent multi-case stage kernel of the batch engine (batch.cuh).
#include <algorithm>

#include "batch.cuh"
#include "solver_fp32.cuh"

namespace lfm {
namespace dev {

namespace {

// A grid barrier gives up after kBarrierTimeoutNs of waiting (read from the
// GPU's global nanosecond timer), or after kBarrierSpinLimit polls should
// that timer not advance.
constexpr unsigned long long kBarrierTimeoutNs = 1000000000ull;   // 1 s
constexpr unsigned kBarrierSpinLimit = 1u << 25;

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier of the blocks of one launch (all resident: the launch is
// cooperative, or its grid is sized to the resident capacity). Arrival is an
// atomic increment after a release fence; waiting is bounded: after about a
// second, or once another block has given up, the block sets the error flag
// and the caller returns without touching further data.
__device__ __forceinline__ bool grid_barrier(unsigned* counter, unsigned target, int* error) {
    __shared__ int sOk;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(counter, 1u);
        int ok = 1;
        unsigned spins = 0;
        const unsigned long long t0 = global_ns();
        while (*(volatile unsigned*)counter < target) {
            if (*(volatile int*)error != 0 || ++spins > kBarrierSpinLimit || global_ns() - t0 > kBarrierTimeoutNs) {
                atomicOr(error, 1);
                ok = 0;
                break;
            }
            __nanosleep(40);
        }
        __threadfence();
        sOk = ok;
    }
    __syncthreads();
    return sOk != 0;
}

// One item of a phase: a cell or ghost (prep, only in a case's first step
// after a new state: afterwards the update writes the next stage's primitives
// of each cell and of its boundary ghosts), a cell (grad + vis, update) or a
// face (flux) of the case in shared memory. FULL = false is the variant
// for batches of M1/M2 cases without viscosity: no gradient or viscous code
// is compiled in, which keeps the kernel's register count (and so its
// occupancy) down.
template <int PH, int D, bool FULL>
__device__ __forceinline__ void item(const BatchCase& bc, int stage, int i) {
    const Args<float>& a = bc.a;
    if (PH == 0) {
        prep32<D>(a, i);
    } else if (PH == 1) {
        if (FULL) {
            if (bc.needGrad) grad32<D>(a, i);
            if (bc.needVis) vis32<D>(a, i);
        }
    } else if (PH == 2) {
        if (bc.scheme == kSchemeM1)
            flux32<D, kSchemeM1, FULL>(a, i);
        else if (!FULL || bc.scheme == kSchemeM2)
            flux32<D, kSchemeM2, FULL>(a, i);
        else
            flux32<D, kSchemeAUSM, FULL>(a, i);
    } else {   // through the fixed-width face table where the case has one
        const int first = stage == 0;
        if (bc.residuals && first) {
            if (a.cfEll) update32<D, true, true, true>(a, i, bc.rkA[stage], bc.rkB[stage], bc.dt, bc.dt32, first);
            else update32<D, true, true, false>(a, i, bc.rkA[stage], bc.rkB[stage], bc.dt, bc.dt32, first);
        } else {
            if (a.cfEll) update32<D, false, true, true>(a, i, bc.rkA[stage], bc.rkB[stage], bc.dt, bc.dt32, first);
            else update32<D, false, true, false>(a, i, bc.rkA[stage], bc.rkB[stage], bc.dt, bc.dt32, first);
        }
    }
}

// The tiles of phase PH assigned to this block: a contiguous range of the
// phase's tile list (neighbouring tiles of a case share cached neighbours).
// The block keeps the current tile's case in shared memory and reloads it when
// the case changes.
template <int PH, int BLOCK, int DIMS, bool FULL>
__device__ __forceinline__ void phase_tiles(const BatchArgs& b, int stage, BatchCase& sc, int& sSlot) {
    const int nT = b.nTiles[PH];
    const long long t0 = (long long)nT * blockIdx.x / gridDim.x;
    const long long t1 = (long long)nT * (blockIdx.x + 1) / gridDim.x;
    const BatchTile* tiles = b.tiles[PH];
    for (long long t = t0; t < t1; ++t) {
        const BatchTile td = tiles[t];
        const bool reload = td.slot != sSlot;
        __syncthreads();
        if (reload) {
            const int4* src = reinterpret_cast<const int4*>(b.cases + td.slot);
            int4* dst = reinterpret_cast<int4*>(&sc);
            constexpr int n16 = (int)(sizeof(BatchCase) / 16);
            for (int k = threadIdx.x; k < n16; k += BLOCK) dst[k] = src[k];
            if (threadIdx.x == 0) sSlot = td.slot;
            __syncthreads();
        }
        const int end = td.start + td.count;
        for (int k = 0; k < b.itemsPerThread; ++k) {
            const int i = td.start + (int)threadIdx.x + k * BLOCK;
            if (i < end) {
                if (DIMS == 2 || sc.a.D == 2)
                    item<PH, 2, FULL>(sc, stage, i);
                else
                    item<PH, 3, FULL>(sc, stage, i);
            }
        }
    }
}

// Stage `stage` of every case: [prep] | [grad + vis] | flux | update, with a
// grid barrier between phases (none after the last; the bracketed phases and
// their barriers only when they have tiles). Within the launch every array
// is written by one phase and read only by later ones, so no block reads a
// line it cached before another block rewrote it.
// DIMS = 2: every case is 2D; DIMS = 0: 2D and 3D cases. FULL: see item().
template <int BLOCK, int DIMS, bool FULL>
__global__ void __launch_bounds__(BLOCK) k_batch_stage(const __grid_constant__ BatchArgs b, int stage) {
    __shared__ BatchCase sc;
    __shared__ int sSlot;
    if (threadIdx.x == 0) sSlot = -1;
    __syncthreads();
    unsigned* counter = &b.ctl->barrier[stage];
    unsigned target = b.barrierExtra;   // 0 except under lfm_batch_debug_barrier
    if (b.nTiles[0] > 0) {
        phase_tiles<0, BLOCK, DIMS, FULL>(b, stage, sc, sSlot);
        target += gridDim.x;
        if (!grid_barrier(counter, target, b.error)) return;
    }
    if (FULL && b.nTiles[1] > 0) {
        phase_tiles<1, BLOCK, DIMS, FULL>(b, stage, sc, sSlot);
        target += gridDim.x;
        if (!grid_barrier(counter, target, b.error)) return;
    }
    phase_tiles<2, BLOCK, DIMS, FULL>(b, stage, sc, sSlot);
    target += gridDim.x;
    if (!grid_barrier(counter, target, b.error)) return;
    phase_tiles<3, BLOCK, DIMS, FULL>(b, stage, sc, sSlot);
}

// One phase of a stage over every case, for the phased launch mode.
template <int PH, int BLOCK, int DIMS, bool FULL>
__global__ void __launch_bounds__(BLOCK) k_batch_phase(const __grid_constant__ BatchArgs b, int stage) {
    __shared__ BatchCase sc;
    __shared__ int sSlot;
    if (threadIdx.x == 0) sSlot = -1;
    __syncthreads();
    phase_tiles<PH, BLOCK, DIMS, FULL>(b, stage, sc, sSlot);
}

template <int PH, int BLOCK, int DIMS, bool FULL>
cudaError_t launch_phase(const BatchArgs& b, int stage, int bps, int sms, cudaStream_t st) {
    static thread_local int fit = -1;   // resident blocks per SM of this kernel
    auto k = k_batch_phase<PH, BLOCK, DIMS, FULL>;
    if (fit < 0) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k, BLOCK, 0);
        if (e != cudaSuccess || fit < 1) return e != cudaSuccess ? e : cudaErrorInvalidConfiguration;
    }
    const int per = bps > 0 ? std::min(bps, fit) : fit;
    k<<<per * sms, BLOCK, 0, st>>>(b, stage);
    return cudaGetLastError();
}

template <int BLOCK, int DIMS, bool FULL>
cudaError_t launch_phases(const BatchArgs& b, int stage, int bps, int sms, cudaStream_t st) {
    cudaError_t e = launch_phase<0, BLOCK, DIMS, FULL>(b, stage, bps, sms, st);
    if (e == cudaSuccess && FULL) e = launch_phase<1, BLOCK, DIMS, FULL>(b, stage, bps, sms, st);
    if (e == cudaSuccess) e = launch_phase<2, BLOCK, DIMS, FULL>(b, stage, bps, sms, st);
    if (e == cudaSuccess) e = launch_phase<3, BLOCK, DIMS, FULL>(b, stage, bps, sms, st);
    return e;
}

template <int BLOCK>
cudaError_t launch_phases_variant(const BatchArgs& b, int stage, int variant, int bps, int sms, cudaStream_t st) {
    switch (variant) {
        case kBatchVariant2DInviscid: return launch_phases<BLOCK, 2, false>(b, stage, bps, sms, st);
        case kBatchVariant2D: return launch_phases<BLOCK, 2, true>(b, stage, bps, sms, st);
        default: return launch_phases<BLOCK, 0, true>(b, stage, bps, sms, st);
    }
}

// Kernel of a launch shape and variant (kBatchVariant*).
template <int BLOCK>
auto kernel_of(int variant) -> void (*)(BatchArgs, int) {
    switch (variant) {
        case kBatchVariant2DInviscid: return k_batch_stage<BLOCK, 2, false>;
        case kBatchVariant2D: return k_batch_stage<BLOCK, 2, true>;
        default: return k_batch_stage<BLOCK, 0, true>;
    }
}

template <int BLOCK>
cudaError_t launch_block(const BatchArgs& b, int stage, int variant, int grid, bool cooperative, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(BLOCK);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = cooperative ? attr : nullptr;
    cfg.numAttrs = cooperative ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel_of<BLOCK>(variant), b, stage);
}

}  // namespace

cudaError_t launch_batch_stage(const BatchArgs& b, int stage, int block, int variant, int grid, bool cooperative,
                               cudaStream_t st) {
    switch (block) {
        case 128: return launch_block<128>(b, stage, variant, grid, cooperative, st);
        case 512: return launch_block<512>(b, stage, variant, grid, cooperative, st);
        default: return launch_block<256>(b, stage, variant, grid, cooperative, st);
    }
}

cudaError_t launch_batch_phased(const BatchArgs& b, int stage, int block, int variant, int bps, int sms,
                                cudaStream_t st) {
    switch (block) {
        case 128: return launch_phases_variant<128>(b, stage, variant, bps, sms, st);
        case 512: return launch_phases_variant<512>(b, stage, variant, bps, sms, st);
        default: return launch_phases_variant<256>(b, stage, variant, bps, sms, st);
    }
}

int batch_blocks_per_sm(int block, int variant) {
    int n = 0;
    cudaError_t e;
    switch (block) {
        case 128: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel_of<128>(variant), 128, 0); break;
        case 512: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel_of<512>(variant), 512, 0); break;
        default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel_of<256>(variant), 256, 0); break;
    }
    return e == cudaSuccess ? n : 0;
}

}  // namespace dev
}  // namespace lfm
