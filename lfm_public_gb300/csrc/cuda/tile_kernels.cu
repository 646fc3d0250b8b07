// Fused FP32-bulk stage kernel over tiles (tile_desc.h): one launch per RK
// stage, one block per tile. The block stages the tile's primitives (its
// cells and two rings around them) in shared memory, computes the gradients
// and viscous terms of its cells and the first ring, the rhs of every face of
// its cells and the update of its cells - the work of the preparation,
// gradient, viscous, flux and update kernels, with the intermediate arrays
// in shared memory instead of HBM. It calls the same device functions on a
// view of the tile (Args whose arrays point into shared memory and into the
// tile's copies of the face data), so every value rounds as in the separate
// kernels. The update writes the next stage's primitives (cells and their
// boundary ghosts) into the other of two primitive buffers, which no block
// of this launch reads.
#include "solver_fp32.cuh"
#include "solver_launch.h"
#include "tile_desc.h"

namespace lfm {
namespace dev {

namespace {

template <int D>
struct TileRows {
    static constexpr int P = 2 * D + 3;        // primitives
    static constexpr int V = D * D + 2 * D;    // dudx, dTdx, sigmaU
    static constexpr int G = 2 * D + D * D;    // rho, p, U gradients
    static constexpr int Q = D + 2;            // face rhs
};

template <int D, int SCH, bool RES>
__global__ void __launch_bounds__(256) k_tile_stage(const __grid_constant__ Args<float> g,
                                                    const __grid_constant__ TileArgs t, double Ak, double Bk,
                                                    double dt, float dt32, int first) {
    using R = TileRows<D>;
    extern __shared__ float sm[];
    __shared__ Args<float> la;
    const TileDesc td = t.tiles[blockIdx.x];
    const int nL = td.nL, nLF = td.nLF;
    // gradients and viscous terms only where the case reads them
    const int vRows = t.haveV ? R::V : 0, gRows = t.haveGrad ? R::G : 0;
    float* sPrim = sm;
    float* sV = sPrim + (size_t)R::P * nL;
    float* sGrad = sV + (size_t)vRows * nL;
    float* sFlux = sGrad + (size_t)gRows * nL;
    const int* L = t.ints + td.iOff;
    if (threadIdx.x == 0) {
        la = g;
        const int* fP = L + nL;
        const int* fN = fP + nLF;
        const int* cfOff = fN + nLF;
        const float* F = t.floats + td.fOff;
        la.prim = sPrim;
        la.V = sV;
        la.grad = sGrad;
        la.flux = sFlux;
        la.nt = nL;
        la.nf = nLF;
        la.fP = fP;
        la.fN = fN;
        la.cfOff = cfOff;
        la.cfList = cfOff + td.nV + 1;
        la.cfNbr = la.cfList + td.nE;
        la.cfEll = nullptr;
        la.S = F;
        la.d = F + (size_t)D * nLF;
        la.w = F + (size_t)2 * D * nLF;
        la.K = F + (size_t)(2 * D + 1) * nLF;
        la.lapc = F + (size_t)(3 * D + 1) * nLF;
        la.dinv = F + (size_t)(3 * D + 2) * nLF;
        la.dnorm = F + (size_t)(3 * D + 3) * nLF;
        la.volInv32 = F + (size_t)(4 * D + 3) * nLF;
        la.fGhost = t.bytes + td.bOff;
    }
    // primitives of every local cell (stage start), zero gradients and
    // viscous terms (ghosts keep zero, as the separate kernels' arrays do)
    for (int k = threadIdx.x; k < R::P * nL; k += blockDim.x) {
        const int row = k / nL, lc = k - row * nL;
        sPrim[k] = t.primIn[(size_t)row * (size_t)g.nt + (size_t)L[lc]];
    }
    for (int k = threadIdx.x; k < (vRows + gRows) * nL; k += blockDim.x) sV[k] = 0.0f;
    __syncthreads();
    const Args<float>& a = la;
    if (t.needGrad || t.needVis)
        for (int lc = threadIdx.x; lc < td.nV; lc += blockDim.x) {
            if (t.needGrad) grad32<D>(a, lc);
            if (t.needVis) vis32<D>(a, lc);
        }
    __syncthreads();
    for (int lf = threadIdx.x; lf < td.nFA; lf += blockDim.x) flux32<D, SCH>(a, lf);
    __syncthreads();
    for (int lc = threadIdx.x; lc < td.nA; lc += blockDim.x) {
        CellIn32<D> in;
        load_cell32<D>(g, td.c0 + lc, first, in);
        float sum[R::Q];
        gather32<D>(a, lc, sum);
        apply32<D, RES, true>(g, td.c0 + lc, sum, in, Ak, Bk, dt, dt32, first);
    }
}

template <int D, int SCH>
cudaError_t launchTiles(const Args<float>& g, const TileArgs& t, const StageConfig& s, cudaStream_t st) {
    auto k = s.withRes ? k_tile_stage<D, SCH, true> : k_tile_stage<D, SCH, false>;
    static thread_local size_t smemSet[2] = {0, 0};   // per kernel instance: attribute raised to
    const size_t smem = t.smemBytes;
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024 && smem > smemSet[s.withRes ? 1 : 0]) {
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        smemSet[s.withRes ? 1 : 0] = smem;
    }
    k<<<t.nTiles, t.block, smem, st>>>(g, t, s.A, s.B, s.dt, (float)s.dt, s.first);
    return cudaGetLastError();
}

}  // namespace

size_t tile_smem_bytes(int D, int maxL, int maxLF, bool haveV, bool haveGrad) {
    const int P = 2 * D + 3, V = D * D + 2 * D, G = 2 * D + D * D;
    const int rows = P + (haveV ? V : 0) + (haveGrad ? G : 0);
    return sizeof(float) * ((size_t)rows * (size_t)maxL + (size_t)(D + 2) * (size_t)maxLF);
}

cudaError_t launch_tile_stage(const Args<float>& g, const TileArgs& t, const StageConfig& s, cudaStream_t st) {
    if (g.D == 2) {
        if (s.scheme == kSchemeM1) return launchTiles<2, kSchemeM1>(g, t, s, st);
        if (s.scheme == kSchemeM2) return launchTiles<2, kSchemeM2>(g, t, s, st);
        return launchTiles<2, kSchemeAUSM>(g, t, s, st);
    }
    if (s.scheme == kSchemeM1) return launchTiles<3, kSchemeM1>(g, t, s, st);
    if (s.scheme == kSchemeM2) return launchTiles<3, kSchemeM2>(g, t, s, st);
    return launchTiles<3, kSchemeAUSM>(g, t, s, st);
}

}  // namespace dev
}  // namespace lfm
