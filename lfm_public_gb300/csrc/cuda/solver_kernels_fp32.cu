// Kernels of the FP32-bulk form, one thread per cell, ghost or face: thin
// wrappers over the device functions of solver_fp32.cuh (which the batched
// multi-case kernel shares).
#include "solver_fp32.cuh"
#include "solver_launch.h"

namespace lfm {
namespace dev {

template <int D>
__global__ void __launch_bounds__(256) k_prep32(const __grid_constant__ Args<float> a) {
    const int t = LFM_GLOBAL_ID();
    if (t < a.nt) prep32<D>(a, t);
}

template <int D>
__global__ void __launch_bounds__(256) k_grad32(const __grid_constant__ Args<float> a) {
    const int c = LFM_GLOBAL_ID();
    if (c < a.nc) grad32<D>(a, c);
}

template <int D>
__global__ void __launch_bounds__(256) k_vis32(const __grid_constant__ Args<float> a) {
    const int c = LFM_GLOBAL_ID();
    if (c < a.nc) vis32<D>(a, c);
}

template <int D, int SCH>
__global__ void __launch_bounds__(256) k_flux32(const __grid_constant__ Args<float> a) {
    const int f = LFM_GLOBAL_ID();
    if (f < a.nf) flux32<D, SCH>(a, f);
}

// ---------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------
static inline unsigned nblocks(int n, int b) { return (unsigned)((n + b - 1) / b); }

template <int D>
void launch_fp32(const Args<float>& a, const StageConfig& s, int which, cudaStream_t st) {
    switch (which) {
        case 0: k_prep32<D><<<nblocks(a.nt, 256), 256, 0, st>>>(a); break;
        case 1:
            if (s.needGrad) k_grad32<D><<<nblocks(a.nc, 256), 256, 0, st>>>(a);
            break;
        case 2:
            if (s.needVis) k_vis32<D><<<nblocks(a.nc, 256), 256, 0, st>>>(a);
            break;
        case 3:
            if (s.scheme == kSchemeM1) k_flux32<D, kSchemeM1><<<nblocks(a.nf, 256), 256, 0, st>>>(a);
            else if (s.scheme == kSchemeM2) k_flux32<D, kSchemeM2><<<nblocks(a.nf, 256), 256, 0, st>>>(a);
            else k_flux32<D, kSchemeAUSM><<<nblocks(a.nf, 256), 256, 0, st>>>(a);
            break;
        case 4: launch_update_fp32(a, s, st); break;
        default: break;
    }
}

void launch_kernel_fp32(const Args<float>& a, const StageConfig& s, int which, cudaStream_t st) {
    if (a.D == 2)
        launch_fp32<2>(a, s, which, st);
    else
        launch_fp32<3>(a, s, which, st);
}

}  // namespace dev
}  // namespace lfm
