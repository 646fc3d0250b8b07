// Kernels of the FP32-bulk form, one thread per cell, ghost or face: thin
// wrappers over the device functions of solver_fp32.cuh (which the batched
// multi-case kernel shares).
#include "solver_fp32.cuh"
#include "solver_launch.h"

namespace lfm {
namespace dev {

// Primitives of cells, ghosts and halos [first, a.nt): first = 0 after a new
// state; once the update kernels keep the cells' current, first = nc (ghosts
// and halos), or nc + ng (halos only) when the update also writes the ghosts.
template <int D>
__global__ void __launch_bounds__(256) k_prep32(const __grid_constant__ Args<float> a, int first) {
    const int t = first + LFM_GLOBAL_ID();
    if (t < a.nt) prep32<D>(a, t);
}

template <int D>
__global__ void __launch_bounds__(256) k_grad32(const __grid_constant__ Args<float> a) {
    const int c = LFM_GLOBAL_ID();
    if (c < a.nc) grad32<D>(a, c);
}

// Six blocks per SM (40 registers, no spills): full-occupancy gathers.
template <int D, bool LES>
__global__ void __launch_bounds__(256, 6) k_vis32(const __grid_constant__ Args<float> a) {
    const int c = LFM_GLOBAL_ID();
    if (c < a.nc) vis32<D, LES>(a, c);
}

template <int D, int SCH, bool LES>
__global__ void __launch_bounds__(256) k_flux32(const __grid_constant__ Args<float> a) {
    const int f = LFM_GLOBAL_ID();
    if (f < a.nf) flux32<D, SCH, true, LES, true>(a, f);
}

// Cell-centred form (flux32_cell): one thread per cell over the faces it
// owns. 3D at three blocks per SM (80 registers; the cell keeps its own 23
// rows across its faces): the 9.4M-cell wake's flux 3.42 -> 3.27 ms per step;
// at four blocks per SM it spills (3.66 ms).
template <int D, int SCH>
__global__ void __launch_bounds__(256, 3) k_flux32_cell(const __grid_constant__ Args<float> a) {
    const int c = LFM_GLOBAL_ID();
    if (c < a.nc) flux32_cell<D, SCH>(a, c);
}

// Warp-interleaved cells: warp j of block b updates the 32 cells of chunk
// j * gridDim.x + b (coalesced within the warp), so a block's eight warps lie
// in chunks spread over the mesh. The cells with boundary faces come first in
// the solver order and write their ghosts' next state in FP64 (boundary
// conditions with divisions, on an FP64 pipe that issues about two
// instructions per clock per SM); interleaved, their warps land on different
// SMs instead of filling the first few blocks, whose SMs would otherwise
// finish last. Without the ghost work (GH false) a block keeps 256
// consecutive cells, which the large cases' gathers from HBM prefer.
template <int D, bool RES, bool GH, bool ELL>
__device__ __forceinline__ void update_thread(const Args<float>& a, double Ak, double Bk, double dt, float dt32,
                                              int first) {
    const int c = GH ? (int)(((threadIdx.x >> 5) * gridDim.x + blockIdx.x) << 5) + (int)(threadIdx.x & 31u)
                     : (int)LFM_GLOBAL_ID();
    if (c < a.nc) update32<D, RES, GH, ELL>(a, c, Ak, Bk, dt, dt32, first);
}

template <int D, bool RES, bool GH, bool ELL>
__global__ void __launch_bounds__(256) k_update32(const __grid_constant__ Args<float> a, double Ak, double Bk,
                                                  double dt, float dt32, int first) {
    update_thread<D, RES, GH, ELL>(a, Ak, Bk, dt, dt32, first);
}

// 2D list-gather updates at six blocks per SM (40 registers; the ghost branch
// spills 40 bytes on the few cells that take it): 0.092 -> 0.087 ms per step
// on the 768x512 cylinder, whose 393k cells then fill 1.7 waves instead of
// 2.02. The table gathers keep their registers (all loads in flight).
template <bool RES, bool GH>
__global__ void __launch_bounds__(256, 6) k_update32_2d(const __grid_constant__ Args<float> a, double Ak, double Bk,
                                                       double dt, float dt32, int first) {
    update_thread<2, RES, GH, false>(a, Ak, Bk, dt, dt32, first);
}

// Fused flux + update (fluxupdate32): one thread per cell, cells mapped as
// in the update kernel that writes ghosts (warp-interleaved chunks).
template <int D, int SCH, bool RES>
__global__ void __launch_bounds__(256) k_fluxupdate32(const __grid_constant__ Args<float> a, double Ak, double Bk,
                                                      double dt, float dt32, int first) {
    const int c = (int)(((threadIdx.x >> 5) * gridDim.x + blockIdx.x) << 5) + (int)(threadIdx.x & 31u);
    if (c < a.nc) fluxupdate32<D, SCH, false, RES, true>(a, c, Ak, Bk, dt, dt32, first);
}

template <int D, int SCH>
void launch_fluxupdate32_scheme(const Args<float>& a, const StageConfig& s, cudaStream_t st) {
    const unsigned nb = (unsigned)((a.nc + 255) / 256);
    const float dt32 = (float)s.dt;
    if (s.withRes) k_fluxupdate32<D, SCH, true><<<nb, 256, 0, st>>>(a, s.A, s.B, s.dt, dt32, s.first);
    else k_fluxupdate32<D, SCH, false><<<nb, 256, 0, st>>>(a, s.A, s.B, s.dt, dt32, s.first);
}

template <int D, bool ELL>
void launch_update32(const Args<float>& a, const StageConfig& s, cudaStream_t st) {
    const unsigned nb = (unsigned)((a.nc + 255) / 256);   // eight 32-cell chunks per block
    const float dt32 = (float)s.dt;
    if (D == 2 && !ELL) {
        if (a.cellGhosts) {
            if (s.withRes) k_update32_2d<true, true><<<nb, 256, 0, st>>>(a, s.A, s.B, s.dt, dt32, s.first);
            else k_update32_2d<false, true><<<nb, 256, 0, st>>>(a, s.A, s.B, s.dt, dt32, s.first);
        } else {
            if (s.withRes) k_update32_2d<true, false><<<nb, 256, 0, st>>>(a, s.A, s.B, s.dt, dt32, s.first);
            else k_update32_2d<false, false><<<nb, 256, 0, st>>>(a, s.A, s.B, s.dt, dt32, s.first);
        }
        return;
    }
    if (a.cellGhosts) {
        if (s.withRes) k_update32<D, true, true, ELL><<<nb, 256, 0, st>>>(a, s.A, s.B, s.dt, dt32, s.first);
        else k_update32<D, false, true, ELL><<<nb, 256, 0, st>>>(a, s.A, s.B, s.dt, dt32, s.first);
    } else {
        if (s.withRes) k_update32<D, true, false, ELL><<<nb, 256, 0, st>>>(a, s.A, s.B, s.dt, dt32, s.first);
        else k_update32<D, false, false, ELL><<<nb, 256, 0, st>>>(a, s.A, s.B, s.dt, dt32, s.first);
    }
}

template <int D>
__global__ void __launch_bounds__(256) k_set_state32(const __grid_constant__ Args<float> a, const double* q,
                                                     int64_t stride) {
    const int c = LFM_GLOBAL_ID();
    if (c < a.nc) set_state32<D>(a, q, stride, c);
}

template <int D>
__global__ void __launch_bounds__(256) k_to_perturbation(const __grid_constant__ Args<float> a, const double* q,
                                                         int64_t stride) {
    const int c = LFM_GLOBAL_ID();
    if (c < a.nc) to_perturbation<D>(a, q, stride, c);
}

// ---------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------
static inline unsigned nblocks(int n, int b) { return (unsigned)((n + b - 1) / b); }

template <int D>
void launch_fp32(const Args<float>& a, const StageConfig& s, int which, cudaStream_t st) {
    switch (which) {
        case 0: {
            const int first = s.fullPrep ? 0 : (a.cellGhosts ? a.nc + a.ng : a.nc);
            if (a.nt > first) k_prep32<D><<<nblocks(a.nt - first, 256), 256, 0, st>>>(a, first);
            break;
        }
        case 1:
            if (s.needGrad) k_grad32<D><<<nblocks(a.nc, 256), 256, 0, st>>>(a);
            break;
        case 2:
            if (s.needVis && a.smagC) k_vis32<D, true><<<nblocks(a.nc, 256), 256, 0, st>>>(a);
            else if (s.needVis) k_vis32<D, false><<<nblocks(a.nc, 256), 256, 0, st>>>(a);
            break;
        case 3:
            if (s.fluxStaging.stages > 0) {   // staged kernel (configured for this scheme, laminar)
                launch_flux32_staged(a, s, st);
            } else if (a.nf == 0) {
            } else if (a.fOwn && !a.smagC && s.scheme != kSchemeAUSM) {   // cell-centred
                if (s.scheme == kSchemeM1) k_flux32_cell<D, kSchemeM1><<<nblocks(a.nc, 256), 256, 0, st>>>(a);
                else k_flux32_cell<D, kSchemeM2><<<nblocks(a.nc, 256), 256, 0, st>>>(a);
            } else if (a.smagC) {   // Smagorinsky LES variants
                if (s.scheme == kSchemeM1) k_flux32<D, kSchemeM1, true><<<nblocks(a.nf, 256), 256, 0, st>>>(a);
                else if (s.scheme == kSchemeM2) k_flux32<D, kSchemeM2, true><<<nblocks(a.nf, 256), 256, 0, st>>>(a);
                else k_flux32<D, kSchemeAUSM, true><<<nblocks(a.nf, 256), 256, 0, st>>>(a);
            } else {
                if (s.scheme == kSchemeM1) k_flux32<D, kSchemeM1, false><<<nblocks(a.nf, 256), 256, 0, st>>>(a);
                else if (s.scheme == kSchemeM2) k_flux32<D, kSchemeM2, false><<<nblocks(a.nf, 256), 256, 0, st>>>(a);
                else k_flux32<D, kSchemeAUSM, false><<<nblocks(a.nf, 256), 256, 0, st>>>(a);
            }
            break;
        case 4:
            if (a.cfEll) launch_update32<D, true>(a, s, st);
            else launch_update32<D, false>(a, s, st);
            break;
        default: break;
    }
}

void launch_kernel_fp32(const Args<float>& a, const StageConfig& s, int which, cudaStream_t st) {
    if (a.D == 2)
        launch_fp32<2>(a, s, which, st);
    else
        launch_fp32<3>(a, s, which, st);
}

void launch_fluxupdate32(const Args<float>& a, const StageConfig& s, cudaStream_t st) {
    if (a.D == 2) {
        if (s.scheme == kSchemeM1) launch_fluxupdate32_scheme<2, kSchemeM1>(a, s, st);
        else if (s.scheme == kSchemeM2) launch_fluxupdate32_scheme<2, kSchemeM2>(a, s, st);
        else launch_fluxupdate32_scheme<2, kSchemeAUSM>(a, s, st);
    } else {
        if (s.scheme == kSchemeM1) launch_fluxupdate32_scheme<3, kSchemeM1>(a, s, st);
        else if (s.scheme == kSchemeM2) launch_fluxupdate32_scheme<3, kSchemeM2>(a, s, st);
        else launch_fluxupdate32_scheme<3, kSchemeAUSM>(a, s, st);
    }
}

void launch_set_state32(const Args<float>& a, const double* q, int64_t stride, cudaStream_t st) {
    if (a.D == 2)
        k_set_state32<2><<<nblocks(a.nc, 256), 256, 0, st>>>(a, q, stride);
    else
        k_set_state32<3><<<nblocks(a.nc, 256), 256, 0, st>>>(a, q, stride);
}

void launch_to_perturbation(const Args<float>& a, const double* q, int64_t stride, cudaStream_t st) {
    if (a.D == 2)
        k_to_perturbation<2><<<nblocks(a.nc, 256), 256, 0, st>>>(a, q, stride);
    else
        k_to_perturbation<3><<<nblocks(a.nc, 256), 256, 0, st>>>(a, q, stride);
}

}  // namespace dev
}  // namespace lfm

// ---------------------------------------------------------------------------
// Self-test of the integer-pipe conversions (lfm_selftest_fp_convert).
// ---------------------------------------------------------------------------
namespace {

__global__ void k_convert_selftest(int64_t n, const unsigned* f32, const unsigned long long* f64,
                                   unsigned long long* f64_of_f32, unsigned* f32_of_f64) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f64_of_f32[i] = (unsigned long long)__double_as_longlong(lfm::dev::f32_to_f64(__uint_as_float(f32[i])));
    f32_of_f64[i] = __float_as_uint(lfm::dev::f64_to_f32(__longlong_as_double((long long)f64[i])));
}

}  // namespace

extern "C" int lfm_selftest_fp_convert(int64_t n, const uint32_t* f32_bits, const uint64_t* f64_bits,
                                       uint64_t* f64_of_f32, uint32_t* f32_of_f64) {
    if (n <= 0 || !f32_bits || !f64_bits || !f64_of_f32 || !f32_of_f64) return -1;
    unsigned *d32 = nullptr, *o32 = nullptr;
    unsigned long long *d64 = nullptr, *o64 = nullptr;
    cudaError_t e = cudaMalloc(&d32, (size_t)n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&o32, (size_t)n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d64, (size_t)n * 8);
    if (e == cudaSuccess) e = cudaMalloc(&o64, (size_t)n * 8);
    if (e == cudaSuccess) e = cudaMemcpy(d32, f32_bits, (size_t)n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d64, f64_bits, (size_t)n * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_convert_selftest<<<(unsigned)((n + 255) / 256), 256>>>(n, d32, d64, o64, o32);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(f64_of_f32, o64, (size_t)n * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(f32_of_f64, o32, (size_t)n * 4, cudaMemcpyDeviceToHost);
    cudaFree(d32);
    cudaFree(o32);
    cudaFree(d64);
    cudaFree(o64);
    return e == cudaSuccess ? 0 : -3;
}
