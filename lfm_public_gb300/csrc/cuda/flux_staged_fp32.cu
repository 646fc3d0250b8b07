// Staged FP32-bulk flux kernel (M1 / M2, laminar): the face rhs of
// face_rhs32 with every value the face reads copied into shared memory ahead
// of its use.
//
// The plain flux kernel (k_flux32) reads a face's cells, then gathers their
// primitives and viscous rows: two dependent round trips to memory per face,
// which its resident warps cannot cover (on the 9.4M-cell wake, whose
// gathers come from HBM, it reaches about half of the measured bandwidth).
// Here a block walks its chunks of `faces` consecutive faces (one face per
// thread) as a software pipeline of `ST` shared-memory buffers per thread:
//
//   iteration k:  issue the copies of chunk k + ST - 1 (cp.async, 4 bytes per
//                 value: the cells' primitive and viscous rows, the face's
//                 geometry rows) with the cell indices loaded one iteration
//                 earlier; load the indices of chunk k + ST; wait for the
//                 copy group of chunk k; compute chunk k from shared memory.
//
// So while a thread computes one face, the values of its next ST - 1 faces
// and the indices of the one after are in flight. Every thread writes and
// reads only its own columns of the buffers (threads are independent: no
// block barrier, no wait on another thread), and cp.async.wait_group makes a
// thread's own copies visible to it. The arithmetic is face_rhs32_cells on a
// view of the buffers, so the rhs has the plain kernel's bits.
//
// Off by default: measured on GB300 (FP32-bulk, CUDA events, per step) the
// staged kernels are slower than the plain one in every configuration tried.
// The 9.4M-cell M2 wake's flux takes 3.43 ms plain, 5.3 ms with two buffers
// of 128 or 256 faces, 5.4 (three of 128), 6.2 (four of 64), 8.3-9.0 (chunks
// of 32 or 64), 5.8 in the slot form below; the 768 x 512 M1 cylinder's
// 0.068 ms plain, 0.102-0.125 staged. The plain kernel's neighbour re-reads
// (the P side of three consecutive faces, the N side of nearby faces) hit L1;
// the 166-221 KB of shared memory the buffers take leave L1 a fraction of its
// 256 KB, and the faces in flight per SM are fewer than the plain kernel keeps
// in registers (1024 threads at 64 registers). LFM_FLUX_STAGES selects them
// (capi_solver.cu).
//
// Buffer of one chunk (F = faces, floats; columns: face slot t, P side t,
// N side F + t):
//   cell rows   [PR + VR][2F]   rho', m'[D], u'[D], R psi' | dudx, dTdx, sigmaU
//   face rows   [FR + GR][F]    S[D], w, K[D], lapc | 1/|d|, d/|d| (boundary faces)
//   ghost flags [F] bytes
#include "solver_fp32.cuh"
#include "solver_launch.h"

namespace lfm {
namespace dev {

namespace {

__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <int D>
struct StagedRows {
    static constexpr int PR = 2 * D + 2;        // the primitives the M1 / M2 flux reads (no c)
    static constexpr int VR = kVisRows<D>;      // viscous rows
    static constexpr int FR = 2 * D + 2;        // S[D], w, K[D], lapc
    static constexpr int GR = D + 1;            // 1/|d|, d/|d|[D] (read on boundary faces)
    // floats of one chunk's buffer (F a multiple of 4: the flags end on a float)
    __host__ __device__ static constexpr int floats(int F) { return (2 * (PR + VR) + FR + GR) * F + F / 4; }
};

// The arrays face_rhs32_cells reads, pointing into one chunk's buffer.
struct StagedFace32 {
    const RefState32& ref;
    const float* prim;
    const float* V;
    const float* grad;
    const float* S;
    const float* d;
    const float* w;
    const float* K;
    const float* lapc;
    const float* dinv;
    const float* dnorm;
    const uint8_t* fGhost;
    const float* smagC;
    int nt, nf;
};

// Copies of face f (cells i, j) into buffer `b`, column t.
template <int D>
__device__ __forceinline__ void stage_face(const Args<float>& g, float* b, int F, int t, int f, int i, int j,
                                           uint8_t ghost, bool vis) {
    using R = StagedRows<D>;
    const size_t nt = (size_t)g.nt, nf = (size_t)g.nf;
    float* cb = b;
    float* fb = b + 2 * (R::PR + R::VR) * F;
#pragma unroll
    for (int r = 0; r < R::PR; ++r) {
        cp_async4(cb + r * 2 * F + t, g.prim + r * nt + i);
        cp_async4(cb + r * 2 * F + F + t, g.prim + r * nt + j);
    }
#pragma unroll
    for (int k = 0; k < D; ++k) cp_async4(fb + k * F + t, g.S + k * nf + f);
    cp_async4(fb + D * F + t, g.w + f);
    if (vis) {
#pragma unroll
        for (int k = 0; k < D; ++k) cp_async4(fb + (D + 1 + k) * F + t, g.K + k * nf + f);
        cp_async4(fb + (2 * D + 1) * F + t, g.lapc + f);
        if (!ghost) {
            float* vb = cb + R::PR * 2 * F;
#pragma unroll
            for (int r = 0; r < R::VR; ++r) {
                cp_async4(vb + r * 2 * F + t, g.V + r * nt + i);
                cp_async4(vb + r * 2 * F + F + t, g.V + r * nt + j);
            }
        } else {
            cp_async4(fb + R::FR * F + t, g.dinv + f);
#pragma unroll
            for (int k = 0; k < D; ++k) cp_async4(fb + (R::FR + 1 + k) * F + t, g.dnorm + k * nf + f);
        }
    }
    reinterpret_cast<uint8_t*>(fb + (R::FR + R::GR) * F)[t] = ghost;
}

template <int D, int SCH, int ST>
__global__ void __launch_bounds__(256) k_flux32_staged(const __grid_constant__ Args<float> g, int nChunks) {
    using R = StagedRows<D>;
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    const int F = (int)blockDim.x, t = (int)threadIdx.x;
    const int SF = R::floats(F);
    const int G = (int)gridDim.x, c0 = (int)blockIdx.x;
    const int n = c0 < nChunks ? (nChunks - 1 - c0) / G + 1 : 0;   // chunks of this block
    const int nf = g.nf;
    const bool vis = g.ref.mu != 0.0f;
    // cell indices and boundary flag of the next chunk to issue
    int ni = 0, nj = 0;
    uint8_t ng = 0;
    auto faceOf = [&](int k) { return (c0 + k * G) * F + t; };
    auto loadIdx = [&](int k) {
        const int f = faceOf(k);
        if (k < n && f < nf) {
            ni = g.fP[f];
            nj = g.fN[f];
            ng = g.fGhost[f];
        }
    };
    auto issue = [&](int k) {
        const int f = faceOf(k);
        if (k < n && f < nf) stage_face<D>(g, smem + (k % ST) * SF, F, t, f, ni, nj, ng, vis);
        cp_async_commit();   // one group per chunk (empty past the end)
    };
#pragma unroll
    for (int k = 0; k < ST - 1; ++k) {
        loadIdx(k);
        issue(k);
    }
    loadIdx(ST - 1);
    for (int k = 0; k < n; ++k) {
        issue(k + ST - 1);
        loadIdx(k + ST);
        cp_async_wait<ST - 1>();   // chunk k's group is complete
        const int f = faceOf(k);
        if (f < nf) {
            const float* b = smem + (k % ST) * SF;
            const float* fb = b + 2 * (R::PR + R::VR) * F;
            const StagedFace32 v{g.ref,
                                 b,
                                 b + R::PR * 2 * F,
                                 nullptr,
                                 fb,
                                 nullptr,
                                 fb + D * F,
                                 fb + (D + 1) * F,
                                 fb + (2 * D + 1) * F,
                                 fb + R::FR * F,
                                 fb + (R::FR + 1) * F,
                                 reinterpret_cast<const uint8_t*>(fb + (R::FR + R::GR) * F),
                                 nullptr,
                                 2 * F,
                                 F};
            float rhs[D + 2];
            face_rhs32_cells<D, SCH, true, false, false>(v, t, t, F + t, rhs);
#pragma unroll
            for (int q = 0; q < D + 2; ++q) g.flux[(size_t)q * (size_t)nf + f] = rhs[q];
        }
    }
    cp_async_wait<0>();   // no copy outlives the block
}

// ---------------------------------------------------------------------------
// Slot form (stages == 1): shared memory as a second landing buffer beside
// the registers. Each thread owns one slot of shared memory; it copies its
// face's values from the slot into registers, issues the copies of its next
// face (grid-stride) into the slot, and computes the face from registers,
// so the register file holds the faces being computed while shared memory
// holds the faces in flight, at the plain kernel's occupancy.
// ---------------------------------------------------------------------------
template <int D>
struct SlotRows {
    static constexpr int PR = 2 * D + 2, VR = kVisRows<D>;
    static constexpr int CELL = 2 * (PR + VR);   // P then N side of each row
    static constexpr int FACE = 2 * D + 2;       // S[D], w, K[D], lapc
    static constexpr int N = CELL + FACE;        // boundary faces keep 1/|d|, d/|d| in the V rows' place
};

// A face's values in registers, read by face_rhs32_cells with i = 0, j = 1, f = 0.
template <int D>
struct RegFace32 {
    const RefState32& ref;
    float prim[2 * (2 * D + 2)];
    float V[2 * kVisRows<D>];
    float S[D], w[1], K[D], lapc[1], dinv[1], dnorm[D];
    uint8_t fGhost[1];
    const float* d;
    const float* grad;
    const float* smagC;
    int nt, nf;
};

template <int D>
__device__ __forceinline__ void slot_issue(const Args<float>& g, float* slot, int f, int i, int j, bool ghost,
                                           bool vis) {
    using R = SlotRows<D>;
    const size_t nt = (size_t)g.nt, nf = (size_t)g.nf;
    constexpr int B = 256;   // threads of a block: the slot's row stride
#pragma unroll
    for (int r = 0; r < R::PR; ++r) {
        cp_async4(slot + (2 * r) * B, g.prim + r * nt + i);
        cp_async4(slot + (2 * r + 1) * B, g.prim + r * nt + j);
    }
    float* fb = slot + R::CELL * B;
#pragma unroll
    for (int k = 0; k < D; ++k) cp_async4(fb + k * B, g.S + k * nf + f);
    cp_async4(fb + D * B, g.w + f);
    if (vis) {
#pragma unroll
        for (int k = 0; k < D; ++k) cp_async4(fb + (D + 1 + k) * B, g.K + k * nf + f);
        cp_async4(fb + (2 * D + 1) * B, g.lapc + f);
        float* vb = slot + 2 * R::PR * B;
        if (!ghost) {
#pragma unroll
            for (int r = 0; r < R::VR; ++r) {
                cp_async4(vb + (2 * r) * B, g.V + r * nt + i);
                cp_async4(vb + (2 * r + 1) * B, g.V + r * nt + j);
            }
        } else {
            cp_async4(vb, g.dinv + f);
#pragma unroll
            for (int k = 0; k < D; ++k) cp_async4(vb + (1 + k) * B, g.dnorm + k * nf + f);
        }
    }
}

template <int D>
__device__ __forceinline__ void slot_read(const float* slot, RegFace32<D>& v, bool ghost, bool vis) {
    using R = SlotRows<D>;
    constexpr int B = 256;
#pragma unroll
    for (int r = 0; r < 2 * R::PR; ++r) v.prim[r] = slot[r * B];
    const float* fb = slot + R::CELL * B;
#pragma unroll
    for (int k = 0; k < D; ++k) v.S[k] = fb[k * B];
    v.w[0] = fb[D * B];
    if (vis) {
#pragma unroll
        for (int k = 0; k < D; ++k) v.K[k] = fb[(D + 1 + k) * B];
        v.lapc[0] = fb[(2 * D + 1) * B];
        const float* vb = slot + 2 * R::PR * B;
        if (!ghost) {
#pragma unroll
            for (int r = 0; r < 2 * R::VR; ++r) v.V[r] = vb[r * B];
        } else {
            v.dinv[0] = vb[0];
#pragma unroll
            for (int k = 0; k < D; ++k) v.dnorm[k] = vb[(1 + k) * B];
        }
    }
    v.fGhost[0] = ghost ? 1 : 0;
}

// Blocks per SM: 2D four (64 registers), 3D three (85 registers: at four the
// 3D face spills).
template <int D, int SCH>
__global__ void __launch_bounds__(256, D == 2 ? 4 : 3) k_flux32_slot(const __grid_constant__ Args<float> g) {
    extern __shared__ float4 smem4[];
    float* slot = reinterpret_cast<float*>(smem4) + threadIdx.x;
    const int stride = (int)(gridDim.x * blockDim.x), nf = g.nf;
    const bool vis = g.ref.mu != 0.0f;
    int f = LFM_GLOBAL_ID();
    if (f >= nf) return;
    bool gh = g.fGhost[f] != 0;
    slot_issue<D>(g, slot, f, g.fP[f], g.fN[f], gh, vis);
    cp_async_commit();
    int fn = f + stride, ni = 0, nj = 0;
    bool ngh = false;
    if (fn < nf) {
        ni = g.fP[fn];
        nj = g.fN[fn];
        ngh = g.fGhost[fn] != 0;
    }
    for (; f < nf; f += stride) {
        cp_async_wait<0>();   // face f is in the slot
        RegFace32<D> v{g.ref};
        slot_read<D>(slot, v, gh, vis);
        v.d = nullptr;
        v.grad = nullptr;
        v.smagC = nullptr;
        v.nt = 2;
        v.nf = 1;
        if (fn < nf) {   // the next face into the slot while this one is computed
            slot_issue<D>(g, slot, fn, ni, nj, ngh, vis);
            cp_async_commit();
        }
        gh = ngh;
        const int fnn = fn + stride;
        if (fnn < nf) {
            ni = g.fP[fnn];
            nj = g.fN[fnn];
            ngh = g.fGhost[fnn] != 0;
        }
        float rhs[D + 2];
        face_rhs32_cells<D, SCH, true, false, false>(v, 0, 0, 1, rhs);
#pragma unroll
        for (int q = 0; q < D + 2; ++q) g.flux[(size_t)q * (size_t)nf + f] = rhs[q];
        fn = fnn;
    }
    cp_async_wait<0>();
}

template <int D, int SCH>
cudaError_t configureSlot(int nf, int* grid, size_t* smem) {
    auto k = k_flux32_slot<D, SCH>;
    const size_t bytes = sizeof(float) * (size_t)SlotRows<D>::N * 256;
    int perSM = 0, dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k, 256, bytes)) != cudaSuccess) return e;
    if (perSM < 1) return cudaErrorInvalidConfiguration;
    const int need = (nf + 255) / 256;
    *grid = std::max(1, std::min(need, perSM * sms));
    *smem = bytes;
    return cudaSuccess;
}

template <int D, int SCH, int ST>
cudaError_t configure(int faces, int nf, int* grid, size_t* smem) {
    auto k = k_flux32_staged<D, SCH, ST>;
    const size_t bytes = sizeof(float) * (size_t)StagedRows<D>::floats(faces) * ST;
    int perSM = 0, dev = 0, sms = 0, maxSmem = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess) return e;
    if (bytes > (size_t)maxSmem) return cudaErrorInvalidValue;
    if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k, faces, bytes)) != cudaSuccess) return e;
    if (perSM < 1) return cudaErrorInvalidConfiguration;
    const int chunks = (nf + faces - 1) / faces;
    *grid = std::max(1, std::min(chunks, perSM * sms));
    *smem = bytes;
    return cudaSuccess;
}

template <int D, int SCH>
cudaError_t configureScheme(const FluxStaging& fs, int nf, int* grid, size_t* smem) {
    switch (fs.stages) {
        case 1: return configureSlot<D, SCH>(nf, grid, smem);
        case 2: return configure<D, SCH, 2>(fs.faces, nf, grid, smem);
        case 3: return configure<D, SCH, 3>(fs.faces, nf, grid, smem);
        case 4: return configure<D, SCH, 4>(fs.faces, nf, grid, smem);
        default: return cudaErrorInvalidValue;
    }
}

template <int D, int SCH>
void launchScheme(const Args<float>& a, const FluxStaging& fs, cudaStream_t st) {
    const int chunks = (a.nf + fs.faces - 1) / fs.faces;
    switch (fs.stages) {
        case 1: k_flux32_slot<D, SCH><<<fs.grid, 256, fs.smem, st>>>(a); break;
        case 2: k_flux32_staged<D, SCH, 2><<<fs.grid, fs.faces, fs.smem, st>>>(a, chunks); break;
        case 3: k_flux32_staged<D, SCH, 3><<<fs.grid, fs.faces, fs.smem, st>>>(a, chunks); break;
        case 4: k_flux32_staged<D, SCH, 4><<<fs.grid, fs.faces, fs.smem, st>>>(a, chunks); break;
        default: break;
    }
}

}  // namespace

bool flux_staging_supported(int scheme, bool les) { return !les && (scheme == kSchemeM1 || scheme == kSchemeM2); }

cudaError_t configure_flux_staging(int D, int scheme, int nf, FluxStaging& fs) {
    if (fs.stages == 1) fs.faces = 256;
    if (fs.faces < 32 || fs.faces > 256 || fs.faces % 32 != 0) return cudaErrorInvalidValue;
    cudaError_t e;
    if (D == 2)
        e = scheme == kSchemeM1 ? configureScheme<2, kSchemeM1>(fs, nf, &fs.grid, &fs.smem)
                                : configureScheme<2, kSchemeM2>(fs, nf, &fs.grid, &fs.smem);
    else
        e = scheme == kSchemeM1 ? configureScheme<3, kSchemeM1>(fs, nf, &fs.grid, &fs.smem)
                                : configureScheme<3, kSchemeM2>(fs, nf, &fs.grid, &fs.smem);
    return e;
}

void launch_flux32_staged(const Args<float>& a, const StageConfig& s, cudaStream_t st) {
    const FluxStaging& fs = s.fluxStaging;
    if (a.nf == 0) return;
    if (a.D == 2) {
        if (s.scheme == kSchemeM1) launchScheme<2, kSchemeM1>(a, fs, st);
        else launchScheme<2, kSchemeM2>(a, fs, st);
    } else {
        if (s.scheme == kSchemeM1) launchScheme<3, kSchemeM1>(a, fs, st);
        else launchScheme<3, kSchemeM2>(a, fs, st);
    }
}

}  // namespace dev
}  // namespace lfm
