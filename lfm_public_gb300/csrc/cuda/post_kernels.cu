// Post-processing on the device: per-cell pressure statistics, wall forces
// and pressure probes, computed from the resident state.
//
// The arithmetic follows the reference's order with explicitly rounded FP64
// operations (no contraction), as the reference's CPU code computes them:
// postProcAverage (src/cfd_v0.cpp:3083-3104), postProcForces
// (src/cfd_v0.cpp:3169-3250). Sums over the faces of a patch run in the
// reference's order (ghost order: cells ascending, faces in cell order).
#include "solver_device.cuh"
#include "solver_launch.h"

namespace lfm {
namespace dev {

namespace {

inline unsigned nb(int n, int b) { return (unsigned)((n + b - 1) / b); }

// p = (r (gamma - 1)) (E - |u|^2 / 2), E = rE / r, |u|^2 = sum (rU_k / r)^2
// (postProcAverage, src/cfd_v0.cpp:3088-3098).
template <int D>
__device__ __forceinline__ double pressure_of(const double* qv, double gm1) {
    const double r = qv[0];
    double velMag = 0.0;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const double vel = __ddiv_rn(qv[k + 1], r);
        velMag = __dadd_rn(velMag, __dmul_rn(vel, vel));
    }
    const double E = __ddiv_rn(qv[D + 1], r);
    return __dmul_rn(__dmul_rn(r, gm1), __dsub_rn(E, __dmul_rn(0.5, velMag)));
}

template <int D>
__device__ __forceinline__ void load_state(const double* q, int64_t nt, const QOffset& qo, int c, double* qv) {
#pragma unroll
    for (int v = 0; v < D + 2; ++v) qv[v] = __dadd_rn(q[(size_t)v * nt + c], qo.v[v]);
}

template <int D>
__global__ void __launch_bounds__(256) k_stats(const double* q, int64_t nt, QOffset qo, int nc, double gm1, double n,
                                               double* avg, double* rms) {
    const int c = LFM_GLOBAL_ID();
    if (c >= nc) return;
    double qv[D + 2];
    load_state<D>(q, nt, qo, c, qv);
    const double p = pressure_of<D>(qv, gm1);
    const double a = __dadd_rn(avg[c], p);
    avg[c] = a;
    const double x = __dsub_rn(p, __ddiv_rn(a, n));
    rms[c] = __dadd_rn(rms[c], __dmul_rn(x, x));
}

template <int D>
__global__ void __launch_bounds__(256) k_probe(const double* q, int64_t nt, QOffset qo, const int* cells, int n,
                                               double gm1, double pInf, double* out) {
    const int i = LFM_GLOBAL_ID();
    if (i >= n) return;
    double qv[D + 2];
    load_state<D>(q, nt, qo, cells[i], qv);
    out[i] = __dsub_rn(pressure_of<D>(qv, gm1), pInf);
}

// Force terms of ghost g: S_k (p - p_inf) and the D products tau[k][m] S_m of
// the viscous force, in the order the reference accumulates them
// (src/cfd_v0.cpp:3180-3240). The reference's ghost cells hold, after a
// step, the boundary state of the last stage's starting state. The ghost
// state here is (ghost mode):
//   kGhostStored -- the stored one (FP64 path: written by the last stage),
//   kGhostFresh  -- the boundary state of the current state (no stage run),
//   kGhostUndo   -- the boundary state of q' - B dq, the last stage's
//                   starting state recovered from its update q' += B dq
//                   (FP32-bulk path, which stores no ghost states).
template <typename T, int D>
__global__ void __launch_bounds__(128) k_force_terms(const Args<T> a, QOffset qo, const double* gS, const double* gD,
                                                     int mode, double Blast, double* terms) {
    const int g = LFM_GLOBAL_ID();
    if (g >= a.ng) return;
    const int ng = a.ng;
    const int64_t nt = a.nt;
    const int cell = a.gCell[g];
    double qc[D + 2], qg[D + 2];
    load_state<D>(a.q, nt, qo, cell, qc);
    if (mode == kGhostFresh) {
        ghost_bc<T, D>(a, g, qc, qg);
    } else if (mode == kGhostUndo) {
        double qs[D + 2];
#pragma unroll
        for (int v = 0; v < D + 2; ++v)
            qs[v] = __dadd_rn(__dsub_rn(a.q[(size_t)v * nt + cell],
                                        __dmul_rn(Blast, (double)a.dq[(size_t)v * a.nc + cell])),
                              qo.v[v]);
        ghost_bc<T, D>(a, g, qs, qg);
    } else {
        load_state<D>(a.q, nt, qo, a.nc + g, qg);
    }
    const double r = qc[0];
    double Uvec[D], Umag = 0.0;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        Uvec[k] = __ddiv_rn(qc[k + 1], r);
        Umag = __dadd_rn(Umag, __dmul_rn(Uvec[k], Uvec[k]));
    }
    Umag = __dsqrt_rn(Umag);
    const double E = __ddiv_rn(qc[D + 1], r);
    const double p = __dmul_rn(__dmul_rn(r, a.gm1), __dsub_rn(E, __dmul_rn(__dmul_rn(0.5, Umag), Umag)));
    double S[D], dv[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        S[k] = gS[(size_t)k * ng + g];
        dv[k] = gD[(size_t)k * ng + g];
    }
#pragma unroll
    for (int k = 0; k < D; ++k) terms[(size_t)k * ng + g] = __dmul_rn(S[k], __dsub_rn(p, a.pInf));
    double dmag = __dmul_rn(dv[0], dv[0]);
#pragma unroll
    for (int k = 1; k < D; ++k) dmag = __dadd_rn(dmag, __dmul_rn(dv[k], dv[k]));
    dmag = __dsqrt_rn(dmag);
    const double dinv = __ddiv_rn(1.0, dmag);
    double dn[D];
#pragma unroll
    for (int k = 0; k < D; ++k) dn[k] = __dmul_rn(dv[k], dinv);
    double dudx[D][D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
        const double cu = __ddiv_rn(qc[i + 1], qc[0]);
        const double au = __ddiv_rn(qg[i + 1], qg[0]);
#pragma unroll
        for (int j = 0; j < D; ++j) dudx[i][j] = __dmul_rn(__dmul_rn(__dsub_rn(au, cu), dn[j]), dinv);
    }
    // the deviatoric stress in the reference's evaluation order (:3222-3230)
    const double mu = a.mu;
    double tau[D][D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
        tau[i][i] = __dmul_rn(2.0, dudx[i][i]);
#pragma unroll
        for (int b1 = i + 1; b1 < D + i; ++b1) {
            const int b = b1 % D;
            tau[i][b] = __dmul_rn(mu, __dadd_rn(dudx[i][b], dudx[b][i]));
            tau[i][i] = __dsub_rn(tau[i][i], dudx[b][b]);
        }
        tau[i][i] = __dmul_rn(tau[i][i], __dmul_rn(2.0 / 3.0, mu));
    }
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) terms[(size_t)(D + i * D + j) * ng + g] = __dmul_rn(tau[i][j], S[j]);
}

// One thread per (patch, component): the patch's terms summed in ghost order,
// as the reference's sequential loop does.
template <int D>
__global__ void k_force_sum(const double* terms, int ng, const int* gPatch, const int* patches, int nPatches,
                            double* fp, double* fv) {
    const int t = LFM_GLOBAL_ID();
    if (t >= nPatches * D) return;
    const int i = t / D, k = t % D, patch = patches[i];
    double sp = 0.0, sv = 0.0;
    for (int g = 0; g < ng; ++g) {
        if (gPatch[g] != patch) continue;
        sp = __dadd_rn(sp, terms[(size_t)k * ng + g]);
#pragma unroll
        for (int j = 0; j < D; ++j) sv = __dsub_rn(sv, terms[(size_t)(D + k * D + j) * ng + g]);
    }
    fp[t] = sp;
    fv[t] = sv;
}

}  // namespace

void launch_stats(int D, const double* q, int64_t nt, QOffset qo, int nc, double gm1, int n, double* avg,
                  double* rms, cudaStream_t st) {
    if (nc <= 0) return;
    if (D == 2)
        k_stats<2><<<nb(nc, 256), 256, 0, st>>>(q, nt, qo, nc, gm1, (double)n, avg, rms);
    else
        k_stats<3><<<nb(nc, 256), 256, 0, st>>>(q, nt, qo, nc, gm1, (double)n, avg, rms);
}

void launch_probe(int D, const double* q, int64_t nt, QOffset qo, const int* cells, int n, double gm1, double pInf,
                  double* out, cudaStream_t st) {
    if (n <= 0) return;
    if (D == 2)
        k_probe<2><<<nb(n, 256), 256, 0, st>>>(q, nt, qo, cells, n, gm1, pInf, out);
    else
        k_probe<3><<<nb(n, 256), 256, 0, st>>>(q, nt, qo, cells, n, gm1, pInf, out);
}

template <typename T>
void launch_forces(const Args<T>& a, QOffset qo, const double* gS, const double* gD, const int* gPatch, int mode,
                   double Blast, const int* patches, int nPatches, double* terms, double* fp, double* fv,
                   cudaStream_t st) {
    if (a.ng <= 0 || nPatches <= 0) return;
    if (a.D == 2) {
        k_force_terms<T, 2><<<nb(a.ng, 128), 128, 0, st>>>(a, qo, gS, gD, mode, Blast, terms);
        k_force_sum<2><<<nb(nPatches * 2, 64), 64, 0, st>>>(terms, a.ng, gPatch, patches, nPatches, fp, fv);
    } else {
        k_force_terms<T, 3><<<nb(a.ng, 128), 128, 0, st>>>(a, qo, gS, gD, mode, Blast, terms);
        k_force_sum<3><<<nb(nPatches * 3, 64), 64, 0, st>>>(terms, a.ng, gPatch, patches, nPatches, fp, fv);
    }
}
template void launch_forces<double>(const Args<double>&, QOffset, const double*, const double*, const int*, int,
                                    double, const int*, int, double*, double*, double*, cudaStream_t);
template void launch_forces<float>(const Args<float>&, QOffset, const double*, const double*, const int*, int, double,
                                   const int*, int, double*, double*, double*, cudaStream_t);

}  // namespace dev
}  // namespace lfm
