// Device helpers shared by the FP64 and FP32-bulk time-step kernels.
#pragma once

#include "solver_kernels.cuh"

namespace lfm {
namespace dev {

#define LFM_GLOBAL_ID() ((int)(blockIdx.x * blockDim.x + threadIdx.x))

template <typename T>
__device__ __forceinline__ T interp(T w, T a, T b) {
    return w * a + (T(1) - w) * b;
}

// 1/x in FP64 by Newton-Raphson iteration for the reciprocal (y <- y + y(1 - xy),
// each step squaring the relative error), seeded with the single-precision
// reciprocal approximation of x truncated to binary32 (PTX rcp.approx.ftz.f32,
// relative error near 2^-23 with the truncation): two steps leave the result
// within an ulp or two of the correctly rounded 1/x, for four FP64 FMAs -- GB300
// issues about two FP64 instructions per clock per SM, and a full-precision
// division takes several more. Values outside binary32's normal range take
// the division.
__device__ __forceinline__ double rcp64(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ffu) - 896;   // binary32 biased exponent
    if (ex < 2 || ex > 252) return 1.0 / x;
    const unsigned fb = ((unsigned)(b >> 32) & 0x80000000u) | ((unsigned)ex << 23) | (unsigned)((b >> 29) & 0x7fffffu);
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(__uint_as_float(fb)));
    // widen r exactly: rebias its (normal) exponent, move its mantissa up
    const unsigned rb = __float_as_uint(r);
    double y = __longlong_as_double((long long)(((unsigned long long)(rb & 0x80000000u) << 32) |
                                                ((unsigned long long)(((rb >> 23) & 0xffu) + 896u) << 52) |
                                                ((unsigned long long)(rb & 0x7fffffu) << 29)));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

// -x and isfinite(x) of an FP64 value on the integer pipe (a sign-bit flip;
// an exponent test), leaving GB300's FP64 pipe to the arithmetic.
__device__ __forceinline__ double neg_bits(double x) {
    return __hiloint2double(__double2hiint(x) ^ (int)0x80000000u, __double2loint(x));
}
__device__ __forceinline__ float neg_bits(float x) { return __uint_as_float(__float_as_uint(x) ^ 0x80000000u); }
__device__ __forceinline__ bool finite_bits(double x) {
    return ((unsigned)__double2hiint(x) & 0x7ff00000u) != 0x7ff00000u;
}

// interp with the weight of N given (1 - w, precomputed per face).
template <typename T>
__device__ __forceinline__ T interp2(T w, T wN, T a, T b) {
    return w * a + wN * b;
}

template <typename T, int D>
__device__ __forceinline__ T dotv(const T* a, const T* b) {
    T s = a[0] * b[0];
#pragma unroll
    for (int k = 1; k < D; ++k) s += a[k] * b[k];
    return s;
}

// Deviatoric stress of a velocity gradient g (row a = gradient of u_a), in the
// reference's evaluation order (src/cfd_v0.cpp:1813-1822).
template <typename T, int D>
__device__ __forceinline__ void stress(const T g[D][D], T mu, T tau[D][D]) {
#pragma unroll
    for (int a = 0; a < D; ++a) {
        tau[a][a] = T(2) * g[a][a];
#pragma unroll
        for (int b1 = a + 1; b1 < D + a; ++b1) {
            const int b = b1 % D;
            tau[a][b] = mu * (g[a][b] + g[b][a]);
            tau[a][a] -= g[b][b];
        }
        tau[a][a] *= T(2.0 / 3.0) * mu;
    }
}

// Smagorinsky subgrid stress added to a cell's tauMC (calc_VIS_Smagorinsky,
// src/cfd_v0.cpp:1675-1695): -C |S| S_ab + (C |S| div u / 3) delta_ab with
// S the symmetric part of the velocity gradient g, |S| = sqrt(2 S_ab S_ab)
// and C = -2 (0.16 Delta)^2 the cell's model constant.
template <typename T, int D>
__device__ __forceinline__ void sgs_stress(const T g[D][D], T C, T out[D][D]) {
    T sm = T(0), divu = T(0);
#pragma unroll
    for (int x = 0; x < D; ++x) {
#pragma unroll
        for (int y = 0; y < D; ++y) {
            const T s = T(0.5) * (g[x][y] + g[y][x]);
            sm += s * s;
        }
        divu += g[x][x];
    }
    sm = sqrt(T(2) * sm);
    const T cs = C * sm;
#pragma unroll
    for (int x = 0; x < D; ++x) {
#pragma unroll
        for (int y = 0; y < D; ++y) out[x][y] = -(cs * (T(0.5) * (g[x][y] + g[y][x])));
        out[x][x] += cs * divu / T(3);
    }
}

// Rows of the per-cell viscous array: dudx (D x D), dTdx, sigmaU, then with
// Smagorinsky LES the SGS stress (D x D).
template <int D>
constexpr int kVisRows = D * D + 2 * D;

// Minmod-limited face reconstruction from the upwind side (calc_r and
// interp_minmod, api/cfdv0_solver.h:310-370): flux = +1 reconstructs from P,
// -1 from N.
template <typename T, int D>
__device__ __forceinline__ T minmod_interp(T cp, T ap, const T* grad, const T* d, T w, T flux) {
    const T gradf = ap - cp + T(1.0e-30);
    T gradcf = T(0);
#pragma unroll
    for (int k = 0; k < D; ++k) gradcf += d[k] * grad[k];
    T r;
    if (fabs(gradcf) >= T(1000) * fabs(gradf))
        r = T(2000) * (gradcf < T(0) ? T(-1) : T(1)) * (gradf < T(0) ? T(-1) : T(1)) - T(1);
    else
        r = T(2) * (gradcf / gradf) - T(1);
    T lim = (T(1) < r) ? T(1) : r;
    lim = (lim < T(0)) ? T(0) : lim;
    const T weight = lim * w + (T(1) - lim) * (T(1) + flux) * T(0.5);
    return weight * cp + (T(1) - weight) * ap;
}

// AUSM+ fifth-order pressure polynomials (p5Pos / p5Neg, src/cfd_v0.cpp:1863-1895).
template <typename T>
__device__ __forceinline__ T p5pos(T M, T alpha) {
    const T M2Pos = T(0.25) * (M + T(1)) * (M + T(1));
    const T M2Neg = T(-0.25) * (M - T(1)) * (M - T(1));
    if (fabs(M) < T(1)) return M2Pos * ((T(2) - M) - T(16) * alpha * M * M2Neg);
    return T(0.5) * (M + fabs(M)) / M;
}

template <typename T>
__device__ __forceinline__ T p5neg(T M, T alpha) {
    const T M2Pos = T(0.25) * (M + T(1)) * (M + T(1));
    const T M2Neg = T(-0.25) * (M - T(1)) * (M - T(1));
    if (fabs(M) < T(1)) return M2Neg * ((T(-2) - M) + T(16) * alpha * M * M2Pos);
    return T(0.5) * (M - fabs(M)) / M;
}

// Ghost state qv of ghost g from the conservative state qi of its interior
// cell (FP64): the boundary condition of set_boundary_conditions
// (src/cfd_v0.cpp:1009-1221).
template <typename T, int D>
__device__ __forceinline__ void ghost_bc(const Args<T>& a, int g, const double* qi, double* qv) {
    constexpr int NQ = D + 2;
    const int kind = a.gKind[g];
    if (kind == 1) {  // wall: mirror the momentum
        qv[0] = qi[0];
#pragma unroll
        for (int k = 0; k < D; ++k) qv[k + 1] = -qi[k + 1];
        qv[D + 1] = qi[D + 1];
    } else if (kind >= 2 && kind <= 4) {
        bool inlet = (kind == 2);
        if (kind == 4) inlet = (double)a.S[a.gFace[g]] <= 0.0;  // free stream along +x enters
        const double rhoInt = qi[0];
        double Uint[D], um2 = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            Uint[k] = qi[k + 1] / rhoInt;
            um2 += Uint[k] * Uint[k];
        }
        const double pInt = (qi[D + 1] - 0.5 * um2 * rhoInt) * a.gm1;
        if (inlet) {
            const double TInt = pInt * a.Rinv / rhoInt;
            const double rhoExt = rhoInt * TInt / a.TInf;
            double ue2 = 0.0;
#pragma unroll
            for (int k = 0; k < D; ++k) ue2 += a.UInf[k] * a.UInf[k];
            const double EExt = pInt / (rhoExt * a.gm1) + 0.5 * ue2;
            qv[0] = rhoExt;
#pragma unroll
            for (int k = 0; k < D; ++k) qv[k + 1] = rhoExt * a.UInf[k];
            qv[D + 1] = rhoExt * EExt;
        } else {
            const double rhoExt = rhoInt * a.pInf / pInt;
            const double EExt = a.pInf / (rhoExt * a.gm1) + 0.5 * um2;
            qv[0] = rhoExt;
#pragma unroll
            for (int k = 0; k < D; ++k) qv[k + 1] = rhoExt * Uint[k];
            qv[D + 1] = rhoExt * EExt;
        }
    } else {
        // Patches without a boundary condition keep a zero ghost state, as
        // in the reference (src/cfd_v0.cpp:406-416).
#pragma unroll
        for (int v = 0; v < NQ; ++v) qv[v] = 0.0;
    }
}

// Conservative state of cell, ghost or halo t in FP64 (FP64 path: q holds the
// state itself). A ghost's state is computed from its interior cell and
// stored into q; a halo's was copied in from its partition.
template <typename T, int D>
__device__ __forceinline__ void stage_state(const Args<T>& a, int t, double* qv) {
    constexpr int NQ = D + 2;
    if (t < a.nc || t >= a.nc + a.ng) {
#pragma unroll
        for (int v = 0; v < NQ; ++v) qv[v] = a.q[(size_t)v * a.nt + t];
        return;
    }
    const int g = t - a.nc;
    const int in = a.gCell[g];
    double qi[NQ];
#pragma unroll
    for (int v = 0; v < NQ; ++v) qi[v] = a.q[(size_t)v * a.nt + in];
    ghost_bc<T, D>(a, g, qi, qv);
#pragma unroll
    for (int v = 0; v < NQ; ++v) a.q[(size_t)v * a.nt + t] = qv[v];
}

// FP64 path: the primitives every face reads (1/rho, u, R psi = p/rho, c) of
// cell, ghost or halo t from its conservative state qv (compute_Rpsi,
// api/cfdv0_solver.h:252-261).
template <int D>
__device__ __forceinline__ void prims64(const Args<double>& a, int t, const double* qv) {
    const size_t nt = (size_t)a.nt;
    const double rinv = rcp64(qv[0]);
    double s = qv[1] * qv[1];
#pragma unroll
    for (int k = 1; k < D; ++k) s += qv[k + 1] * qv[k + 1];
    const double Rpsi = a.gm1 * (qv[D + 1] - 0.5 * s * rinv) * rinv;
    a.prim[t] = rinv;
#pragma unroll
    for (int k = 0; k < D; ++k) a.prim[(size_t)(1 + k) * nt + t] = qv[k + 1] * rinv;
    a.prim[(size_t)(D + 1) * nt + t] = Rpsi;
    if (a.primC) a.prim[(size_t)(D + 2) * nt + t] = sqrt(a.gamma * Rpsi);   // read by M2AUSM only
}

// FP64 path: the states and primitives of the boundary ghosts of cell c from
// its conservative state qc (those k_prep computes for the next stage).
template <int D>
__device__ __forceinline__ void ghosts_of64(const Args<double>& a, int c, const double* qc) {
    constexpr int NQ = D + 2;
    const size_t nt = (size_t)a.nt;
    for (int e = a.cfOff[c]; e < a.cfOff[c + 1]; ++e) {
        const int code = a.cfList[e];
        if (code < 0) continue;
        const int j = a.fN[code];
        if (j < a.nc || j >= a.nc + a.ng) continue;
        double qv[NQ];
        ghost_bc<double, D>(a, j - a.nc, qc, qv);
#pragma unroll
        for (int v = 0; v < NQ; ++v) a.q[(size_t)v * nt + j] = qv[v];
        prims64<D>(a, j, qv);
    }
}

// FP64 path: gather of the face rhs of cell c, sponge source and low-storage
// RK update (src/cfd_v0.cpp:2800-2822). The rhs are summed in ascending face
// order (the order in which the reference's scatter reaches the cell); the
// sum is the cell residual RES. PRIM: the cell also writes the next stage's
// primitives from the registers it holds, and (a.cellGhosts) the next stage's
// states and primitives of its boundary ghosts -- a ghost depends on its
// interior cell only -- so that no preparation pass runs between the stages.
template <typename T, int D, bool RES, bool PRIM = false>
__device__ __forceinline__ void update_cell(const Args<T>& a, int c, double Ak, double Bk, double dt, int first) {
    constexpr int NQ = D + 2;
    const size_t nt = (size_t)a.nt, nf = (size_t)a.nf, nc = (size_t)a.nc;
    double qv[NQ];
#pragma unroll
    for (int v = 0; v < NQ; ++v) qv[v] = a.q[v * nt + c];
    T sum[NQ];
#pragma unroll
    for (int v = 0; v < NQ; ++v) sum[v] = T(0);
    const int e0 = a.cfOff[c], e1 = a.cfOff[c + 1];
    constexpr int W = kEllWidth<D>;
    if (e1 - e0 <= W) {
        // every face index of the cell, then every rhs value, in flight at
        // once; summed in the same (ascending face) order as the loop below
        int code[W];
#pragma unroll
        for (int k = 0; k < W; ++k) code[k] = e0 + k < e1 ? a.cfList[e0 + k] : kEllPad;
        // The face's sign (+ where c is P, - where N) goes on the value as a
        // sign-bit flip on the integer pipe, so each entry costs one FP64 add
        // (a - b is a + (-b) in IEEE arithmetic: the same bits)
        T fl[W][NQ];
#pragma unroll
        for (int k = 0; k < W; ++k) {
            const int f = code[k] >= 0 ? code[k] : ~code[k];
#pragma unroll
            for (int v = 0; v < NQ; ++v) {
                const T x = code[k] != kEllPad ? a.flux[v * nf + f] : T(0);
                fl[k][v] = code[k] >= 0 ? x : neg_bits(x);
            }
        }
#pragma unroll
        for (int k = 0; k < W; ++k) {
            if (code[k] == kEllPad) continue;
#pragma unroll
            for (int v = 0; v < NQ; ++v) sum[v] += fl[k][v];
        }
    } else {
        for (int e = e0; e < e1; ++e) {
            const int code = a.cfList[e];
            if (code >= 0) {
#pragma unroll
                for (int v = 0; v < NQ; ++v) sum[v] += a.flux[v * nf + code];
            } else {
                const int f = ~code;
#pragma unroll
                for (int v = 0; v < NQ; ++v) sum[v] -= a.flux[v * nf + f];
            }
        }
    }
    double acc[NQ];
    bool finite = true;
    const double dtvi = dt * a.volInv[c];
#pragma unroll
    for (int v = 0; v < NQ; ++v) acc[v] = (first ? 0.0 : Ak * a.dq[v * nc + c]) + dtvi * (double)sum[v];
    const double sg = a.sponge[c];
    if (sg != 0.0) {
        acc[0] += dt * sg * (a.rhoInf - qv[0]);
#pragma unroll
        for (int k = 0; k < D; ++k) acc[k + 1] += dt * sg * (a.rhoInf * a.UInf[k] - qv[k + 1]);
        acc[D + 1] += dt * sg * (a.rhoInf * a.EInf - qv[D + 1]);
    }
    double qn[NQ];
#pragma unroll
    for (int v = 0; v < NQ; ++v) {
        a.dq[v * nc + c] = acc[v];
        qn[v] = qv[v] + Bk * acc[v];
        finite = finite && finite_bits(qn[v]);
        a.q[v * nt + c] = qn[v];
        if (RES) a.res[v * nc + c] = (double)sum[v];
    }
    if (!finite) atomicOr(a.flag, 1);
    if constexpr (PRIM) {
        prims64<D>(a, c, qn);
        if (a.cellGhosts && a.cellGhosts[c]) ghosts_of64<D>(a, c, qn);
    }
}

}  // namespace dev
}  // namespace lfm
