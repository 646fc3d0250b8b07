// FP32-bulk form of the time step: face fluxes, limiter, residual sums and
// the RK increment register dq in FP32; the accumulation of the conserved
// state, boundary ghost states, geometry precompute and the dt reduction in
// FP64.
//
// Perturbation form. The FP64 state is stored as its deviation from a
// constant reference state q_ref = (rho_inf, rho_inf U_inf, rho_inf E_inf):
// q' = q - q_ref (exact differences of nearby numbers, and no cancellation
// when it is rounded to FP32). Every FP32 quantity is a perturbation too:
// r' = rho - rho_inf, m' = rho u - rho_inf U_inf, u' = u - U_inf and
// R psi' = p/rho - p_ref/rho_inf, derived by expressions whose terms are all
// perturbation-sized. Each face rhs is F(q_f).S - F(q_ref).S. The
// reference-state flux through the faces of a cell sums to
// F(q_ref).(sum_f S_f) = 0 because the face vectors of a closed cell cancel,
// so dropping it leaves every cell residual unchanged while FP32 rounding only
// ever scales perturbations. Evaluated on absolute values, FP32 would round
// the pressure (~1e5 Pa) by ~1e-2 Pa per face, the size of an acoustic wave;
// here the rounding is ~1e-7 of the perturbation.
//
// GB300 runs FP64 instructions (conversions included) at about two per clock
// per SM, so the FP64 work is kept to one FMA per component, the
// accumulation of the conserved state: conversions between FP32 and FP64 run on the
// integer pipes (fp_convert.cuh), and the update kernel derives the next
// stage's primitives from the new state while it holds it in registers
// (prims32), so a stage reads q' once. The primitive formulas use explicitly
// rounded operations, so they give the same bits wherever they are inlined.
//
// The schemes are those of the FP64 kernels (solver_kernels.cu), which follow
// the reference (src/cfd_v0.cpp:1896-2822): M1 as the central flux its
// Kurganov-Tadmor formula reduces to, M2 and M2AUSM as written, with the
// perfect-gas enthalpy h = e + p/rho = gamma/(gamma-1) R psi.
#pragma once

#include "fp_convert.cuh"
#include "solver_device.cuh"

namespace lfm {
namespace dev {

// Row of the FP32 primitive array (rho', m'[D], u'[D], R psi', c).
template <int D>
struct PRow {
    static constexpr int r = 0, m = 1, u = 1 + D, Rpsi = 1 + 2 * D, c = 2 + 2 * D;
};

__device__ __forceinline__ float ld(const float* p, int row, size_t nt, int i) { return p[(size_t)row * nt + i]; }

// p - p_ref of a state with perturbations r', R psi':
// rho R psi - rho_inf R psi_inf = rho_inf R psi' + r' (R psi_inf + R psi').
__device__ __forceinline__ float pressure_dev(const RefState32& R, float r, float Rpsi) {
    return R.rho * Rpsi + r * (R.Rpsi + Rpsi);
}

// ---------------------------------------------------------------------------
// prims32: FP32 primitives of interior cell t from its FP64 perturbation state
// qp = q - q_ref. Explicitly rounded operations only (no contraction), so the
// preparation and update kernels produce identical bits.
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void prims32(const Args<float>& a, int t, const double* qp, float* dst) {
    using P = PRow<D>;
    const RefState32& R = a.ref;
    const size_t nt = (size_t)a.nt;
    const float r = f64_to_f32(qp[0]);
    float m[D];
#pragma unroll
    for (int k = 0; k < D; ++k) m[k] = f64_to_f32(qp[k + 1]);
    const float E = f64_to_f32(qp[D + 1]);
    const float rho = __fadd_rn(R.rho, r);
    const float rinv = __frcp_rn(rho);
    float u[D], Uu = 0.0f, uu = 0.0f, U2 = 0.0f;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        u[k] = __fmul_rn(__fmaf_rn(-R.U[k], r, m[k]), rinv);   // (m' - U_inf r') / rho
        Uu = __fmaf_rn(R.U[k], u[k], Uu);
        uu = __fmaf_rn(u[k], u[k], uu);
        U2 = __fmaf_rn(R.U[k], R.U[k], U2);
    }
    // kinetic energy: rho|u|^2/2 - rho_inf|U_inf|^2/2 = r'|U_inf|^2/2 + rho (U_inf.u' + |u'|^2/2)
    const float K = __fmaf_rn(rho, __fmaf_rn(0.5f, uu, Uu), __fmul_rn(__fmul_rn(0.5f, r), U2));
    const float p = __fmul_rn(R.gm1, __fsub_rn(E, K));            // p - p_ref
    const float Rpsi = __fmul_rn(__fmaf_rn(-R.Rpsi, r, p), rinv);  // p/rho - p_ref/rho_inf
    dst[(size_t)P::r * nt + t] = r;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        dst[(size_t)(P::m + k) * nt + t] = m[k];
        dst[(size_t)(P::u + k) * nt + t] = u[k];
    }
    dst[(size_t)P::Rpsi * nt + t] = Rpsi;
    dst[(size_t)P::c * nt + t] = __fsqrt_rn(__fmul_rn(R.gamma, __fadd_rn(R.Rpsi, Rpsi)));
}

// ---------------------------------------------------------------------------
// ghost32: boundary state of ghost g (FP64) from the absolute state qi of its
// interior cell, and its FP32 primitives. A ghost state can lie far from the
// free stream (a wall mirrors the momentum, u' = -2 U_inf - u'), where the
// FP32 kinetic-energy difference of prims32 would cancel; ghosts are few, so
// theirs is FP64.
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void ghost32(const Args<float>& a, int g, const double* qi, float* dst) {
    constexpr int NQ = D + 2;
    using P = PRow<D>;
    const size_t nt = (size_t)a.nt;
    const int t = a.nc + g;
    double qv[NQ];
    ghost_bc<float, D>(a, g, qi, qv);
    const double rinv = 1.0 / qv[0];
    double ke = 0.0;
    dst[(size_t)P::r * nt + t] = (float)(qv[0] - a.qRef[0]);
#pragma unroll
    for (int k = 0; k < D; ++k) {
        dst[(size_t)(P::m + k) * nt + t] = (float)(qv[k + 1] - a.qRef[k + 1]);
        dst[(size_t)(P::u + k) * nt + t] = (float)(qv[k + 1] * rinv - a.UInf[k]);
        ke += qv[k + 1] * qv[k + 1];
    }
    const double p = a.gm1 * (qv[D + 1] - 0.5 * ke * rinv);
    const float Rpsi = (float)(p * rinv - a.pRef / a.qRef[0]);
    dst[(size_t)P::Rpsi * nt + t] = Rpsi;
    dst[(size_t)P::c * nt + t] = sqrtf(a.ref.gamma * (a.ref.Rpsi + Rpsi));
}

// ---------------------------------------------------------------------------
// prep32: primitives of cell or halo t from the stored perturbation state, or,
// for a ghost, its boundary state (FP64, from the interior cell) and primitives.
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void prep32(const Args<float>& a, int t) {
    constexpr int NQ = D + 2;
    using P = PRow<D>;
    const size_t nt = (size_t)a.nt;
    if (t < a.nc || t >= a.nc + a.ng) {
        double qp[NQ];
#pragma unroll
        for (int v = 0; v < NQ; ++v) qp[v] = a.q[(size_t)v * nt + t];
        prims32<D>(a, t, qp, a.prim);
        return;
    }
    const int g = t - a.nc;
    const int in = a.gCell[g];
    double qi[NQ];
#pragma unroll
    for (int v = 0; v < NQ; ++v) qi[v] = a.q[(size_t)v * nt + in] + a.qRef[v];
    ghost32<D>(a, g, qi, a.prim);
}

// ---------------------------------------------------------------------------
// update32: gather of the face rhs of cell c in ascending face order (the
// reference's scatter order; the sum is the cell residual RES), sponge source
// and low-storage RK update of the FP64 perturbation state
// (src/cfd_v0.cpp:2800-2822), then the next stage's primitives of the cell.
// The increment dt/V RES, the sponge source and the RK register
// dq = A dq + increment are FP32: dq restarts at every step (A = 0 in stage
// 0) and holds only that step's increments, so its rounding is that of the
// FP32 rhs it sums. The conserved state accumulates in FP64,
// q' = q' + B dq (one FP64 FMA per component), so rounding does not build up
// over the steps. The sponge pulls q towards q_ref:
// dt sigma (q_ref - q) = -dt sigma q'.
// GH: the cell also writes the next stage's state of its boundary ghosts
// (a ghost depends on its interior cell only), so no preparation pass over
// the ghosts is needed; the values are those prep32 computes.
// ---------------------------------------------------------------------------
// ghosts_of32: the FP64 states and FP32 primitives of the boundary ghosts of
// cell c from its perturbation state qp (those prep32 computes).
template <int D>
__device__ __forceinline__ void ghosts_of32(const Args<float>& a, int c, const double* qp, float* dst) {
    constexpr int NQ = D + 2;
    double qa[NQ];
#pragma unroll
    for (int v = 0; v < NQ; ++v) qa[v] = qp[v] + a.qRef[v];
    for (int e = a.cfOff[c]; e < a.cfOff[c + 1]; ++e) {
        const int code = a.cfList[e];
        if (code < 0) continue;
        const int j = a.fN[code];
        if (j >= a.nc && j < a.nc + a.ng) ghost32<D>(a, j - a.nc, qa, dst);
    }
}

// gather32: the face rhs sum of cell c (ascending face order).
template <int D>
__device__ __forceinline__ void gather32(const Args<float>& a, int c, float* sum) {
    constexpr int NQ = D + 2;
    const size_t nf = (size_t)a.nf;
#pragma unroll
    for (int v = 0; v < NQ; ++v) sum[v] = 0.0f;
    for (int e = a.cfOff[c]; e < a.cfOff[c + 1]; ++e) {
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

// gather32_ell: gather32 through the fixed-width table. Every face index of
// the cell is loaded at once (coalesced rows), then every flux value, so the
// gather costs two memory round trips instead of one per face; the sum runs
// in the same (ascending face) order, so it has gather32's bits.
template <int D>
__device__ __forceinline__ void gather32_ell(const Args<float>& a, int c, float* sum) {
    constexpr int NQ = D + 2, W = kEllWidth<D>;
    const size_t nf = (size_t)a.nf, nc = (size_t)a.nc;
    int code[W];
#pragma unroll
    for (int k = 0; k < W; ++k) code[k] = a.cfEll[k * nc + c];
    float fl[W][NQ];
#pragma unroll
    for (int k = 0; k < W; ++k) {
        const int f = code[k] >= 0 ? code[k] : ~code[k];
#pragma unroll
        for (int v = 0; v < NQ; ++v) {   // the face's sign as a sign-bit flip: one add per entry
            const float x = code[k] != kEllPad ? a.flux[v * nf + f] : 0.0f;
            fl[k][v] = code[k] >= 0 ? x : neg_bits(x);
        }
    }
#pragma unroll
    for (int v = 0; v < NQ; ++v) sum[v] = 0.0f;
#pragma unroll
    for (int k = 0; k < W; ++k) {
        if (code[k] == kEllPad) continue;
#pragma unroll
        for (int v = 0; v < NQ; ++v) sum[v] += fl[k][v];
    }
}

// The cell's own values the update reads, loaded before its rhs gather so
// that they are in flight together with it.
template <int D>
struct CellIn32 {
    double qp[D + 2];   // q'
    float dq[D + 2];
    float vi, sg;       // 1/V, sponge sigma
};

template <int D>
__device__ __forceinline__ void load_cell32(const Args<float>& a, int c, int first, CellIn32<D>& in) {
    const size_t nt = (size_t)a.nt, nc = (size_t)a.nc;
#pragma unroll
    for (int v = 0; v < D + 2; ++v) {
        in.qp[v] = a.q[v * nt + c];
        in.dq[v] = first ? 0.0f : a.dq[v * nc + c];
    }
    in.vi = a.volInv32[c];
    in.sg = a.sponge[c];
}

// apply32: the update of cell c from its rhs sum and its loaded values
// (see update32).
template <int D, bool RES, bool GH>
__device__ __forceinline__ void apply32(const Args<float>& a, int c, const float* sum, const CellIn32<D>& in,
                                        double Ak, double Bk, double dt, float dt32, int first) {
    constexpr int NQ = D + 2;
    const size_t nt = (size_t)a.nt, nc = (size_t)a.nc;
    const float dtvi = __fmul_rn(dt32, in.vi);
    const float sg = in.sg;
    const float dts = -__fmul_rn(dt32, sg);
    const float A32 = __double2float_rn(Ak);
    double qn[NQ];
    bool finite = true;
#pragma unroll
    for (int v = 0; v < NQ; ++v) {
        const float inc = __fmul_rn(dtvi, sum[v]);
        float acc = first ? inc : __fmaf_rn(A32, in.dq[v], inc);
        const double qp = in.qp[v];
        if (sg != 0.0f) acc = __fmaf_rn(dts, f64_to_f32(qp), acc);
        a.dq[v * nc + c] = acc;
        qn[v] = fma(Bk, f32_to_f64(acc), qp);
        a.q[v * nt + c] = qn[v];
        finite = finite && isfinite(sum[v]);
        if (RES) a.res[v * nc + c] = f32_to_f64(sum[v]);
    }
    if (!finite) atomicOr(a.flag, 1);
    prims32<D>(a, c, qn, a.primW);
    if (GH && a.cellGhosts[c]) ghosts_of32<D>(a, c, qn, a.primW);
}

template <int D, bool RES, bool GH = false, bool ELL = false>
__device__ __forceinline__ void update32(const Args<float>& a, int c, double Ak, double Bk, double dt,
                                         float dt32, int first) {
    CellIn32<D> in;
    load_cell32<D>(a, c, first, in);
    float sum[D + 2];
    if (ELL) gather32_ell<D>(a, c, sum);
    else gather32<D>(a, c, sum);
    apply32<D, RES, GH>(a, c, sum, in, Ak, Bk, dt, dt32, first);
}

// A new state: q' = q - q_ref of cell c from a caller's absolute state q
// ([nq][stride] doubles), its primitives and, where the update keeps them
// (a.cellGhosts), its boundary ghosts' -- the values the preparation pass
// derives from the stored q', from registers.
template <int D>
__device__ __forceinline__ void set_state32(const Args<float>& a, const double* q, int64_t stride, int c) {
    double qp[D + 2];
#pragma unroll
    for (int v = 0; v < D + 2; ++v) {
        qp[v] = q[(size_t)v * stride + c] - a.qRef[v];
        a.q[(size_t)v * a.nt + c] = qp[v];
    }
    prims32<D>(a, c, qp, a.prim);
    if (a.cellGhosts && a.cellGhosts[c]) ghosts_of32<D>(a, c, qp, a.prim);
}

// Perturbation state q' = q - q_ref of cells [0, n) from a caller's absolute
// state q ([nq][stride] doubles).
template <int D>
__device__ __forceinline__ void to_perturbation(const Args<float>& a, const double* q, int64_t stride, int c) {
#pragma unroll
    for (int v = 0; v < D + 2; ++v) a.q[(size_t)v * a.nt + c] = q[(size_t)v * stride + c] - a.qRef[v];
}

// ---------------------------------------------------------------------------
// grad32: Gauss gradients of rho', p' and u' (those of rho, p and u up to
// the reference state's closed-cell sum) for M2AUSM's minmod reconstruction.
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void grad32(const Args<float>& a, int c) {
    using P = PRow<D>;
    const RefState32& R = a.ref;
    const size_t nt = (size_t)a.nt, nf = (size_t)a.nf;
    float gr[D], gp[D], gu[D][D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        gr[k] = gp[k] = 0.0f;
#pragma unroll
        for (int l = 0; l < D; ++l) gu[k][l] = 0.0f;
    }
    const float vi = a.volInv32[c];
    // the cell's own primitives once; the cell across each face from the
    // face list's neighbour column (P and N sides kept for the interpolation)
    float cu[D];
#pragma unroll
    for (int k = 0; k < D; ++k) cu[k] = ld(a.prim, P::u + k, nt, c);
    const float cr = ld(a.prim, P::r, nt, c);
    const float cpr = pressure_dev(R, cr, ld(a.prim, P::Rpsi, nt, c));
    for (int e = a.cfOff[c]; e < a.cfOff[c + 1]; ++e) {
        const int code = a.cfList[e];
        const int o = a.cfNbr[e];
        const bool own = code >= 0;   // c is the face's P side
        const int f = own ? code : ~code;
        const float w = a.w[f];
        float ou[D];
#pragma unroll
        for (int k = 0; k < D; ++k) ou[k] = ld(a.prim, P::u + k, nt, o);
        const float orr = ld(a.prim, P::r, nt, o);
        const float opr = pressure_dev(R, orr, ld(a.prim, P::Rpsi, nt, o));
        float so[D], uu[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const float Sk = a.S[(size_t)k * nf + f];
            so[k] = own ? Sk * vi : -Sk * vi;
            uu[k] = own ? interp(w, cu[k], ou[k]) : interp(w, ou[k], cu[k]);
        }
        const float ri = own ? cr : orr, rj = own ? orr : cr;
        const float pi = own ? cpr : opr;
        const float pj = own ? opr : cpr;
        const float rho = interp(w, ri, rj);
        const float p = interp(w, pi, pj);
#pragma unroll
        for (int x = 0; x < D; ++x) {
            gp[x] += p * so[x];
            gr[x] += rho * so[x];
#pragma unroll
            for (int b = 0; b < D; ++b) gu[b][x] += uu[b] * so[x];
        }
    }
#pragma unroll
    for (int k = 0; k < D; ++k) {
        a.grad[(size_t)k * nt + c] = gr[k];
        a.grad[(size_t)(D + k) * nt + c] = gp[k];
#pragma unroll
        for (int l = 0; l < D; ++l) a.grad[(size_t)(2 * D + k * D + l) * nt + c] = gu[k][l];
    }
}

// ---------------------------------------------------------------------------
// vis32: dudx and dTdx from u' and T', sigmaU = (U_inf + u') . tau.
// ---------------------------------------------------------------------------
// LES compiles in the Smagorinsky SGS stress (cases with a.smagC).
template <int D, bool LES = false>
__device__ __forceinline__ void vis32(const Args<float>& a, int c) {
    using P = PRow<D>;
    const size_t nt = (size_t)a.nt, nf = (size_t)a.nf;
    float g[D][D], gT[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        gT[k] = 0.0f;
#pragma unroll
        for (int l = 0; l < D; ++l) g[k][l] = 0.0f;
    }
    const float vi = a.volInv32[c];
    const float Rinv = a.ref.Rinv;
    // the cell's own primitives once; the cell across each face from the
    // face list's neighbour column (P and N sides kept for the interpolation)
    float cu[D];
#pragma unroll
    for (int k = 0; k < D; ++k) cu[k] = ld(a.prim, P::u + k, nt, c);
    const float cR = ld(a.prim, P::Rpsi, nt, c);
    for (int e = a.cfOff[c]; e < a.cfOff[c + 1]; ++e) {
        const int code = a.cfList[e];
        const int o = a.cfNbr[e];
        const bool own = code >= 0;   // c is the face's P side
        const int f = own ? code : ~code;
        const float w = a.w[f];
        float so[D], fU[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const float Sk = a.S[(size_t)k * nf + f];
            const float ouk = ld(a.prim, P::u + k, nt, o);
            so[k] = own ? Sk * vi : -Sk * vi;
            fU[k] = own ? interp(w, cu[k], ouk) : interp(w, ouk, cu[k]);
        }
        const float oR = ld(a.prim, P::Rpsi, nt, o);
        const float fT = (own ? interp(w, cR, oR) : interp(w, oR, cR)) * Rinv;
#pragma unroll
        for (int x = 0; x < D; ++x) {
#pragma unroll
            for (int y = 0; y < D; ++y) g[x][y] += fU[x] * so[y];
            gT[x] += fT * so[x];
        }
    }
    const float mu = a.ref.mu;
    float tau[D][D];
    stress<float, D>(g, mu, tau);
    float U[D];
#pragma unroll
    for (int k = 0; k < D; ++k) U[k] = a.ref.U[k] + cu[k];
#pragma unroll
    for (int x = 0; x < D; ++x) {
#pragma unroll
        for (int y = 0; y < D; ++y) a.V[(size_t)(x * D + y) * nt + c] = g[x][y];
        a.V[(size_t)(D * D + x) * nt + c] = gT[x];
        a.V[(size_t)(D * D + D + x) * nt + c] = dotv<float, D>(U, tau[x]);
    }
    if (LES && a.smagC) {   // Smagorinsky LES: the cell's SGS stress
        float sg[D][D];
        sgs_stress<float, D>(g, a.smagC[c], sg);
#pragma unroll
        for (int x = 0; x < D; ++x)
#pragma unroll
            for (int y = 0; y < D; ++y) a.V[(size_t)(kVisRows<D> + x * D + y) * nt + c] = sg[x][y];
    }
}

// d(M) = p5pos(M) - p5neg(M) is, for |M| < 1, the odd polynomial
// (3M - M^3)/2 + 2 alpha M (1 - M^2)^2. Its divided difference
// (d(a) - d(b)) / (a - b), so that d(MN) - d(MP) is formed as a product with
// MN - MP instead of a difference of two O(1) numbers.
__device__ __forceinline__ float p5diff_dd(float a, float b, float alpha) {
    const float s2 = a * a + a * b + b * b;                                   // (a^3 - b^3)/(a - b)
    const float s4 = a * a * a * a + a * a * a * b + a * a * b * b + a * b * b * b + b * b * b * b;
    return 1.5f - 0.5f * s2 + 2.0f * alpha * (1.0f - 2.0f * s2 + s4);
}

// ---------------------------------------------------------------------------
// flux32: perturbation rhs of face f, F(q_f).S - F(q_ref).S, plus the
// viscous terms (linear in the gradients, so unchanged in form).
// ---------------------------------------------------------------------------
// VIS = false compiles the viscous terms out (for callers that know mu = 0).
// EARLYV loads the viscous rows of both cells and the face's viscous geometry
// together with the primitives, so the gathers overlap instead of following
// one another (2 x 8 more live values in 2D, 2 x 15 in 3D): the stand-alone
// flux kernel (3D flux 4.05 -> 3.43 ms per step on the 9.4M-cell wake, whose
// gathers come from HBM; 2 % in 2D, whose gathers hit L2). The fused kernels,
// whose registers other phases already fill, keep the late loads.
//
// face_rhs32_cells takes the face's cells i (P) and j (N) as arguments and
// reads every array through `a`: the solver's Args, or a view of the same
// rows staged in shared memory (the staged flux kernel, flux_staged_fp32.cu),
// which gives the same bits because only the addresses differ.
template <int D, int SCH, bool VIS, bool LES, bool EARLYV, class A>
__device__ __forceinline__ void face_rhs32_cells(const A& a, int f, int i, int j, float* rhs) {
    using P = PRow<D>;
    const RefState32& R = a.ref;
    const size_t nt = (size_t)a.nt, nf = (size_t)a.nf;
    const float w = a.w[f];
    float S[D];
#pragma unroll
    for (int k = 0; k < D; ++k) S[k] = a.S[(size_t)k * nf + f];
    const float ri = ld(a.prim, P::r, nt, i), rj = ld(a.prim, P::r, nt, j);
    float mi[D], mj[D], ui[D], uj[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        mi[k] = ld(a.prim, P::m + k, nt, i);
        mj[k] = ld(a.prim, P::m + k, nt, j);
        ui[k] = ld(a.prim, P::u + k, nt, i);
        uj[k] = ld(a.prim, P::u + k, nt, j);
    }
    const float Ri = ld(a.prim, P::Rpsi, nt, i), Rj = ld(a.prim, P::Rpsi, nt, j);
    constexpr bool early = VIS && EARLYV;
    constexpr int VR = early ? kVisRows<D> : 1;
    float Vi[VR], Vj[VR], eK[early ? D : 1], eLapc = 0.0f;
    if (early && a.ref.mu != 0.0f) {
#pragma unroll
        for (int k = 0; k < (early ? D : 1); ++k) eK[k] = a.K[(size_t)k * nf + f];
        eLapc = a.lapc[f];
        if (!a.fGhost[f]) {
#pragma unroll
            for (int r = 0; r < VR; ++r) {
                Vi[r] = a.V[(size_t)r * nt + i];
                Vj[r] = a.V[(size_t)r * nt + j];
            }
        }
    }
    // Face state: linear interpolation for M1, the mid-point for M2 / M2AUSM.
    const float wf = (SCH == kSchemeM1) ? w : 0.5f;
    const float rf = interp(wf, ri, rj);
    const float rinv = 1.0f / (R.rho + rf);
    float mf[D], uf[D];
    float mS = 0.0f, ufS = 0.0f, UrS = 0.0f, mrS = 0.0f;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        mf[k] = interp(wf, mi[k], mj[k]);
        uf[k] = (mf[k] - R.U[k] * rf) * rinv;      // u_f - U_inf with u_f = m_f / rho_f
        mS += mf[k] * S[k];
        ufS += uf[k] * S[k];
        UrS += R.U[k] * S[k];
        mrS += R.m[k] * S[k];
    }
    const float phi = UrS + ufS;                    // u_f . S
    const float Rf = interp(wf, Ri, Rj);
    float pf = pressure_dev(R, rf, Rf);             // rho_f R psi_f - p_ref
    float Hf;                                       // H - H_ref
    if (SCH == kSchemeM1) {
        // H_f = e_f + |u_f|^2/2 + R psi_f with e_f = R psi_f / (gamma - 1)
        float Uu = 0.0f, uu = 0.0f;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            Uu += R.U[k] * uf[k];
            uu += uf[k] * uf[k];
        }
        Hf = R.gh * Rf + Uu + 0.5f * uu;
    } else {
        // mean of the cells' H = gamma/(gamma-1) R psi + |u|^2/2
        float Hi = R.gh * Ri, Hj = R.gh * Rj;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            Hi += R.U[k] * ui[k] + 0.5f * ui[k] * ui[k];
            Hj += R.U[k] * uj[k] + 0.5f * uj[k] * uj[k];
        }
        Hf = 0.5f * (Hi + Hj);
    }
    if (SCH == kSchemeAUSM) {
        // shock sensor, minmod reconstructions and AUSM+ pressure dissipation
        // (src/cfd_v0.cpp:2288-2339) on the perturbation variables; minmod is
        // invariant under a common shift of both sides.
        const float cavg = 0.5f * (ld(a.prim, P::c, nt, i) + ld(a.prim, P::c, nt, j));
        float d[D];
#pragma unroll
        for (int k = 0; k < D; ++k) d[k] = a.d[(size_t)k * nf + f];
        float cdiv = 0.0f, ndiv = 0.0f, ccurl = 0.0f, ncurl = 0.0f, unPos = 0.0f, unNeg = 0.0f, dUn = 0.0f,
              norm = 0.0f;
#pragma unroll
        for (int x = 0; x < D; ++x) {
            cdiv += a.V[(size_t)(x * D + x) * nt + i];
            ndiv += a.V[(size_t)(x * D + x) * nt + j];
#pragma unroll
            for (int y = x + 1; y < D; ++y) {
                const float cc = a.V[(size_t)(x * D + y) * nt + i] - a.V[(size_t)(y * D + x) * nt + i];
                const float nn = a.V[(size_t)(x * D + y) * nt + j] - a.V[(size_t)(y * D + x) * nt + j];
                ccurl += cc * cc;
                ncurl += nn * nn;
            }
            float gi[D], gj[D];
#pragma unroll
            for (int y = 0; y < D; ++y) {
                gi[y] = a.grad[(size_t)(2 * D + x * D + y) * nt + i];
                gj[y] = a.grad[(size_t)(2 * D + x * D + y) * nt + j];
            }
            const float uP = minmod_interp<float, D>(ui[x], uj[x], gi, d, w, 1.0f);
            const float uN = minmod_interp<float, D>(ui[x], uj[x], gj, d, w, -1.0f);
            unPos += (R.U[x] + uP) * S[x];
            unNeg += (R.U[x] + uN) * S[x];
            dUn += (uN - uP) * S[x];
            norm += S[x] * S[x];
        }
        float ct = -(cdiv / sqrtf(cdiv * cdiv + ccurl + 4e-2f));
        ct = (ct < 0.0f) ? 0.0f : ct;
        float nt_ = -(ndiv / sqrtf(ndiv * ndiv + ncurl + 4e-2f));
        nt_ = (nt_ < 0.0f) ? 0.0f : nt_;
        const float theta = 0.5f * (ct + nt_);
        const float pi = pressure_dev(R, ri, Ri), pj = pressure_dev(R, rj, Rj);
        float gri[D], grj[D], gpi[D], gpj[D];
#pragma unroll
        for (int y = 0; y < D; ++y) {
            gri[y] = a.grad[(size_t)y * nt + i];
            grj[y] = a.grad[(size_t)y * nt + j];
            gpi[y] = a.grad[(size_t)(D + y) * nt + i];
            gpj[y] = a.grad[(size_t)(D + y) * nt + j];
        }
        const float rhoPos = R.rho + minmod_interp<float, D>(ri, rj, gri, d, w, 1.0f);
        const float rhoNeg = R.rho + minmod_interp<float, D>(ri, rj, grj, d, w, -1.0f);
        const float pPos = minmod_interp<float, D>(pi, pj, gpi, d, w, 1.0f);    // p - p_ref
        const float pNeg = minmod_interp<float, D>(pi, pj, gpj, d, w, -1.0f);
        const float Msq = (unPos * unPos + unNeg * unNeg) / (2.0f * cavg * cavg * norm);
        const float sc = 1.0f / (sqrtf(norm) * cavg);
        const float MPos = unPos * sc, MNeg = unNeg * sc;
        const float Minf = 0.2f;
        float mm = (Msq < Minf * Minf) ? Minf * Minf : Msq;
        mm = (mm < 1.0f) ? mm : 1.0f;
        const float M0 = sqrtf(mm);
        const float fa = M0 * (2.0f - M0);
        const float alpha = 3.0f * (5.0f * fa * fa - 4.0f) / 16.0f;
        const float ppP = p5pos(MPos, alpha), pnP = p5neg(MPos, alpha);
        const float ppN = p5pos(MNeg, alpha), pnN = p5neg(MNeg, alpha);
        const float dN = ppN - pnN, dP = ppP - pnP;
        const float dNdP = (fabsf(MPos) < 1.0f && fabsf(MNeg) < 1.0f) ? dUn * sc * p5diff_dd(MNeg, MPos, alpha)
                                                                       : dN - dP;
        // pNeg dN - pPos dP with p = p_ref + p'
        const float phalf = R.p * dNdP + pNeg * dN - pPos * dP;
        const float pu = -0.75f * ppP * pnN * (rhoPos + rhoNeg) * cavg * fa * dUn;
        pf += theta * (pu - 0.5f * phalf);
    }
    // F(q_f).S - F(q_ref).S
    rhs[0] = -mS;
#pragma unroll
    for (int k = 0; k < D; ++k) rhs[k + 1] = -(R.m[k] * ufS + mf[k] * phi + pf * S[k]);
    rhs[D + 1] = -(mS * R.H + (mrS + mS) * Hf);

    // Viscous face terms (src/cfd_v0.cpp:2682-2796), as in the FP64 kernel.
    const float mu = a.ref.mu;
    if (VIS && mu != 0.0f) {
        const float Rinv = a.ref.Rinv;
        const float Ti = Ri * Rinv, Tj = Rj * Rinv;   // T - T_ref
        const float lapc = early ? eLapc : a.lapc[f];
        float Kf[D], g[D][D], gT[D], sU[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            if constexpr (early) Kf[k] = eK[k];
            else Kf[k] = a.K[(size_t)k * nf + f];
        }
        if (!a.fGhost[f]) {
            auto vI = [&](int r) -> float {
                if constexpr (early) return Vi[r];
                else return a.V[(size_t)r * nt + i];
            };
            auto vJ = [&](int r) -> float {
                if constexpr (early) return Vj[r];
                else return a.V[(size_t)r * nt + j];
            };
#pragma unroll
            for (int x = 0; x < D; ++x) {
#pragma unroll
                for (int y = 0; y < D; ++y) g[x][y] = interp(w, vI(x * D + y), vJ(x * D + y));
                gT[x] = interp(w, vI(D * D + x), vJ(D * D + x));
                sU[x] = interp(w, vI(D * D + D + x), vJ(D * D + D + x));
            }
        } else {
            const float dinv = a.dinv[f];
            float dn[D], tau[D][D], Uf[D];
#pragma unroll
            for (int k = 0; k < D; ++k) dn[k] = a.dnorm[(size_t)k * nf + f];
#pragma unroll
            for (int x = 0; x < D; ++x) {
#pragma unroll
                for (int y = 0; y < D; ++y) g[x][y] = (uj[x] - ui[x]) * dn[y] * dinv;
                gT[x] = (Tj - Ti) * dn[x] * dinv;
                Uf[x] = R.U[x] + interp(w, ui[x], uj[x]);
            }
            stress<float, D>(g, mu, tau);
#pragma unroll
            for (int x = 0; x < D; ++x) sU[x] = dotv<float, D>(Uf, tau[x]);
        }
        float tr = g[0][0];
#pragma unroll
        for (int x = 1; x < D; ++x) tr += g[x][x];
        const float dsum = -(mu * 2.0f / 3.0f) * tr;
        const float kc = a.ref.kcond;
#pragma unroll
        for (int x = 0; x < D; ++x) {
            float gtS = g[0][x] * S[0];
#pragma unroll
            for (int y = 1; y < D; ++y) gtS += g[y][x] * S[y];
            rhs[x + 1] += mu * gtS + dsum * S[x] + mu * (lapc * (uj[x] - ui[x]) + dotv<float, D>(Kf, g[x]));
        }
        rhs[D + 1] += dotv<float, D>(sU, S) + kc * (lapc * (Tj - Ti) + dotv<float, D>(Kf, gT));
        if (LES && a.smagC && !a.fGhost[f]) {   // Smagorinsky LES, as in the FP64 kernel
#pragma unroll
            for (int x = 0; x < D; ++x) {
                float s = 0.0f;
#pragma unroll
                for (int y = 0; y < D; ++y)
                    s += interp(w, a.V[(size_t)(kVisRows<D> + x * D + y) * nt + i],
                                a.V[(size_t)(kVisRows<D> + x * D + y) * nt + j]) *
                         S[y];
                rhs[x + 1] += s;
            }
        }
    }
}

template <int D, int SCH, bool VIS = true, bool LES = false, bool EARLYV = false>
__device__ __forceinline__ void face_rhs32(const Args<float>& a, int f, float* rhs) {
    face_rhs32_cells<D, SCH, VIS, LES, EARLYV>(a, f, a.fP[f], a.fN[f], rhs);
}

template <int D, int SCH, bool VIS = true, bool LES = false, bool EARLYV = false>
__device__ __forceinline__ void flux32(const Args<float>& a, int f) {
    float rhs[D + 2];
    face_rhs32<D, SCH, VIS, LES, EARLYV>(a, f, rhs);
    const size_t nf = (size_t)a.nf;
#pragma unroll
    for (int v = 0; v < D + 2; ++v) a.flux[(size_t)v * nf + f] = rhs[v];
}

// ---------------------------------------------------------------------------
// flux32_cell: the rhs of the faces cell c owns (it is their P side), one
// after another in face order. The cell's own primitive and viscous rows are
// read once, into registers, for all its faces (a face-per-thread kernel
// reads them once per face); the cell across each face is read per face, its
// index one face ahead. face_rhs32_cells sees the rows through a view of the
// registers (side 0 = P, 1 = N), so the rhs keeps flux32's bits. M1 / M2
// without the LES terms (whose extra rows the view does not carry).
// ---------------------------------------------------------------------------
template <int D>
struct CellFaceView32 {
    const RefState32& ref;
    float prim[2 * (2 * D + 2)];   // [row][side]: rho', m'[D], u'[D], R psi'
    float V[2 * kVisRows<D>];      // [row][side]: dudx, dTdx, sigmaU
    const float *S, *d, *w, *K, *lapc, *dinv, *dnorm;
    const uint8_t* fGhost;
    const float *grad, *smagC;
    int nt, nf;
};

template <int D, int SCH>
__device__ __forceinline__ void flux32_cell(const Args<float>& a, int c) {
    static_assert(SCH != kSchemeAUSM, "the cell-centred flux carries no sound speed or gradients");
    const int f0 = a.fOwn[c], f1 = a.fOwn[c + 1];
    if (f0 >= f1) return;
    const size_t nt = (size_t)a.nt, nf = (size_t)a.nf;
    CellFaceView32<D> v{a.ref};
    v.S = a.S;
    v.d = a.d;
    v.w = a.w;
    v.K = a.K;
    v.lapc = a.lapc;
    v.dinv = a.dinv;
    v.dnorm = a.dnorm;
    v.fGhost = a.fGhost;
    v.grad = nullptr;
    v.smagC = nullptr;
    v.nt = 2;
    v.nf = a.nf;
    const bool vis = a.ref.mu != 0.0f;
#pragma unroll
    for (int r = 0; r < 2 * D + 2; ++r) v.prim[2 * r] = a.prim[(size_t)r * nt + c];
    if (vis) {
#pragma unroll
        for (int r = 0; r < kVisRows<D>; ++r) v.V[2 * r] = a.V[(size_t)r * nt + c];
    }
    int jn = a.fN[f0];
    for (int f = f0; f < f1; ++f) {
        const int j = jn;
        if (f + 1 < f1) jn = a.fN[f + 1];
#pragma unroll
        for (int r = 0; r < 2 * D + 2; ++r) v.prim[2 * r + 1] = a.prim[(size_t)r * nt + j];
        if (vis && !a.fGhost[f]) {
#pragma unroll
            for (int r = 0; r < kVisRows<D>; ++r) v.V[2 * r + 1] = a.V[(size_t)r * nt + j];
        }
        float rhs[D + 2];
        face_rhs32_cells<D, SCH, true, false, false>(v, f, 0, 1, rhs);
#pragma unroll
        for (int q = 0; q < D + 2; ++q) a.flux[(size_t)q * nf + f] = rhs[q];
    }
}

// ---------------------------------------------------------------------------
// fluxupdate32: the rhs of every face of cell c, evaluated by the cell itself
// (each face is evaluated by both of its cells, from the face's own data, so
// both get the bits flux32 stores), summed in ascending face order as the
// update's gather sums the stored values, then the update of apply32. The
// face rhs never reaches memory and a stage needs one kernel less; the next
// stage's primitives go to a.primW, the other of two buffers (the cells of
// this launch still read a.prim).
// ---------------------------------------------------------------------------
template <int D, int SCH, bool LES, bool RES, bool GH>
__device__ __forceinline__ void fluxupdate32(const Args<float>& a, int c, double Ak, double Bk, double dt,
                                             float dt32, int first) {
    constexpr int NQ = D + 2;
    CellIn32<D> in;
    load_cell32<D>(a, c, first, in);
    float sum[NQ];
#pragma unroll
    for (int v = 0; v < NQ; ++v) sum[v] = 0.0f;
    for (int e = a.cfOff[c]; e < a.cfOff[c + 1]; ++e) {
        const int code = a.cfList[e];
        float r[NQ];
        face_rhs32<D, SCH, true, LES, false>(a, code >= 0 ? code : ~code, r);
#pragma unroll
        for (int v = 0; v < NQ; ++v) sum[v] += code >= 0 ? r[v] : neg_bits(r[v]);
    }
    apply32<D, RES, GH>(a, c, sum, in, Ak, Bk, dt, dt32, first);
}

}  // namespace dev
}  // namespace lfm
