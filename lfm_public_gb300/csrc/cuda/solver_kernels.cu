// Device kernels of the explicit finite-volume time step (see solver_kernels.cuh).
#include "solver_device.cuh"
#include "solver_launch.h"

namespace lfm {
namespace dev {

// ---------------------------------------------------------------------------
// k_prep: ghost states and per-cell primitives of entries [first, nt). The
// update writes the cells' and ghosts' primitives for the next stage, so
// between stages only processor halos (copied in) need this pass.
// ---------------------------------------------------------------------------
template <typename T, int D>
__global__ void __launch_bounds__(256) k_prep(Args<T> a, int first) {
    const int t = first + LFM_GLOBAL_ID();
    if (t >= a.nt) return;
    constexpr int NQ = D + 2;
    double qv[NQ];
    stage_state<T, D>(a, t, qv);
    prims64<D>(a, t, qv);
}

// D consecutive FP64 values starting at an index that is a multiple of D:
// one 16-byte load in 2D (the constants of an incidence entry or a cell).
template <int D>
__device__ __forceinline__ void load_vec(const double* p, size_t i, double* out) {
    if constexpr (D == 2) {
        const double2 v = reinterpret_cast<const double2*>(p)[i];
        out[0] = v.x;
        out[1] = v.y;
    } else {
#pragma unroll
        for (int k = 0; k < D; ++k) out[k] = p[i * D + k];
    }
}

// ---------------------------------------------------------------------------
// k_grad: gradients read by M2AUSM's minmod reconstruction.
// ---------------------------------------------------------------------------
template <typename T, int D>
__global__ void __launch_bounds__(256) k_grad(Args<T> a) {
    const int c = LFM_GLOBAL_ID();
    if (c >= a.nc) return;
    T gr[D], gp[D], gu[D][D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        gr[k] = gp[k] = T(0);
#pragma unroll
        for (int l = 0; l < D; ++l) gu[k][l] = T(0);
    }
    // Gauss gradients of rho, p and u: the cell's own share through its
    // constant cellSoW, each neighbour's through the entry constant cfSoN
    // (the face values w v_P + (1 - w) v_N expanded)
    const size_t nt = (size_t)a.nt;
    {
        T sw[D], Uc[D];
        load_vec<D>(a.cellSoW, (size_t)c, sw);
#pragma unroll
        for (int k = 0; k < D; ++k) Uc[k] = a.prim[(size_t)(1 + k) * nt + c];
        const T rhoc = a.q[c];
        const T pc = rhoc * a.prim[(size_t)(D + 1) * nt + c];
#pragma unroll
        for (int x = 0; x < D; ++x) {
            gp[x] = pc * sw[x];
            gr[x] = rhoc * sw[x];
#pragma unroll
            for (int b = 0; b < D; ++b) gu[b][x] = Uc[b] * sw[x];
        }
    }
    for (int e = a.cfOff[c]; e < a.cfOff[c + 1]; ++e) {
        const int j = a.cfNbr[e];
        T so[D];
        load_vec<D>(a.cfSoN, (size_t)e, so);
        const T rhoj = a.q[j];
        const T pj = rhoj * a.prim[(size_t)(D + 1) * nt + j];
#pragma unroll
        for (int x = 0; x < D; ++x) {
            gp[x] += pj * so[x];
            gr[x] += rhoj * so[x];
#pragma unroll
            for (int b = 0; b < D; ++b) gu[b][x] += a.prim[(size_t)(1 + b) * nt + j] * so[x];
        }
    }
#pragma unroll
    for (int k = 0; k < D; ++k) {
        a.grad[(size_t)k * a.nt + c] = gr[k];
        a.grad[(size_t)(D + k) * a.nt + c] = gp[k];
#pragma unroll
        for (int l = 0; l < D; ++l) a.grad[(size_t)(2 * D + k * D + l) * a.nt + c] = gu[k][l];
    }
}

// ---------------------------------------------------------------------------
// k_vis: dudx, dTdx and sigmaU per cell (tauMC is rebuilt per face from dudx).
// ---------------------------------------------------------------------------
// LES compiles in the Smagorinsky SGS stress (cases with a.smagC).
template <typename T, int D, bool LES>
__global__ void __launch_bounds__(256) k_vis(Args<T> a) {
    const int c = LFM_GLOBAL_ID();
    if (c >= a.nc) return;
    T g[D][D], gT[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        gT[k] = T(0);
#pragma unroll
        for (int l = 0; l < D; ++l) g[k][l] = T(0);
    }
    // Gauss gradients of u and of R psi (T = R psi / R: the 1/R factor is
    // applied once to the sum). With the face value v_f = w v_P + (1 - w) v_N
    // and so = S/V seen from c, sum_f v_f so = v_c cellSoW_c + sum_e v_j
    // cfSoN_e: the cell's own share through one cell constant, each
    // neighbour's through an entry constant (the other cell j = cfNbr[e]).
    {
        T sw[D];
        load_vec<D>(a.cellSoW, (size_t)c, sw);
        const T Rc = a.prim[(size_t)(D + 1) * a.nt + c];
#pragma unroll
        for (int x = 0; x < D; ++x) {
            const T Ux = a.prim[(size_t)(1 + x) * a.nt + c];
#pragma unroll
            for (int y = 0; y < D; ++y) g[x][y] = Ux * sw[y];
            gT[x] = Rc * sw[x];
        }
    }
    for (int e = a.cfOff[c]; e < a.cfOff[c + 1]; ++e) {
        const int j = a.cfNbr[e];
        T so[D], fU[D];
        load_vec<D>(a.cfSoN, (size_t)e, so);
#pragma unroll
        for (int k = 0; k < D; ++k) fU[k] = a.prim[(size_t)(1 + k) * a.nt + j];
        const T fR = a.prim[(size_t)(D + 1) * a.nt + j];
#pragma unroll
        for (int x = 0; x < D; ++x) {
#pragma unroll
            for (int y = 0; y < D; ++y) g[x][y] += fU[x] * so[y];
            gT[x] += fR * so[x];
        }
    }
    const T Rinv = (T)a.Rinv;
#pragma unroll
    for (int x = 0; x < D; ++x) gT[x] *= Rinv;
    const T mu = (T)a.mu;
    T tau[D][D];
    stress<T, D>(g, mu, tau);
    T U[D];
#pragma unroll
    for (int k = 0; k < D; ++k) U[k] = a.prim[(size_t)(1 + k) * a.nt + c];
    const size_t nt = (size_t)a.nt;
#pragma unroll
    for (int x = 0; x < D; ++x) {
#pragma unroll
        for (int y = 0; y < D; ++y) a.V[(size_t)(x * D + y) * nt + c] = g[x][y];
        a.V[(size_t)(D * D + x) * nt + c] = gT[x];
        a.V[(size_t)(D * D + D + x) * nt + c] = dotv<T, D>(U, tau[x]);
    }
    if (LES && a.smagC) {   // Smagorinsky LES: the cell's SGS stress
        T sg[D][D];
        sgs_stress<T, D>(g, a.smagC[c], sg);
#pragma unroll
        for (int x = 0; x < D; ++x)
#pragma unroll
            for (int y = 0; y < D; ++y) a.V[(size_t)(kVisRows<D> + x * D + y) * nt + c] = sg[x][y];
    }
}

// ---------------------------------------------------------------------------
// k_flux: rhs of one face.
// ---------------------------------------------------------------------------
template <typename T, int D, int SCH, bool LES>
__global__ void __launch_bounds__(128) k_flux(Args<T> a) {
    const int f = LFM_GLOBAL_ID();
    if (f >= a.nf) return;
    constexpr int NQ = D + 2;
    const size_t nt = (size_t)a.nt, nf = (size_t)a.nf;
    const int i = a.fP[f], j = a.fN[f];
    const bool ghost = a.fGhost[f] != 0;
    const T w = a.w[f], wN = a.wN[f];
    T S[D], Kf[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        S[k] = a.S[k * nf + f];
        Kf[k] = a.K[k * nf + f];
    }
    T qi[NQ], qj[NQ];
#pragma unroll
    for (int v = 0; v < NQ; ++v) {
        qi[v] = (T)a.q[v * nt + i];
        qj[v] = (T)a.q[v * nt + j];
    }
    const T cri = a.prim[i], ari = a.prim[j];
    T cU[D], aU[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
        cU[k] = a.prim[(1 + k) * nt + i];
        aU[k] = a.prim[(1 + k) * nt + j];
    }
    const T cRpsi = a.prim[(D + 1) * nt + i], aRpsi = a.prim[(D + 1) * nt + j];
    const T Rinv = (T)a.Rinv;
    const T dT = (aRpsi - cRpsi) * Rinv;   // T_N - T_P
    T rhs[NQ];

    if (SCH == kSchemeM1) {
        // One_rk_step_M1's Kurganov-Tadmor flux (src/cfd_v0.cpp:2588-2675)
        // builds its "+" and "-" states with the same linear interpolation
        // (w*P + (1-w)*N and (1-w)*N + w*P), so both states are equal, the
        // dissipation terms (q- - q+)*psi+ psi-/(psi+ - psi-) vanish and the
        // wave-speed weights cancel: the flux is the central flux of the
        // interpolated state, F(q_f).S. It is evaluated in that form - one
        // division per face instead of three, no sound speeds - and equals
        // the reference's value up to rounding. The interpolated internal
        // energy per unit mass is that of the interpolated R psi,
        // e = R psi / (gamma - 1) (R psi = (gamma - 1) e in every cell), so
        // e + R psi = gamma / (gamma - 1) R psi.
        const T rho = interp2(w, wN, qi[0], qj[0]);
        T m[D];
#pragma unroll
        for (int k = 0; k < D; ++k) m[k] = interp2(w, wN, qi[k + 1], qj[k + 1]);
        const T Rpsi = interp2(w, wN, cRpsi, aRpsi);
        const T rinv = rcp64(rho);
        T mS = T(0), u2 = T(0);
#pragma unroll
        for (int k = 0; k < D; ++k) {
            mS += m[k] * S[k];
            u2 += m[k] * m[k];
        }
        const T phi = mS * rinv;                          // u_f . S
        const T p = rho * Rpsi;
        rhs[0] = -mS;
#pragma unroll
        for (int k = 0; k < D; ++k) rhs[k + 1] = -(m[k] * phi + p * S[k]);
        rhs[D + 1] = -mS * ((T)a.gh * Rpsi + T(0.5) * u2 * (rinv * rinv));
    } else {
        // Pirozzoli kinetic-energy-preserving mid-point flux (src/cfd_v0.cpp:1966-2023)
        const T rhoavg = T(0.5) * (qi[0] + qj[0]);
        const T rhoavg_inv = rcp64(rhoavg);
        T rhoUavg[D];
#pragma unroll
        for (int k = 0; k < D; ++k) rhoUavg[k] = T(0.5) * (qi[k + 1] + qj[k + 1]);
        T pavg = rhoavg * (T(0.5) * (cRpsi + aRpsi));
        const T Havg = T(0.5) * ((qi[D + 1] * cri + cRpsi) + (qj[D + 1] * ari + aRpsi));
        if (SCH == kSchemeAUSM) {
            // shock sensor, minmod reconstructions and AUSM+ pressure
            // dissipation (src/cfd_v0.cpp:2288-2339)
            const T cavg = T(0.5) * (a.prim[(D + 2) * nt + i] + a.prim[(D + 2) * nt + j]);
            T d[D];
#pragma unroll
            for (int k = 0; k < D; ++k) d[k] = a.d[k * nf + f];
            T cdiv = T(0), ndiv = T(0), ccurl = T(0), ncurl = T(0), cv2 = T(0), nv2 = T(0), unPos = T(0),
              unNeg = T(0), norm = T(0);
#pragma unroll
            for (int x = 0; x < D; ++x) {
                cdiv += a.V[(x * D + x) * nt + i];
                ndiv += a.V[(x * D + x) * nt + j];
#pragma unroll
                for (int y = x + 1; y < D; ++y) {
                    const T cc = a.V[(x * D + y) * nt + i] - a.V[(y * D + x) * nt + i];
                    const T nn = a.V[(x * D + y) * nt + j] - a.V[(y * D + x) * nt + j];
                    ccurl += cc * cc;
                    ncurl += nn * nn;
                }
                cv2 += cU[x] * cU[x];
                nv2 += aU[x] * aU[x];
                T gi[D], gj[D];
#pragma unroll
                for (int y = 0; y < D; ++y) {
                    gi[y] = a.grad[(2 * D + x * D + y) * nt + i];
                    gj[y] = a.grad[(2 * D + x * D + y) * nt + j];
                }
                const T uP = minmod_interp<T, D>(cU[x], aU[x], gi, d, w, T(1));
                const T uN = minmod_interp<T, D>(cU[x], aU[x], gj, d, w, T(-1));
                unPos += uP * S[x];
                unNeg += uN * S[x];
                norm += S[x] * S[x];
            }
            T ct = -(cdiv / sqrt(cdiv * cdiv + ccurl + T(4e-2)));
            ct = (ct < T(0)) ? T(0) : ct;
            T nt_ = -(ndiv / sqrt(ndiv * ndiv + ncurl + T(4e-2)));
            nt_ = (nt_ < T(0)) ? T(0) : nt_;
            const T theta = T(0.5) * (ct + nt_);
            const T cp = qi[0] * (T)a.gm1 * (qi[D + 1] * cri - T(0.5) * cv2);
            const T np = qj[0] * (T)a.gm1 * (qj[D + 1] * ari - T(0.5) * nv2);
            T gri[D], grj[D], gpi[D], gpj[D];
#pragma unroll
            for (int y = 0; y < D; ++y) {
                gri[y] = a.grad[y * nt + i];
                grj[y] = a.grad[y * nt + j];
                gpi[y] = a.grad[(D + y) * nt + i];
                gpj[y] = a.grad[(D + y) * nt + j];
            }
            const T rhoPos = minmod_interp<T, D>(qi[0], qj[0], gri, d, w, T(1));
            const T rhoNeg = minmod_interp<T, D>(qi[0], qj[0], grj, d, w, T(-1));
            const T pPos = minmod_interp<T, D>(cp, np, gpi, d, w, T(1));
            const T pNeg = minmod_interp<T, D>(cp, np, gpj, d, w, T(-1));
            const T Msq = (unPos * unPos + unNeg * unNeg) / (T(2) * cavg * cavg * norm);
            const T snorm = sqrt(norm);
            const T MPos = unPos / (snorm * cavg);
            const T MNeg = unNeg / (snorm * cavg);
            const T Minf = T(0.2);
            T m = (Msq < Minf * Minf) ? Minf * Minf : Msq;
            m = (m < T(1)) ? m : T(1);
            const T M0 = sqrt(m);
            const T fa = M0 * (T(2) - M0);
            const T alpha = T(3) * (T(5) * fa * fa - T(4)) / T(16);
            const T phalf = pNeg * (p5pos(MNeg, alpha) - p5neg(MNeg, alpha)) -
                            pPos * (p5pos(MPos, alpha) - p5neg(MPos, alpha));
            const T pu = T(-0.75) * p5pos(MPos, alpha) * p5neg(MNeg, alpha) * (rhoPos + rhoNeg) * cavg * fa *
                         (unNeg - unPos);
            pavg += theta * (pu - T(0.5) * phalf);
        }
        T phiavg = T(0);
#pragma unroll
        for (int k = 0; k < D; ++k) phiavg += (rhoUavg[k] * rhoavg_inv) * S[k];
        rhs[0] = -rhoavg * phiavg;
#pragma unroll
        for (int k = 0; k < D; ++k) rhs[k + 1] = -(rhoUavg[k] * phiavg + pavg * S[k]);
        rhs[D + 1] = -(rhoavg * Havg * phiavg);
    }

    // Viscous face terms (src/cfd_v0.cpp:2682-2796). With mu == 0 every term
    // is an exact zero and the block is skipped.
    const T mu = (T)a.mu;
    if (mu != T(0)) {
        const T lapc = a.lapc[f];   // |delta| / |d|
        T g[D][D], gT[D], sU[D];
        if (!ghost) {
#pragma unroll
            for (int x = 0; x < D; ++x) {
#pragma unroll
                for (int y = 0; y < D; ++y)
                    g[x][y] = interp2(w, wN, a.V[(x * D + y) * nt + i], a.V[(x * D + y) * nt + j]);
                gT[x] = interp2(w, wN, a.V[(D * D + x) * nt + i], a.V[(D * D + x) * nt + j]);
                sU[x] = interp2(w, wN, a.V[(D * D + D + x) * nt + i], a.V[(D * D + D + x) * nt + j]);
            }
        } else {
            // explicit two-point gradients on physical boundaries
            const T dinv = a.dinv[f];
            T dn[D], tau[D][D], Uf[D];
#pragma unroll
            for (int k = 0; k < D; ++k) dn[k] = a.dnorm[k * nf + f];
#pragma unroll
            for (int x = 0; x < D; ++x) {
#pragma unroll
                for (int y = 0; y < D; ++y) g[x][y] = (aU[x] - cU[x]) * dn[y] * dinv;
                gT[x] = dT * dn[x] * dinv;
                Uf[x] = interp(w, cU[x], aU[x]);
            }
            stress<T, D>(g, mu, tau);
#pragma unroll
            for (int x = 0; x < D; ++x) sU[x] = dotv<T, D>(Uf, tau[x]);
        }
        // The face tauMC: the reference interpolates the cells' tauMC =
        // mu dudx^T - (2/3) mu tr(dudx) I (and on boundary faces applies the
        // same expression to the two-point gradient); it is linear in dudx,
        // so it is rebuilt here from the face gradient g.
        T tr = g[0][0];
#pragma unroll
        for (int x = 1; x < D; ++x) tr += g[x][x];
        const T dsum = -(T)a.mu23 * tr;
        const T kc = (T)a.kcond;
#pragma unroll
        for (int x = 0; x < D; ++x) {
            T gtS = g[0][x] * S[0];
#pragma unroll
            for (int y = 1; y < D; ++y) gtS += g[y][x] * S[y];
            // div tauMC + the Laplacian split: mu (g^T S + |delta|/|d| du + K.g) + dsum S
            rhs[x + 1] += mu * (gtS + lapc * (aU[x] - cU[x]) + dotv<T, D>(Kf, g[x])) + dsum * S[x];
        }
        const T lapT = kc * (lapc * dT + dotv<T, D>(Kf, gT));
        rhs[D + 1] += dotv<T, D>(sU, S) + lapT;
        // Smagorinsky LES: the face tauMC also interpolates the cells' SGS
        // stress (boundary faces keep the laminar two-point one, as in the
        // reference)
        if (LES && a.smagC && !ghost) {
#pragma unroll
            for (int x = 0; x < D; ++x) {
                T s = T(0);
#pragma unroll
                for (int y = 0; y < D; ++y)
                    s += interp(w, a.V[(kVisRows<D> + x * D + y) * nt + i], a.V[(kVisRows<D> + x * D + y) * nt + j]) *
                         S[y];
                rhs[x + 1] += s;
            }
        }
    }
#pragma unroll
    for (int v = 0; v < NQ; ++v) a.flux[v * nf + f] = rhs[v];
}

// ---------------------------------------------------------------------------
// k_update: gather, sponge, RK update (update_cell, solver_device.cuh), then
// the next stage's primitives of the cell and, with a.cellGhosts, the states
// and primitives of its boundary ghosts.
// ---------------------------------------------------------------------------
template <typename T, int D, bool RES>
__global__ void __launch_bounds__(256) k_update(const __grid_constant__ Args<T> a, double Ak, double Bk, double dt, int first) {
    const int c = LFM_GLOBAL_ID();
    if (c >= a.nc) return;
    update_cell<T, D, RES, true>(a, c, Ak, Bk, dt, first);
}

// ---------------------------------------------------------------------------
// Reductions: compute_cfl / compute_dt (max / min over cells) and the sum of
// squared cell residuals. Block results go to partials, a single block
// finishes; both levels use a fixed tree, so results are reproducible.
// ---------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(256) k_cfl(const double* q, QOffset qo, int nt, int nc, const double* volInv,
                                             const int* sOff, const double* cellS, double dt, int mode, double maxCo,
                                             double* partial) {
    __shared__ double sh[256];
    const int c = LFM_GLOBAL_ID();
    double v = (mode == 0) ? 0.0 : 100.0;
    if (c < nc) {
        const double rho = q[c] + qo.v[0];
        if (mode == 0) {
            double cfl = 0;
            for (int e = sOff[c]; e < sOff[c + 1]; ++e) {
                double flux = 0.;
                for (int k = 0; k < D; ++k) flux += (q[(size_t)(k + 1) * nt + c] + qo.v[k + 1]) * cellS[(size_t)e * D + k];
                cfl += fabs(flux);
            }
            v = cfl * ((1.0 / rho) * volInv[c] * dt);
        } else {
            double sumFlux = 0;
            for (int e = sOff[c]; e < sOff[c + 1]; ++e) {
                const double* S = &cellS[(size_t)e * D];
                double sMag = 0.;
                for (int k = 0; k < D; ++k) sMag += S[k] * S[k];
                sMag = sqrt(sMag);
                double flux = 0.;
                for (int k = 0; k < D; ++k) flux += (q[(size_t)(k + 1) * nt + c] + qo.v[k + 1]) * S[k] / sMag;
                sumFlux += fabs(flux);
            }
            v = maxCo * rho * 2.0 * (1.0 / volInv[c]) / sumFlux;
        }
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            const double o = sh[threadIdx.x + s];
            sh[threadIdx.x] = (mode == 0) ? fmax(sh[threadIdx.x], o) : fmin(sh[threadIdx.x], o);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(256) k_reduce_final(const double* partial, int n, int mode, double* out) {
    __shared__ double sh[256];
    double v = (mode == 0) ? 0.0 : (mode == 1 ? 100.0 : 0.0);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const double o = partial[k];
        v = (mode == 0) ? fmax(v, o) : (mode == 1 ? fmin(v, o) : v + o);
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            const double o = sh[threadIdx.x + s];
            sh[threadIdx.x] = (mode == 0) ? fmax(sh[threadIdx.x], o) : (mode == 1 ? fmin(sh[threadIdx.x], o) : sh[threadIdx.x] + o);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

__global__ void __launch_bounds__(256) k_res_sq(const double* res, int nc, double* partial) {
    __shared__ double sh[256];
    const int c = LFM_GLOBAL_ID();
    const double v = (c < nc) ? res[c] * res[c] : 0.0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void k_set_flag(int* flag, int v) { *flag = v; }

// ---------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------
static inline unsigned blocks(int n, int b) { return (unsigned)((n + b - 1) / b); }

template <typename T, int D, int SCH, bool LES>
void launch_flux(const Args<T>& a, cudaStream_t st) {
    k_flux<T, D, SCH, LES><<<blocks(a.nf, 128), 128, 0, st>>>(a);
}

template <typename T, int D, bool LES>
void launch_fp64(const Args<T>& a, const StageConfig& s, int which, cudaStream_t st) {
    switch (which) {
        case 0: {
            // the update keeps the cells' and (a.cellGhosts) the ghosts'
            // primitives current: only halos remain, unless the state is new
            const int first = s.fullPrep ? 0 : (a.cellGhosts ? a.nc + a.ng : a.nc);
            if (a.nt > first) k_prep<T, D><<<blocks(a.nt - first, 256), 256, 0, st>>>(a, first);
            break;
        }
        case 1:
            if (s.needGrad) k_grad<T, D><<<blocks(a.nc, 256), 256, 0, st>>>(a);
            break;
        case 2:
            if (s.needVis) k_vis<T, D, LES><<<blocks(a.nc, 256), 256, 0, st>>>(a);
            break;
        case 3:
            if (s.scheme == kSchemeM1) launch_flux<T, D, kSchemeM1, LES>(a, st);
            else if (s.scheme == kSchemeM2) launch_flux<T, D, kSchemeM2, LES>(a, st);
            else launch_flux<T, D, kSchemeAUSM, LES>(a, st);
            break;
        case 4:
            if (s.withRes) k_update<T, D, true><<<blocks(a.nc, 256), 256, 0, st>>>(a, s.A, s.B, s.dt, s.first);
            else k_update<T, D, false><<<blocks(a.nc, 256), 256, 0, st>>>(a, s.A, s.B, s.dt, s.first);
            break;
        default: break;
    }
}

// Individual kernels (a stage is kernels 0..kKernelsPerStage-1 in order).
template <typename T>
void launch_kernel(const Args<T>& a, const StageConfig& s, int which, cudaStream_t st) {
    const bool les = a.smagC != nullptr;
    if (a.D == 2)
        les ? launch_fp64<T, 2, true>(a, s, which, st) : launch_fp64<T, 2, false>(a, s, which, st);
    else
        les ? launch_fp64<T, 3, true>(a, s, which, st) : launch_fp64<T, 3, false>(a, s, which, st);
}

template <typename T>
void launch_stage(const Args<T>& a, const StageConfig& s, cudaStream_t st) {
    for (int k = 0; k < kKernelsPerStage; ++k) launch_kernel<T>(a, s, k, st);
}
template void launch_stage<double>(const Args<double>&, const StageConfig&, cudaStream_t);
// The FP32-bulk form runs its own kernels (solver_kernels_fp32.cu).
template <>
void launch_stage<float>(const Args<float>& a, const StageConfig& s, cudaStream_t st) {
    for (int k = 0; k < kKernelsPerStage; ++k) launch_kernel_fp32(a, s, k, st);
}
template void launch_kernel<double>(const Args<double>&, const StageConfig&, int, cudaStream_t);
template <>
void launch_kernel<float>(const Args<float>& a, const StageConfig& s, int which, cudaStream_t st) {
    launch_kernel_fp32(a, s, which, st);
}

void launch_cfl(int D, const double* q, QOffset qo, int nt, int nc, const double* volInv, const int* sOff, const double* cellS,
                double dt, int mode, double maxCo, double* partial, double* out, cudaStream_t st) {
    const unsigned nb = blocks(nc, 256);
    if (D == 2)
        k_cfl<2><<<nb, 256, 0, st>>>(q, qo, nt, nc, volInv, sOff, cellS, dt, mode, maxCo, partial);
    else
        k_cfl<3><<<nb, 256, 0, st>>>(q, qo, nt, nc, volInv, sOff, cellS, dt, mode, maxCo, partial);
    k_reduce_final<<<1, 256, 0, st>>>(partial, (int)nb, mode, out);
}

void launch_res_sum(const double* res, int nc, double* partial, double* out, cudaStream_t st) {
    const unsigned nb = blocks(nc, 256);
    k_res_sq<<<nb, 256, 0, st>>>(res, nc, partial);
    k_reduce_final<<<1, 256, 0, st>>>(partial, (int)nb, 2, out);
}

void launch_set_flag(int* flag, int v, cudaStream_t st) { k_set_flag<<<1, 1, 0, st>>>(flag, v); }

// dst[v][c] = src[v][c] + sign * off[v] for nq rows of n cells (converts
// between the FP32-bulk form's stored q - q_ref and the absolute state).
__global__ void __launch_bounds__(256) k_offset_rows(double* dst, int64_t dstStride, const double* src,
                                                     int64_t srcStride, int n, int nq, QOffset off, double sign) {
    const int c = LFM_GLOBAL_ID();
    if (c >= n) return;
    for (int v = 0; v < nq; ++v) dst[(size_t)v * dstStride + c] = src[(size_t)v * srcStride + c] + sign * off.v[v];
}

void launch_offset_rows(double* dst, int64_t dstStride, const double* src, int64_t srcStride, int n, int nq,
                        QOffset off, double sign, cudaStream_t st) {
    if (n > 0) k_offset_rows<<<blocks(n, 256), 256, 0, st>>>(dst, dstStride, src, srcStride, n, nq, off, sign);
}

// Halo copies between the partitions of a decomposed case: halo slot h (index
// first + h of the destination) takes `rows` values of cell srcCell[h] of
// partition srcPart[h] -- the on-device form of the reference's MPI halo
// exchange (src/cfd_v0.cpp:3283-3374, 3607-3692).
template <typename X>
__global__ void __launch_bounds__(256) k_halo_gather(X* dst, int dstNt, int first, int rows, int nh,
                                                     const int* srcPart, const int* srcCell, X* const* srcBase,
                                                     const int* srcNt) {
    const int h = LFM_GLOBAL_ID();
    if (h >= nh) return;
    const int p = srcPart[h], c = srcCell[h];
    const X* src = srcBase[p];
    const size_t snt = (size_t)srcNt[p];
    for (int r = 0; r < rows; ++r) dst[(size_t)r * dstNt + first + h] = src[(size_t)r * snt + c];
}

template <typename X>
void launch_halo_gather(X* dst, int dstNt, int first, int rows, int nh, const int* srcPart, const int* srcCell,
                        X* const* srcBase, const int* srcNt, cudaStream_t st) {
    if (nh > 0)
        k_halo_gather<X><<<blocks(nh, 256), 256, 0, st>>>(dst, dstNt, first, rows, nh, srcPart, srcCell, srcBase,
                                                          srcNt);
}
template void launch_halo_gather<double>(double*, int, int, int, int, const int*, const int*, double* const*,
                                         const int*, cudaStream_t);
template void launch_halo_gather<float>(float*, int, int, int, int, const int*, const int*, float* const*,
                                        const int*, cudaStream_t);

}  // namespace dev
}  // namespace lfm
