/* CPU restatement of libFastMesh's explicit time step - the oracle.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the CPU
 * baseline legs of bench.py may load this library; the product path never
 * calls it. It restates, in plain C over the flattened lfm_solver_desc, the
 * reference's per-stage loops in the reference's own order of operations:
 *
 *   prepare_for_timestep      src/cfd_v0.cpp:1325-1333
 *   prepare_for_RKstep        src/cfd_v0.cpp:1338-1377
 *   set_boundary_conditions   src/cfd_v0.cpp:1009-1221
 *   calc_gradients_M2AUSM     src/cfd_v0.cpp:1383-1495 (the gradients M2AUSM reads)
 *   calc_VIS                  src/cfd_v0.cpp:1743-1860
 *   calc_VIS_Smagorinsky      src/cfd_v0.cpp:1573-1737 (desc->smag_c set)
 *   one_rk_step_M2            src/cfd_v0.cpp:1896-2179
 *   one_rk_step_M2AUSM        src/cfd_v0.cpp:2185-2523, p5Pos/p5Neg :1862-1894,
 *                             calc_r / interp_minmod api/cfdv0_solver.h:306-370
 *   one_rk_step_M1            src/cfd_v0.cpp:2529-2832
 *   compute_cfl / compute_dt  src/cfd_v0.cpp:2886-2942
 *   stage schedule            src/mesh_solver.cpp:474-727
 *
 * Cells are processed in solver order, which is the reference's
 * (submesh, index) order, and each cell's owned faces in slot order, so every
 * scatter lands in the same sequence as in the reference. The per-face
 * constants in the description (|S|, 1/|d|, d/|d|, |delta|, K) are the values
 * the reference computes inside its face loop, evaluated once with the same
 * expressions. Build with -ffp-contract=off so that every product and sum is
 * rounded on its own, as in the reference's x86-64 -O3 build. */
#include "lfm_port.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define MAXD 3

typedef struct {
    const lfm_solver_desc* c;
    int D, nq;
    int64_t nc, ng, nf;
    double* q;        /* nq x (nc + ng), cells then ghosts */
    double* dq;       /* nq x nc */
    double* res;      /* nq x (nc + ng) cell residuals */
    double* dudx;     /* (nc + ng) x D x D */
    double* dTdx;     /* (nc + ng) x D */
    double* tauMC;    /* (nc + ng) x D x D */
    double* sigmaU;   /* (nc + ng) x D */
    double* rhoGrad;  /* (nc + ng) x D */
    double* pGrad;    /* (nc + ng) x D */
    double* UGrad;    /* (nc + ng) x D x D */
    double* volInvAll;/* nc + ng, ghosts 0 */
    int64_t* faceStart; /* owned-face range of each cell */
    double Rinv, gm1;
} Port;

static double Q(const Port* P, int v, int64_t i) { return P->q[(int64_t)v * (P->nc + P->ng) + i]; }
static double* Qp(Port* P, int v, int64_t i) { return &P->q[(int64_t)v * (P->nc + P->ng) + i]; }

static double compute_Rpsi(const Port* P, int64_t i) {
    const int D = P->D;
    const double rho_inv = 1.0 / Q(P, 0, i);
    double s = Q(P, 1, i) * Q(P, 1, i);
    for (int k = 1; k < D; ++k) s += Q(P, k + 1, i) * Q(P, k + 1, i);
    return P->gm1 * (Q(P, D + 1, i) - 0.5 * s * rho_inv) * rho_inv;
}

static double interp(double w, double a, double b) { return w * a + (1.0 - w) * b; }

static double dot(const double* a, const double* b, int D) {
    double s = a[0] * b[0];
    for (int k = 1; k < D; ++k) s += a[k] * b[k];
    return s;
}

static double sgn(double a) { return a < 0.0 ? -1.0 : 1.0; }
static double dmax(double a, double b) { return (a < b) ? b : a; } /* std::max */
static double dmin(double a, double b) { return (b < a) ? b : a; } /* std::min */

/* tau from a velocity gradient (src/cfd_v0.cpp:1813-1822 and repeated). */
static void stress(const double* g, double mu, int D, double tau[MAXD][MAXD]) {
    for (int a = 0; a < D; ++a) {
        tau[a][a] = 2.0 * g[a * D + a];
        for (int b1 = a + 1; b1 < D + a; ++b1) {
            const int b = b1 % D;
            tau[a][b] = mu * (g[a * D + b] + g[b * D + a]);
            tau[a][a] -= g[b * D + b];
        }
        tau[a][a] *= 2.0 / 3.0 * mu;
    }
}

/* tauMC and sigmaU of a cell from its current dudx (src/cfd_v0.cpp:1813-1857);
 * with a Smagorinsky constant C (smag, or NULL for laminar) the SGS terms of
 * calc_VIS_Smagorinsky (src/cfd_v0.cpp:1675-1695) are added to tauMC. */
static void viscous_derived(Port* P, int64_t i, const double* U, double mu, const double* smag) {
    const int D = P->D;
    const double* g = &P->dudx[i * D * D];
    double tau[MAXD][MAXD];
    stress(g, mu, D, tau);
    double diagSum = 0;
    for (int a = 0; a < D; ++a) diagSum -= g[a * D + a];
    diagSum *= mu * 2.0 / 3.0;
    for (int a = 0; a < D; ++a) {
        P->sigmaU[i * D + a] = dot(U, tau[a], D);
        for (int b = 0; b < D; ++b) P->tauMC[i * D * D + a * D + b] = mu * g[b * D + a];
        P->tauMC[i * D * D + a * D + a] += diagSum;
    }
    if (smag) {
        const double C = *smag;
        double strainMag = 0.0, divu = 0.0;
        for (int a = 0; a < D; ++a) {
            for (int b = 0; b < D; ++b) {
                const double sij = 0.5 * (g[a * D + b] + g[b * D + a]);
                strainMag += pow(sij, 2);
            }
            divu += g[a * D + a];
        }
        strainMag = sqrt(2.0 * strainMag);
        for (int a = 0; a < D; ++a) {
            for (int b = 0; b < D; ++b) {
                const double sij = 0.5 * (g[a * D + b] + g[b * D + a]);
                P->tauMC[i * D * D + a * D + b] -= C * strainMag * sij;
            }
            P->tauMC[i * D * D + a * D + a] += C * strainMag * divu / 3.0;
        }
    }
}

static void set_boundary_conditions(Port* P) {
    const lfm_solver_desc* c = P->c;
    const int D = P->D;
    for (int64_t g = 0; g < P->ng; ++g) {
        const int64_t in = c->ghost_cell[g];
        const int64_t gi = P->nc + g;
        const int kind = c->ghost_kind[g];
        if (kind == LFM_GHOST_WALL) {
            *Qp(P, 0, gi) = Q(P, 0, in);
            for (int k = 0; k < D; ++k) *Qp(P, k + 1, gi) = -Q(P, k + 1, in);
            *Qp(P, D + 1, gi) = Q(P, D + 1, in);
            continue;
        }
        int inlet = (kind == LFM_GHOST_INLET);
        if (kind == LFM_GHOST_FARFIELD) {
            /* Inflow where the free-stream direction enters the face. The
             * reference reads an uninitialised angle of attack and indexes S
             * transposed here; this uses angle 0 and the face's own S. */
            double T = 0.0;
            for (int64_t k = c->cell_face_offsets[in]; k < c->cell_face_offsets[in + 1]; ++k) {
                const int64_t ff = c->cell_faces[k];
                if (c->face_n[ff] == gi) T = c->S[ff]; /* x component, direction (1,0,0) */
            }
            inlet = (T <= 0.0);
        }
        if (kind != LFM_GHOST_INLET && kind != LFM_GHOST_OUTLET && kind != LFM_GHOST_FARFIELD) continue;
        const double rhoInt = Q(P, 0, in);
        double Uint[MAXD], um2 = 0.0;
        for (int k = 0; k < D; ++k) {
            Uint[k] = Q(P, k + 1, in) / rhoInt;
            um2 += Uint[k] * Uint[k];
        }
        const double pInt = (Q(P, D + 1, in) - 0.5 * um2 * rhoInt) * P->gm1;
        if (inlet) {
            const double TInt = pInt * P->Rinv / rhoInt;
            const double TExt = c->TInf;
            const double rhoExt = rhoInt * TInt / TExt;
            double ue2 = 0.0;
            for (int k = 0; k < D; ++k) ue2 += c->UInf[k] * c->UInf[k];
            const double pExt = pInt;
            const double EExt = pExt / (rhoExt * P->gm1) + 0.5 * ue2;
            *Qp(P, 0, gi) = rhoExt;
            for (int k = 0; k < D; ++k) *Qp(P, k + 1, gi) = rhoExt * c->UInf[k];
            *Qp(P, D + 1, gi) = rhoExt * EExt;
        } else {
            const double pExt = c->pInf;
            const double rhoExt = rhoInt * pExt / pInt;
            double ue2 = 0.0;
            for (int k = 0; k < D; ++k) ue2 += Uint[k] * Uint[k];
            const double EExt = pExt / (rhoExt * P->gm1) + 0.5 * ue2;
            *Qp(P, 0, gi) = rhoExt;
            for (int k = 0; k < D; ++k) *Qp(P, k + 1, gi) = rhoExt * Uint[k];
            *Qp(P, D + 1, gi) = rhoExt * EExt;
        }
    }
}

static void calc_gradients_ausm(Port* P) {
    const lfm_solver_desc* c = P->c;
    const int D = P->D;
    for (int64_t f = 0; f < P->nf; ++f) {
        const int64_t i = c->face_p[f], j = c->face_n[f];
        const double w = c->w[f];
        double S[MAXD], UU[MAXD], cso[MAXD], aso[MAXD];
        for (int k = 0; k < D; ++k) S[k] = c->S[k * P->nf + f];
        for (int k = 0; k < D; ++k) UU[k] = interp(w, Q(P, k + 1, i) / Q(P, 0, i), Q(P, k + 1, j) / Q(P, 0, j));
        const double rho = interp(w, Q(P, 0, i), Q(P, 0, j));
        for (int k = 0; k < D; ++k) {
            cso[k] = S[k] * P->volInvAll[i];
            aso[k] = -S[k] * P->volInvAll[j];
        }
        double r = Q(P, 0, i), E = Q(P, D + 1, i) / r, vmag = 0.0;
        for (int k = 0; k < D; ++k) vmag += (Q(P, k + 1, i) / r) * (Q(P, k + 1, i) / r);
        const double cell_p = r * P->gm1 * (E - 0.5 * vmag);
        r = Q(P, 0, j);
        E = Q(P, D + 1, j) / r;
        vmag = 0.0;
        for (int k = 0; k < D; ++k) vmag += (Q(P, k + 1, j) / r) * (Q(P, k + 1, j) / r);
        const double neigh_p = r * P->gm1 * (E - 0.5 * vmag);
        const double p = interp(w, cell_p, neigh_p);
        for (int a = 0; a < D; ++a) {
            P->pGrad[i * D + a] += p * cso[a];
            P->pGrad[j * D + a] += p * aso[a];
            for (int b = 0; b < D; ++b) {
                P->UGrad[i * D * D + b * D + a] += UU[b] * cso[a];
                P->UGrad[j * D * D + b * D + a] += UU[b] * aso[a];
            }
            P->rhoGrad[i * D + a] += rho * cso[a];
            P->rhoGrad[j * D + a] += rho * aso[a];
        }
    }
}

static void calc_VIS(Port* P) {
    const lfm_solver_desc* c = P->c;
    const int D = P->D;
    const double mu = c->mu;
    for (int64_t f = 0; f < P->nf; ++f) {
        const int64_t i = c->face_p[f], j = c->face_n[f];
        const double w = c->w[f];
        const double cell_Rpsi = compute_Rpsi(P, i);
        const double adjc_Rpsi = compute_Rpsi(P, j);
        const double cri = 1.0 / Q(P, 0, i), ari = 1.0 / Q(P, 0, j);
        double fU[MAXD], S[MAXD], cso[MAXD], aso[MAXD], cU[MAXD], aU[MAXD];
        for (int k = 0; k < D; ++k) S[k] = c->S[k * P->nf + f];
        for (int k = 0; k < D; ++k) fU[k] = interp(w, Q(P, k + 1, i) * cri, Q(P, k + 1, j) * ari);
        const double fT = interp(w, cell_Rpsi, adjc_Rpsi) * P->Rinv;
        for (int k = 0; k < D; ++k) {
            cso[k] = S[k] * P->volInvAll[i];
            aso[k] = -S[k] * P->volInvAll[j];
        }
        for (int a = 0; a < D; ++a)
            for (int b = 0; b < D; ++b) {
                P->dudx[i * D * D + a * D + b] += fU[a] * cso[b];
                P->dudx[j * D * D + a * D + b] += fU[a] * aso[b];
            }
        for (int a = 0; a < D; ++a) {
            P->dTdx[i * D + a] += fT * cso[a];
            P->dTdx[j * D + a] += fT * aso[a];
        }
        for (int k = 0; k < D; ++k) {
            cU[k] = Q(P, k + 1, i) / Q(P, 0, i);
            aU[k] = Q(P, k + 1, j) / Q(P, 0, j);
        }
        /* the owner's constant for both sides, as calc_VIS_Smagorinsky
         * computes it once per visiting cell (src/cfd_v0.cpp:1601) */
        const double* smag = c->smag_c ? &c->smag_c[i] : NULL;
        viscous_derived(P, i, cU, mu, smag);
        viscous_derived(P, j, aU, mu, smag);
    }
}

static double minmod_interp(double cp, double ap, const double* grad, const double* d, double w, double flux,
                            int D) {
    const double gradf = ap - cp + 1.0e-30;
    double gradcf = 0.0;
    for (int k = 0; k < D; ++k) gradcf += d[k] * grad[k];
    double r;
    if (fabs(gradcf) >= 1000.0 * fabs(gradf))
        r = 2.0 * 1000.0 * sgn(gradcf) * sgn(gradf) - 1.0;
    else
        r = 2.0 * (gradcf / gradf) - 1.0;
    const double limiter = dmax(dmin(r, 1.0), 0.0);
    const double weight = limiter * w + (1.0 - limiter) * (1.0 + flux) * 0.5;
    return weight * cp + (1.0 - weight) * ap;
}

static double p5Pos(double M, double alpha) {
    const double M2Pos = 0.25 * (M + 1.0) * (M + 1.0);
    const double M2Neg = -0.25 * (M - 1.0) * (M - 1.0);
    const double M1Pos = 0.5 * (M + fabs(M));
    if (fabs(M) < 1) return M2Pos * ((2.0 - M) - 16.0 * alpha * M * M2Neg);
    return M1Pos / M;
}

static double p5Neg(double M, double alpha) {
    const double M2Pos = 0.25 * (M + 1.0) * (M + 1.0);
    const double M2Neg = -0.25 * (M - 1.0) * (M - 1.0);
    const double M1Neg = 0.5 * (M - fabs(M));
    if (fabs(M) < 1) return M2Neg * ((-2.0 - M) + 16.0 * alpha * M * M2Pos);
    return M1Neg / M;
}

/* one_rk_step_M{1,2,2AUSM} for all cells in order. */
static void rk_step(Port* P, int rk, double dt, int resCheck) {
    const lfm_solver_desc* c = P->c;
    const int D = P->D, nq = P->nq;
    const double mu = c->mu, gamma = c->gamma;
    const int solver = c->solver;
    for (int64_t i = 0; i < P->nc; ++i) {
        const double cri = 1.0 / Q(P, 0, i);
        double cU[MAXD];
        for (int k = 0; k < D; ++k) cU[k] = Q(P, k + 1, i) * cri;
        const double cell_Rpsi = compute_Rpsi(P, i);
        const double cell_T = cell_Rpsi * P->Rinv;
        for (int64_t f = P->faceStart[i]; f < P->faceStart[i + 1]; ++f) {
            const int64_t j = c->face_n[f];
            const int ghost = c->face_ghost[f];
            const double weight = c->w[f], omw = 1.0 - weight;
            double S[MAXD], d[MAXD], dn[MAXD], Kf[MAXD];
            for (int k = 0; k < D; ++k) {
                S[k] = c->S[k * P->nf + f];
                d[k] = c->d[k * P->nf + f];
                dn[k] = c->dnorm[k * P->nf + f];
                Kf[k] = c->K[k * P->nf + f];
            }
            const double S_mag = c->smag[f], dmag_inv = c->dmag_inv[f], delta_mag = c->delta_mag[f];
            const double ari = 1.0 / Q(P, 0, j);
            double aU[MAXD];
            for (int k = 0; k < D; ++k) aU[k] = Q(P, k + 1, j) * ari;
            const double adjc_Rpsi = compute_Rpsi(P, j);
            const double adjc_T = adjc_Rpsi * P->Rinv;
            double rhs[MAXD + 2];

            if (solver == LFM_SOLVER_M1) {
                const double rhoPos = interp(weight, Q(P, 0, i), Q(P, 0, j));
                const double rhoNeg = interp(omw, Q(P, 0, j), Q(P, 0, i));
                const double rhoPos_inv = 1.0 / rhoPos, rhoNeg_inv = 1.0 / rhoNeg;
                double rhoUPos[MAXD], rhoUNeg[MAXD], uPos[MAXD], uNeg[MAXD];
                for (int k = 0; k < D; ++k) {
                    rhoUPos[k] = interp(weight, Q(P, k + 1, i), Q(P, k + 1, j));
                    rhoUNeg[k] = interp(omw, Q(P, k + 1, j), Q(P, k + 1, i));
                }
                double cell_e = 2 * Q(P, D + 1, i) * cri;
                double adjc_e = 2 * Q(P, D + 1, j) * ari;
                for (int k = 0; k < D; ++k) {
                    cell_e -= cU[k] * cU[k];
                    adjc_e -= aU[k] * aU[k];
                }
                cell_e *= 0.5;
                adjc_e *= 0.5;
                const double ePos = interp(weight, cell_e, adjc_e), eNeg = interp(omw, adjc_e, cell_e);
                const double RpsiPos = interp(weight, cell_Rpsi, adjc_Rpsi);
                const double RpsiNeg = interp(omw, adjc_Rpsi, cell_Rpsi);
                const double pPos = rhoPos * RpsiPos, pNeg = rhoNeg * RpsiNeg;
                const double cP = sqrt(gamma * cell_Rpsi), cN = sqrt(gamma * adjc_Rpsi);
                const double cPos = interp(weight, cP, cN), cNeg = interp(omw, cN, cP);
                double phiPos = 0.0, phiNeg = 0.0;
                for (int k = 0; k < D; ++k) {
                    uPos[k] = rhoUPos[k] * rhoPos_inv;
                    uNeg[k] = rhoUNeg[k] * rhoNeg_inv;
                    phiPos += uPos[k] * S[k];
                    phiNeg += -uNeg[k] * S[k];
                }
                /* std::max / std::min over {a, b, 0}: the first extreme wins */
                double psiPos = phiPos + cPos * S_mag;
                const double b1 = -phiNeg + cNeg * S_mag;
                if (psiPos < b1) psiPos = b1;
                if (psiPos < 0.0) psiPos = 0.0;
                double psiNeg = phiPos - cPos * S_mag;
                const double b2 = -phiNeg - cNeg * S_mag;
                if (b2 < psiNeg) psiNeg = b2;
                if (0.0 < psiNeg) psiNeg = 0.0;
                const double a0 = 1.0 / (psiPos - psiNeg);
                const double a1 = psiPos * psiNeg;
                const double aPos = psiPos * phiPos;
                const double aNeg = psiNeg * phiNeg;
                double rhoEPos = ePos, rhoENeg = eNeg;
                for (int k = 0; k < D; ++k) {
                    rhoEPos += 0.5 * uPos[k] * uPos[k];
                    rhoENeg += 0.5 * uNeg[k] * uNeg[k];
                }
                rhoEPos *= rhoPos;
                rhoENeg *= rhoNeg;
                rhs[0] = -(aPos * rhoPos + aNeg * rhoNeg + (rhoNeg - rhoPos) * a1) * a0;
                for (int k = 0; k < D; ++k) {
                    const double phiUp = (aPos * rhoUPos[k] + aNeg * rhoUNeg[k] + (rhoUNeg[k] - rhoUPos[k]) * a1) * a0 +
                                         (pPos * psiPos - pNeg * psiNeg) * a0 * S[k];
                    rhs[k + 1] = -phiUp;
                }
                rhs[D + 1] = -(aPos * rhoEPos + aNeg * rhoENeg + (rhoENeg - rhoEPos) * a1 + (aPos * pPos + aNeg * pNeg)) * a0;
            } else {
                const double rhoavg = 0.5 * (Q(P, 0, i) + Q(P, 0, j));
                const double rhoavg_inv = 1.0 / rhoavg;
                double rhoUavg[MAXD], uavg[MAXD];
                for (int k = 0; k < D; ++k) rhoUavg[k] = 0.5 * (Q(P, k + 1, i) + Q(P, k + 1, j));
                const double Rpsiavg = 0.5 * (cell_Rpsi + adjc_Rpsi);
                double pavg = rhoavg * Rpsiavg;
                const double cell_H = Q(P, D + 1, i) / Q(P, 0, i) + cell_Rpsi;
                const double adjc_H = Q(P, D + 1, j) / Q(P, 0, j) + adjc_Rpsi;
                const double Havg = 0.5 * (cell_H + adjc_H);
                const double cP = sqrt(gamma * cell_Rpsi), cN = sqrt(gamma * adjc_Rpsi);
                const double cavg = 0.5 * (cP + cN);
                if (solver == LFM_SOLVER_M2AUSM) {
                    double cell_divu = 0., neigh_divu = 0., cell_curlu = 0., neigh_curlu = 0.;
                    double cell_vmag = 0., neigh_vmag = 0., unPos = 0., unNeg = 0., norm = 0.;
                    const double* gi = &P->dudx[i * D * D];
                    const double* gj = &P->dudx[j * D * D];
                    for (int a = 0; a < D; ++a) {
                        cell_divu += gi[a * D + a];
                        neigh_divu += gj[a * D + a];
                        for (int b = a + 1; b < D; ++b) {
                            cell_curlu += (gi[a * D + b] - gi[b * D + a]) * (gi[a * D + b] - gi[b * D + a]);
                            neigh_curlu += (gj[a * D + b] - gj[b * D + a]) * (gj[a * D + b] - gj[b * D + a]);
                        }
                        const double cu = Q(P, a + 1, i) / Q(P, 0, i);
                        cell_vmag += cu * cu;
                        const double nu = Q(P, a + 1, j) / Q(P, 0, j);
                        neigh_vmag += nu * nu;
                        const double uPos = minmod_interp(cu, nu, &P->UGrad[i * D * D + a * D], d, weight, 1.0, D);
                        const double uNeg = minmod_interp(cu, nu, &P->UGrad[j * D * D + a * D], d, weight, -1.0, D);
                        unPos += uPos * S[a];
                        unNeg += uNeg * S[a];
                        norm += S[a] * S[a];
                    }
                    const double cell_theta = dmax(-(cell_divu / sqrt(cell_divu * cell_divu + cell_curlu + 4e-2)), 0.);
                    const double neigh_theta =
                        dmax(-(neigh_divu / sqrt(neigh_divu * neigh_divu + neigh_curlu + 4e-2)), 0.);
                    const double theta_avg = 0.5 * (cell_theta + neigh_theta);
                    double r = Q(P, 0, i), E = Q(P, D + 1, i) / r;
                    const double cell_p = r * P->gm1 * (E - 0.5 * cell_vmag);
                    r = Q(P, 0, j);
                    E = Q(P, D + 1, j) / r;
                    const double neigh_p = r * P->gm1 * (E - 0.5 * neigh_vmag);
                    const double rhoPos = minmod_interp(Q(P, 0, i), Q(P, 0, j), &P->rhoGrad[i * D], d, weight, 1.0, D);
                    const double rhoNeg = minmod_interp(Q(P, 0, i), Q(P, 0, j), &P->rhoGrad[j * D], d, weight, -1.0, D);
                    const double pPos = minmod_interp(cell_p, neigh_p, &P->pGrad[i * D], d, weight, 1.0, D);
                    const double pNeg = minmod_interp(cell_p, neigh_p, &P->pGrad[j * D], d, weight, -1.0, D);
                    const double Msq = (unPos * unPos + unNeg * unNeg) / (2. * cavg * cavg * norm);
                    const double MPos = unPos / (sqrt(norm) * cavg);
                    const double MNeg = unNeg / (sqrt(norm) * cavg);
                    const double Minf = 0.2;
                    const double M0 = sqrt(dmin(1.0, dmax(Msq, Minf * Minf)));
                    const double fa = M0 * (2.0 - M0);
                    const double alpha = 3.0 * (5.0 * fa * fa - 4.0) / 16.0;
                    const double phalf =
                        pNeg * (p5Pos(MNeg, alpha) - p5Neg(MNeg, alpha)) - pPos * (p5Pos(MPos, alpha) - p5Neg(MPos, alpha));
                    const double pu =
                        -0.75 * p5Pos(MPos, alpha) * p5Neg(MNeg, alpha) * (rhoPos + rhoNeg) * cavg * fa * (unNeg - unPos);
                    pavg += theta_avg * (pu - 0.5 * phalf);
                }
                double phiavg = 0.0;
                for (int k = 0; k < D; ++k) {
                    uavg[k] = rhoUavg[k] * rhoavg_inv;
                    phiavg += uavg[k] * S[k];
                }
                rhs[0] = -rhoavg * phiavg;
                for (int k = 0; k < D; ++k) rhs[k + 1] = -(rhoUavg[k] * phiavg + pavg * S[k]);
                rhs[D + 1] = -(rhoavg * Havg * phiavg);
            }

            /* viscous face terms (src/cfd_v0.cpp:2682-2796) */
            double dudx[MAXD][MAXD], dTdx[MAXD], tau[MAXD][MAXD], tauMC[MAXD][MAXD];
            const double* gi = &P->dudx[i * D * D];
            const double* gj = &P->dudx[j * D * D];
            for (int a = 0; a < D; ++a) {
                for (int b = 0; b < D; ++b) dudx[a][b] = interp(weight, gi[a * D + b], gj[a * D + b]);
                dTdx[a] = interp(weight, P->dTdx[i * D + a], P->dTdx[j * D + a]);
            }
            if (ghost) {
                for (int a = 0; a < D; ++a) {
                    for (int b = 0; b < D; ++b) dudx[a][b] = (aU[a] - cU[a]) * dn[b] * dmag_inv;
                    dTdx[a] = (adjc_T - cell_T) * dn[a] * dmag_inv;
                }
            }
            {
                double flat[MAXD * MAXD];
                for (int a = 0; a < D; ++a)
                    for (int b = 0; b < D; ++b) flat[a * D + b] = dudx[a][b];
                stress(flat, mu, D, tau);
            }
            const double k_cond = c->Cp * mu * c->PrInv;
            for (int a = 0; a < D; ++a)
                for (int b = 0; b < D; ++b)
                    tauMC[a][b] = interp(weight, P->tauMC[i * D * D + a * D + b], P->tauMC[j * D * D + a * D + b]);
            if (ghost) {
                double diagSum = 0;
                for (int a = 0; a < D; ++a) diagSum -= dudx[a][a];
                diagSum *= mu * 2.0 / 3.0;
                for (int a = 0; a < D; ++a) {
                    for (int b = 0; b < D; ++b) tauMC[a][b] = mu * dudx[b][a];
                    tauMC[a][a] += diagSum;
                }
            }
            double divTauMC[MAXD], lapU[MAXD], sigmaU[MAXD];
            for (int a = 0; a < D; ++a) divTauMC[a] = dot(tauMC[a], S, D);
            for (int a = 0; a < D; ++a) lapU[a] = mu * (delta_mag * (aU[a] - cU[a]) * dmag_inv + dot(Kf, dudx[a], D));
            const double lapT = k_cond * (delta_mag * (adjc_T - cell_T) * dmag_inv + dot(Kf, dTdx, D));
            for (int a = 0; a < D; ++a) sigmaU[a] = interp(weight, P->sigmaU[i * D + a], P->sigmaU[j * D + a]);
            if (ghost) {
                double Uf[MAXD];
                for (int a = 0; a < D; ++a) Uf[a] = interp(weight, cU[a], aU[a]);
                for (int a = 0; a < D; ++a) sigmaU[a] = dot(Uf, tau[a], D);
            }
            const double divSigmaU = dot(sigmaU, S, D);
            for (int a = 0; a < D; ++a) rhs[a + 1] += divTauMC[a] + lapU[a];
            rhs[D + 1] += divSigmaU + lapT;

            if (resCheck) {
                for (int v = 0; v < nq; ++v) {
                    P->res[(int64_t)v * (P->nc + P->ng) + i] += rhs[v];
                    P->res[(int64_t)v * (P->nc + P->ng) + j] -= rhs[v];
                }
            }
            for (int v = 0; v < nq; ++v) {
                P->dq[(int64_t)v * P->nc + i] += dt * rhs[v] * P->volInvAll[i];
                if (j < P->nc) P->dq[(int64_t)v * P->nc + j] -= dt * rhs[v] * P->volInvAll[j];
            }
        }
        /* sponge layer and stage update (src/cfd_v0.cpp:2807-2822) */
        const double sg = c->sponge[i];
        P->dq[i] += dt * sg * (c->rhoInf - Q(P, 0, i));
        for (int k = 0; k < D; ++k) P->dq[(int64_t)(k + 1) * P->nc + i] += dt * sg * (c->rhoInf * c->UInf[k] - Q(P, k + 1, i));
        P->dq[(int64_t)(D + 1) * P->nc + i] += dt * sg * (c->rhoInf * c->EInf - Q(P, D + 1, i));
        for (int v = 0; v < nq; ++v) *Qp(P, v, i) += c->rkB[rk] * P->dq[(int64_t)v * P->nc + i];
    }
}

static int port_init(Port* P, const lfm_solver_desc* c) {
    memset(P, 0, sizeof(*P));
    P->c = c;
    P->D = c->dim;
    P->nq = c->nq;
    P->nc = c->n_cells;
    P->ng = c->n_ghosts;
    P->nf = c->n_faces;
    const int64_t nt = P->nc + P->ng;
    const int D = P->D;
    P->q = (double*)calloc((size_t)(P->nq * nt), sizeof(double));
    P->dq = (double*)calloc((size_t)(P->nq * P->nc), sizeof(double));
    P->res = (double*)calloc((size_t)(P->nq * nt), sizeof(double));
    P->dudx = (double*)calloc((size_t)(nt * D * D), sizeof(double));
    P->dTdx = (double*)calloc((size_t)(nt * D), sizeof(double));
    P->tauMC = (double*)calloc((size_t)(nt * D * D), sizeof(double));
    P->sigmaU = (double*)calloc((size_t)(nt * D), sizeof(double));
    P->rhoGrad = (double*)calloc((size_t)(nt * D), sizeof(double));
    P->pGrad = (double*)calloc((size_t)(nt * D), sizeof(double));
    P->UGrad = (double*)calloc((size_t)(nt * D * D), sizeof(double));
    P->volInvAll = (double*)calloc((size_t)nt, sizeof(double));
    P->faceStart = (int64_t*)calloc((size_t)(P->nc + 1), sizeof(int64_t));
    if (!P->q || !P->dq || !P->res || !P->dudx || !P->dTdx || !P->tauMC || !P->sigmaU || !P->rhoGrad ||
        !P->pGrad || !P->UGrad || !P->volInvAll || !P->faceStart)
        return -1;
    for (int64_t i = 0; i < P->nc; ++i) P->volInvAll[i] = c->vol_inv[i];
    for (int64_t f = 0; f < P->nf; ++f) P->faceStart[c->face_p[f] + 1] = f + 1;
    for (int64_t i = 0; i < P->nc; ++i)
        if (P->faceStart[i + 1] < P->faceStart[i]) P->faceStart[i + 1] = P->faceStart[i];
    P->Rinv = 1.0 / c->Rgas;
    P->gm1 = c->gamma - 1.0;
    return 0;
}

static void port_free(Port* P) {
    free(P->q);
    free(P->dq);
    free(P->res);
    free(P->dudx);
    free(P->dTdx);
    free(P->tauMC);
    free(P->sigmaU);
    free(P->rhoGrad);
    free(P->pGrad);
    free(P->UGrad);
    free(P->volInvAll);
    free(P->faceStart);
}

static int port_run(const lfm_solver_desc* c, double* q, int nsteps, double dt, double* residual,
                    double* cell_res) {
    Port P;
    if (!c || !q || c->dim < 2 || c->dim > 3) return -1;
    if (port_init(&P, c) != 0) {
        port_free(&P);
        return -4;
    }
    const int D = P.D, nq = P.nq;
    const int64_t nc = P.nc, nt = P.nc + P.ng;
    for (int v = 0; v < nq; ++v) memcpy(&P.q[(int64_t)v * nt], &q[(int64_t)v * nc], (size_t)nc * sizeof(double));
    for (int step = 0; step < nsteps; ++step) {
        memset(P.dq, 0, (size_t)(nq * nc) * sizeof(double));
        memset(P.res, 0, (size_t)(nq * nt) * sizeof(double));
        for (int rk = 0; rk < c->rk_order; ++rk) {
            for (int64_t k = 0; k < nq * nc; ++k) P.dq[k] *= c->rkA[rk];
            memset(P.dudx, 0, (size_t)(nc * D * D) * sizeof(double));
            memset(P.dTdx, 0, (size_t)(nc * D) * sizeof(double));
            memset(P.tauMC, 0, (size_t)(nc * D * D) * sizeof(double));
            memset(P.rhoGrad, 0, (size_t)(nc * D) * sizeof(double));
            if (c->solver == LFM_SOLVER_M2AUSM) {
                memset(P.pGrad, 0, (size_t)(nc * D) * sizeof(double));
                memset(P.UGrad, 0, (size_t)(nc * D * D) * sizeof(double));
            }
            set_boundary_conditions(&P);
            if (c->minmod && c->solver == LFM_SOLVER_M2AUSM) calc_gradients_ausm(&P);
            calc_VIS(&P);
            rk_step(&P, rk, dt, c->residuals && rk == 0);
        }
        if (residual && c->residuals) {
            for (int v = 0; v < nq; ++v) {
                double s = 0;
                for (int64_t i = 0; i < nc; ++i) s += P.res[(int64_t)v * nt + i] * P.res[(int64_t)v * nt + i];
                residual[v] = s;
            }
        }
        if (cell_res && c->residuals)
            for (int v = 0; v < nq; ++v)
                memcpy(&cell_res[(int64_t)v * nc], &P.res[(int64_t)v * nt], (size_t)nc * sizeof(double));
    }
    for (int v = 0; v < nq; ++v) memcpy(&q[(int64_t)v * nc], &P.q[(int64_t)v * nt], (size_t)nc * sizeof(double));
    port_free(&P);
    return 0;
}

int lfm_port_run(const lfm_solver_desc* c, double* q, int nsteps, double dt, double* residual) {
    return port_run(c, q, nsteps, dt, residual, NULL);
}

int lfm_port_run_cell_residual(const lfm_solver_desc* c, double* q, int nsteps, double dt, double* cell_res) {
    return port_run(c, q, nsteps, dt, NULL, cell_res);
}

int lfm_port_cfl(const lfm_solver_desc* c, const double* q, double dt, double* cfl_out) {
    const int D = c->dim;
    const int64_t nc = c->n_cells;
    double cfl_max = 0.;
    for (int64_t i = 0; i < nc; ++i) {
        double cfl = 0;
        const double rho_inv = 1.0 / q[i];
        for (int64_t e = c->cell_s_offsets[i]; e < c->cell_s_offsets[i + 1]; ++e) {
            double flux = 0.;
            for (int k = 0; k < D; ++k) flux += q[(int64_t)(k + 1) * nc + i] * c->cell_s[e * D + k];
            cfl += fabs(flux);
        }
        cfl *= rho_inv * c->vol_inv[i] * dt;
        if (cfl_max < cfl) cfl_max = cfl;
    }
    *cfl_out = cfl_max;
    return 0;
}

int lfm_port_min_dt(const lfm_solver_desc* c, const double* q, double max_co, double* dt_out) {
    const int D = c->dim;
    const int64_t nc = c->n_cells;
    double dt_min = 100.0;
    for (int64_t i = 0; i < nc; ++i) {
        double sumFlux = 0;
        const double rho = q[i];
        for (int64_t e = c->cell_s_offsets[i]; e < c->cell_s_offsets[i + 1]; ++e) {
            const double* S = &c->cell_s[e * D];
            double sMag = 0.;
            for (int k = 0; k < D; ++k) sMag += S[k] * S[k];
            sMag = sqrt(sMag);
            double flux = 0.;
            for (int k = 0; k < D; ++k) flux += q[(int64_t)(k + 1) * nc + i] * S[k] / sMag;
            sumFlux += fabs(flux);
        }
        const double vol = 1.0 / c->vol_inv[i];
        const double dt = max_co * rho * 2.0 * vol / sumFlux;
        if (dt_min > dt) dt_min = dt;
    }
    *dt_out = dt_min;
    return 0;
}
