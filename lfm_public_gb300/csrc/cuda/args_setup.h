// Host-side set-up shared by the single-case solver and the batch engine:
// validation of a solver description, the device index arrays derived from
// it, and the scalar constants of the kernel arguments.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../host/capi_internal.h"
#include "lfm_gpu.h"
#include "solver_kernels.cuh"

namespace lfm {
namespace setup {

inline int validateDesc(const lfm_solver_desc* d) {
    if (!d) return lfm::setError(LFM_ERR_INVALID, "null solver description");
    if (d->dim != 2 && d->dim != 3) return lfm::setError(LFM_ERR_INVALID, "dim must be 2 or 3");
    if (d->nq != d->dim + 2) return lfm::setError(LFM_ERR_INVALID, "nq must be dim + 2");
    if (d->solver < 0 || d->solver > 2) return lfm::setError(LFM_ERR_INVALID, "unknown solver");
    if (d->n_cells <= 0 || d->n_faces <= 0 || d->n_ghosts < 0)
        return lfm::setError(LFM_ERR_INVALID, "empty mesh");
    if (d->n_cells + d->n_ghosts + d->n_halos > 0x7fffffffLL / 32 || d->n_faces > 0x7fffffffLL / 8)
        return lfm::setError(LFM_ERR_UNSUPPORTED, "mesh too large for 32-bit device indexing");
    if (!d->face_p || !d->face_n || !d->face_ghost || !d->S || !d->d || !d->w || !d->smag || !d->dmag_inv ||
        !d->dnorm || !d->delta_mag || !d->K || !d->vol_inv || !d->sponge || !d->cell_face_offsets ||
        !d->cell_faces || !d->cell_face_sign || !d->cell_s_offsets || !d->cell_s ||
        (d->rk_order > 0 && (!d->rkA || !d->rkB)) ||
        (d->n_ghosts > 0 && (!d->ghost_cell || !d->ghost_kind)) ||
        (d->n_halos > 0 && (!d->halo_src_part || !d->halo_src_cell)))
        return lfm::setError(LFM_ERR_INVALID, "incomplete solver description");
    if (d->n_halos < 0) return lfm::setError(LFM_ERR_INVALID, "negative halo count");
    // rkOrder 0 runs no stage (the reference's stage loop runs rkOrder times)
    if (d->rk_order < 0 || d->rk_order > 8) return lfm::setError(LFM_ERR_INVALID, "rk_order out of range");
    const int64_t nt = d->n_cells + d->n_ghosts + d->n_halos;
    for (int64_t f = 0; f < d->n_faces; ++f) {
        if (d->face_p[f] < 0 || d->face_p[f] >= d->n_cells || d->face_n[f] < 0 || d->face_n[f] >= nt)
            return lfm::setError(LFM_ERR_INVALID, "face index out of range at face " + std::to_string(f));
        if (f > 0 && d->face_p[f] < d->face_p[f - 1])
            return lfm::setError(LFM_ERR_INVALID, "faces are not in processing order");
    }
    for (int64_t g = 0; g < d->n_ghosts; ++g)
        if (d->ghost_cell[g] < 0 || d->ghost_cell[g] >= d->n_cells)
            return lfm::setError(LFM_ERR_INVALID, "ghost cell out of range");
    for (int64_t c = 0; c < d->n_cells; ++c) {
        if (d->cell_face_offsets[c + 1] < d->cell_face_offsets[c])
            return lfm::setError(LFM_ERR_INVALID, "cell_face_offsets not monotone");
    }
    for (int64_t e = 0; e < d->cell_face_offsets[d->n_cells]; ++e)
        if (d->cell_faces[e] < 0 || d->cell_faces[e] >= d->n_faces)
            return lfm::setError(LFM_ERR_INVALID, "cell_faces entry out of range");
    return LFM_OK;
}

// Which optional passes a case runs: the gradients only for M2AUSM with
// minmod; the viscous pass when mu != 0 or when M2AUSM reads dudx.
inline bool needGrad(const lfm_solver_desc* d) { return d->solver == LFM_SOLVER_M2AUSM && d->minmod; }
inline bool needVis(const lfm_solver_desc* d) { return d->mu != 0.0 || d->solver == LFM_SOLVER_M2AUSM; }

// 32-bit device index arrays of a description.
struct DescIndex {
    std::vector<int> fP, fN, cfOff, cfList, cfNbr, gCell, gKind, gFace;
    std::vector<double> lapc;   // |delta| / |d| per face

    explicit DescIndex(const lfm_solver_desc* d) {
        const size_t nf = (size_t)d->n_faces, nc = (size_t)d->n_cells, ng = (size_t)d->n_ghosts;
        fP.resize(nf);
        fN.resize(nf);
        lapc.resize(nf);
        for (size_t f = 0; f < nf; ++f) {
            fP[f] = (int)d->face_p[f];
            fN[f] = (int)d->face_n[f];
            lapc[f] = d->delta_mag[f] * d->dmag_inv[f];
        }
        cfOff.resize(nc + 1);
        for (size_t c = 0; c <= nc; ++c) cfOff[c] = (int)d->cell_face_offsets[c];
        const size_t ne = (size_t)d->cell_face_offsets[nc];
        cfList.resize(ne);
        // face index, one's complement when the cell is the face's N side,
        // and the cell (ghost, halo) across the face
        cfNbr.resize(ne);
        for (size_t k = 0; k < ne; ++k) {
            const int64_t f = d->cell_faces[k];
            cfList[k] = d->cell_face_sign[k] > 0 ? (int)f : ~(int)f;
            cfNbr[k] = (int)(d->cell_face_sign[k] > 0 ? d->face_n[f] : d->face_p[f]);
        }
        gCell.resize(ng);
        gKind.resize(ng);
        gFace.assign(ng, 0);
        for (size_t g = 0; g < ng; ++g) {
            gCell[g] = (int)d->ghost_cell[g];
            gKind[g] = d->ghost_kind[g];
        }
        for (size_t f = 0; f < nf; ++f)   // ghosts only (halos follow them)
            if (fN[f] >= (int)nc && fN[f] < (int)(nc + ng)) gFace[(size_t)fN[f] - nc] = (int)f;
    }
};

// Scalar constants of the kernel arguments (counts, gas constants, free
// stream, and the reference state of the FP32-bulk perturbation form).
template <typename T>
void setConstants(dev::Args<T>& a, const lfm_solver_desc* d) {
    a.D = d->dim;
    a.nq = d->nq;
    a.nc = (int)d->n_cells;
    a.ng = (int)d->n_ghosts;
    a.nf = (int)d->n_faces;
    a.nh = (int)d->n_halos;
    a.nt = a.nc + a.ng + a.nh;
    a.gamma = d->gamma;
    a.gm1 = d->gamma - 1.0;
    a.Rinv = 1.0 / d->Rgas;
    a.rhoInf = d->rhoInf;
    a.EInf = d->EInf;
    a.pInf = d->pInf;
    a.TInf = d->TInf;
    for (int k = 0; k < 3; ++k) a.UInf[k] = d->UInf[k];
    a.mu = d->mu;
    a.kcond = d->Cp * d->mu * d->PrInv;
    // Reference state of the FP32 perturbation form: any constant state works
    // (its flux through a closed cell sums to zero); the free stream keeps the
    // perturbations small. Its pressure follows from q_ref.
    const int D = d->dim;
    double u2 = 0.0;
    for (int k = 0; k < D; ++k) u2 += d->UInf[k] * d->UInf[k];
    a.qRef[0] = d->rhoInf;
    for (int k = 0; k < 3; ++k) a.qRef[1 + k] = 0.0;
    for (int k = 0; k < D; ++k) a.qRef[1 + k] = d->rhoInf * d->UInf[k];
    a.qRef[D + 1] = d->rhoInf * d->EInf;
    const double pRef = (d->gamma - 1.0) * (a.qRef[D + 1] - 0.5 * d->rhoInf * u2);
    const double RpsiRef = pRef / d->rhoInf;
    const double gh = d->gamma / (d->gamma - 1.0);
    a.pRef = pRef;
    a.gh = gh;
    a.mu23 = d->mu * 2.0 / 3.0;
    a.ref.rho = (float)d->rhoInf;
    for (int k = 0; k < 3; ++k) {
        a.ref.U[k] = k < D ? (float)d->UInf[k] : 0.0f;
        a.ref.m[k] = k < D ? (float)(d->rhoInf * d->UInf[k]) : 0.0f;
    }
    a.ref.Rpsi = (float)RpsiRef;
    a.ref.p = (float)pRef;
    a.ref.H = (float)(gh * RpsiRef + 0.5 * u2);
    a.ref.gh = (float)gh;
    a.ref.gamma = (float)d->gamma;
    a.ref.gm1 = (float)(d->gamma - 1.0);
    a.ref.Rinv = (float)(1.0 / d->Rgas);
    a.ref.mu = (float)d->mu;
    a.ref.kcond = (float)(d->Cp * d->mu * d->PrInv);
}

}  // namespace setup
}  // namespace lfm
