// Solver setup restated from the reference (file:line ranges in case_setup.h).
#include "case_setup.h"

#include "renumber.h"

#include <algorithm>
#include <tuple>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <stdexcept>

#include "lfm_gpu.h"
#include "meshReader.h"

namespace lfm {

void rkCoefficients(int rkOrder, std::vector<double>& A, std::vector<double>& B) {
    A.clear();
    B.clear();
    switch (rkOrder) {
        case 0:
        case 1:
            A = {0.0};
            B = {1.0};
            break;
        case 2:
            A = {0.0, -1.0};
            B = {1.0, 0.5};
            break;
        case 3:
        case 4:
            // Carpenter-Kennedy low-storage coefficients; rkOrder 3 runs the
            // first three stages of this four-stage set, as the reference does.
            A = {0.0, -756391.0 / 934407.0, -36441873.0 / 15625000.0, -1953125.0 / 1085297.0};
            B = {8.0 / 141.0, 6627.0 / 2000.0, 609375.0 / 1085297.0, 198961.0 / 526383.0};
            break;
        case 5:
            A = {0.0, -0.4178904745, -1.192151694643, -1.697784692471, -1.514183444257};
            B = {0.1496590219993, 0.3792103129999, 0.8229550293869, 0.6994504559488, 0.1530572479681};
            break;
        default:
            break;
    }
}

namespace {

struct Slot {            // one valid face of a cell, as the reference stores it
    int64_t face;        // polyMesh face label
    int nbType;          // 0 regular / submesh cell, 1 boundary ghost, 2 processor halo
    int64_t nbSolver;    // solver index of the neighbour cell (nbType 0)
    int nbSm;            // neighbour submesh (nbType 0)
    int64_t nbLocal;     // neighbour index inside its submesh (nbType 0)
    int bound;           // patch of a boundary face
    int nbProc;          // neighbouring partition (nbType 2)
    int64_t faceId;      // global face id (nbType 2)
    double S[3], d[3], w;
    bool owned;
};

}  // namespace

SolverCase buildSolverCase(IMeshReader& r, const CaseParams& prm, const HaloLookup* halos) {
    const int D = prm.dimension;
    if (D != 2 && D != 3) throw std::runtime_error("invalid dimension " + std::to_string(D));
    SolverCase sc;
    sc.dim = D;
    sc.nq = D + 2;

    // -- submeshes and solver order (src/mesh_reader.cpp:56-87) ----------------
    const int nSub = r.getSubmeshCount();
    std::vector<std::vector<int>> subCells((size_t)nSub);
    std::vector<int64_t> subOffset((size_t)nSub + 1, 0);
    for (int s = 0; s < nSub; ++s) {
        subCells[(size_t)s] = r.getSubmeshCellIndexList(s);
        subOffset[(size_t)s + 1] = subOffset[(size_t)s] + (int64_t)subCells[(size_t)s].size();
    }
    const int64_t nc = subOffset.back();
    if (nc != r.getCellCount()) throw std::runtime_error("submesh split does not cover every cell");
    // locality order of the cells inside each submesh (the polyMesh keeps its own)
    if (prm.renumber == RENUMBER_HPATH) {
        // one walk over the whole mesh; each submesh in the order of the walk
        const std::vector<int> order = hpathCellOrder(r);
        if (!order.empty()) {
            std::vector<int> rank((size_t)r.getCellCount());
            for (size_t i = 0; i < order.size(); ++i) rank[(size_t)order[i]] = (int)i;
            for (int s = 0; s < nSub; ++s)
                std::sort(subCells[(size_t)s].begin(), subCells[(size_t)s].end(),
                          [&](int a, int b) { return rank[(size_t)a] < rank[(size_t)b]; });
        }
    } else if (prm.renumber != RENUMBER_NONE) {
        for (int s = 0; s < nSub; ++s) renumberCells(r, subCells[(size_t)s], prm.renumber, D);
    }
    sc.nCells = nc;
    sc.nCells0 = nSub > 0 ? (int64_t)subCells[0].size() : 0;
    std::vector<int64_t> solverOf((size_t)nc), smOf((size_t)nc), localOf((size_t)nc);
    sc.cellId.resize((size_t)nc);
    for (int s = 0; s < nSub; ++s)
        for (size_t i = 0; i < subCells[(size_t)s].size(); ++i) {
            const int64_t cell = subCells[(size_t)s][i];
            const int64_t idx = subOffset[(size_t)s] + (int64_t)i;
            solverOf[(size_t)cell] = idx;
            smOf[(size_t)cell] = s;
            localOf[(size_t)cell] = (int64_t)i;
            sc.cellId[(size_t)idx] = cell;
        }

    // -- per cell-face geometry (setParams, calculateVNeighbour, init_params) ---
    std::vector<std::vector<Slot>> slots((size_t)nc);
    int maxF = 0;
    for (int64_t ci = 0; ci < nc; ++ci) {
        const int cell = (int)sc.cellId[(size_t)ci];
        double xc[3];
        r.getCellCenter(cell, xc);
        const int nValid = r.getCellValidFaceCount(cell);
        maxF = std::max(maxF, nValid);
        std::vector<Slot>& cs = slots[(size_t)ci];
        cs.resize((size_t)nValid);
        for (int k = 0; k < nValid; ++k) {
            Slot& sl = cs[(size_t)k];
            const int f = r.getCellValidFaceIndex(cell, k);
            sl.face = f;
            const int own = r.getFaceOwner(f);
            const int nbr = r.getFaceNeighbour(f);
            const int other = (own == cell) ? nbr : own;
            sl.bound = r.getFaceBoundary(f);
            if (other != -1) {
                sl.nbType = 0;
                sl.nbSolver = solverOf[(size_t)other];
                sl.nbSm = (int)smOf[(size_t)other];
                sl.nbLocal = localOf[(size_t)other];
            } else if (r.getBoundaryProcessorRank(sl.bound) == -1) {
                sl.nbType = 1;
            } else {
                if (!halos)
                    throw std::runtime_error("a processor patch needs its neighbouring partitions: open the "
                                             "decomposed case as a whole");
                sl.nbType = 2;
                sl.nbProc = r.getBoundaryProcessorRank(sl.bound);
                sl.faceId = r.getFaceId(f);
            }
            const double sign = (own == cell) ? 1.0 : -1.0;
            double an[3], xf[3];
            r.getFaceAreaNormal(f, an);
            r.getFaceCenter(f, xf);
            for (int dd = 0; dd < D; ++dd) sl.S[dd] = sign * an[dd];
            double dP[3];
            for (int dd = 0; dd < D; ++dd) dP[dd] = xc[dd] - xf[dd];
            if (sl.nbType == 2) {
                // neighbour centre from the other partition: its cell centre
                // relative to its face centre, plus this face's centre
                // relative to this cell (src/mesh_reader.cpp:548-601)
                double x[3] = {0, 0, 0};
                if (!halos->neighbourOffset(sl.nbProc, sl.faceId, x))
                    throw std::runtime_error("processor face " + std::to_string(sl.faceId) +
                                             " has no partner in partition " + std::to_string(sl.nbProc));
                for (int dd = 0; dd < D; ++dd) sl.d[dd] = sign * (x[dd] + xf[dd] - xc[dd]);
            } else if (sl.nbType == 1) {
                double smag2 = 0.0, dps = 0.0;
                for (int dd = 0; dd < D; ++dd) smag2 += sl.S[dd] * sl.S[dd];
                for (int dd = 0; dd < D; ++dd) dps += dP[dd] * sl.S[dd];
                for (int dd = 0; dd < D; ++dd) sl.d[dd] = 2.0 * std::fabs(dps) * sl.S[dd] / smag2;
            } else {
                // Neighbour-centre vector of the face, seen from its owner
                // (src/mesh_reader.cpp:418-442), then signed for this cell.
                double xo[3], xn[3], vn[3];
                r.getCellCenter(own, xo);
                r.getCellCenter(r.getFaceNeighbour(f), xn);
                for (int dd = 0; dd < D; ++dd) vn[dd] = xn[dd] - xo[dd];
                const int cyc = r.getCyclicFaceIndex(f);
                if (cyc != f) {
                    double xf1[3], xf2[3];
                    r.getFaceCenter(f, xf1);
                    r.getFaceCenter(cyc, xf2);
                    for (int dd = 0; dd < D; ++dd) vn[dd] += xf1[dd] - xf2[dd];
                }
                for (int dd = 0; dd < D; ++dd) sl.d[dd] = sign * vn[dd];
            }
            double dN[3];
            for (int dd = 0; dd < D; ++dd) dN[dd] = dP[dd] + sl.d[dd];
            double wnum = 0.0, wden = 0.0;
            for (int dd = 0; dd < D; ++dd) {
                wnum += sl.S[dd] * dN[dd];
                wden += (-sl.S[dd] * dP[dd] + sl.S[dd] * dN[dd]);
            }
            sl.w = wnum / wden;
            // Ownership (src/cfd_v0.cpp:295-305): boundary ghosts and MPI halos
            // rank above every cell (sm_id = MAX_MPI_RANKS, :428, :514).
            if (sl.nbType != 0) {
                sl.owned = true;
            } else {
                const int mySm = (int)smOf[(size_t)cell];
                const int64_t myLocal = localOf[(size_t)cell];
                sl.owned = !(sl.nbSm < mySm || (sl.nbSm == mySm && sl.nbLocal < myLocal));
            }
        }
        if (nValid > 0 && smOf[(size_t)cell] != 0)
            for (const Slot& sl : cs)
                if (sl.nbType == 1)
                    throw std::runtime_error(
                        "a boundary face belongs to an interior-submesh cell; the reference allocates boundary "
                        "ghosts only for submesh 0 (src/cfd_v0.cpp:352-353)");
    }
    sc.maxFacesPerCell = maxF;

    // -- patch -> boundary-condition kind (src/cfd_v0.cpp:972-1005) -------------
    const int nPatch = r.getBoundaryCount();
    std::vector<int> patchKind((size_t)nPatch, GHOST_NONE);
    for (int b = 0; b < nPatch; ++b) {
        const std::string type = r.getBoundaryType(b), name = r.getBoundaryName(b);
        if (type == "wall") patchKind[(size_t)b] = GHOST_WALL;
        if (type == "farfield") patchKind[(size_t)b] = GHOST_FARFIELD;
        if (type == "patch") {
            if (name == "inlet" || name == "Inlet" || name == "Inflow" || name == "inflow")
                patchKind[(size_t)b] = GHOST_INLET;
            if (name == "outlet" || name == "Outlet" || name == "Outflow" || name == "outflow")
                patchKind[(size_t)b] = GHOST_OUTLET;
        }
    }

    // -- flux faces in processing order, ghosts, per-face constants -------------
    for (int64_t ci = 0; ci < nc; ++ci)
        for (const Slot& sl : slots[(size_t)ci])
            if (sl.owned) ++sc.nFaces;
    const int64_t nf = sc.nFaces;
    sc.faceP.resize((size_t)nf);
    sc.faceN.resize((size_t)nf);
    sc.faceGhost.assign((size_t)nf, 0);
    sc.S.assign((size_t)(D * nf), 0.0);
    sc.d.assign((size_t)(D * nf), 0.0);
    sc.w.resize((size_t)nf);
    sc.Smag.resize((size_t)nf);
    sc.dmagInv.resize((size_t)nf);
    sc.dnorm.assign((size_t)(D * nf), 0.0);
    sc.deltaMag.resize((size_t)nf);
    sc.K.assign((size_t)(D * nf), 0.0);
    int64_t fi = 0;
    for (int64_t ci = 0; ci < nc; ++ci) {
        for (const Slot& sl : slots[(size_t)ci]) {
            if (!sl.owned) continue;
            sc.faceP[(size_t)fi] = ci;
            if (sl.nbType == 2) {
                // halos follow the ghosts: N fixed up once the ghosts are counted
                sc.faceN[(size_t)fi] = -1 - (int64_t)sc.haloFace.size();
                sc.haloFace.push_back(fi);
                sc.haloProc.push_back(sl.nbProc);
                sc.haloFaceId.push_back(sl.faceId);
                sc.haloCell.push_back(ci);
            } else if (sl.nbType == 1) {
                const int64_t g = (int64_t)sc.ghostCell.size();
                sc.ghostCell.push_back(ci);
                sc.ghostKind.push_back(patchKind[(size_t)sl.bound]);
                sc.ghostFace.push_back(fi);
                sc.ghostPatch.push_back(sl.bound);
                sc.faceN[(size_t)fi] = nc + g;
                sc.faceGhost[(size_t)fi] = 1;
            } else {
                sc.faceN[(size_t)fi] = sl.nbSolver;
            }
            for (int dd = 0; dd < D; ++dd) {
                sc.S[(size_t)(dd * nf + fi)] = sl.S[dd];
                sc.d[(size_t)(dd * nf + fi)] = sl.d[dd];
            }
            sc.w[(size_t)fi] = sl.w;
            // The reference's per-face expressions, evaluated once.
            double dm = sl.d[0] * sl.d[0];
            for (int dd = 1; dd < D; ++dd) dm += sl.d[dd] * sl.d[dd];
            dm = std::sqrt(dm);
            const double dinv = 1.0 / dm;
            double smag = 0.0;
            for (int dd = 0; dd < D; ++dd) smag += sl.S[dd] * sl.S[dd];
            smag = std::sqrt(smag);
            double sd = sl.S[0] * sl.d[0];
            for (int dd = 1; dd < D; ++dd) sd += sl.S[dd] * sl.d[dd];
            double dmag = 0.0;
            for (int dd = 0; dd < D; ++dd) {
                const double delta = sl.d[dd] * smag * smag / sd;
                dmag += delta * delta;
                sc.K[(size_t)(dd * nf + fi)] = sl.S[dd] - delta;
                sc.dnorm[(size_t)(dd * nf + fi)] = sl.d[dd] * dinv;
            }
            sc.Smag[(size_t)fi] = smag;
            sc.dmagInv[(size_t)fi] = dinv;
            sc.deltaMag[(size_t)fi] = std::sqrt(dmag);
            ++fi;
        }
    }
    sc.nGhosts = (int64_t)sc.ghostCell.size();
    sc.nHalos = (int64_t)sc.haloFace.size();
    for (int64_t h = 0; h < sc.nHalos; ++h) sc.faceN[(size_t)sc.haloFace[(size_t)h]] = nc + sc.nGhosts + h;

    // -- cell -> face incidence (ascending face index) --------------------------
    std::vector<int64_t> cnt((size_t)nc, 0);
    for (int64_t f = 0; f < nf; ++f) {
        ++cnt[(size_t)sc.faceP[(size_t)f]];
        if (sc.faceN[(size_t)f] < nc) ++cnt[(size_t)sc.faceN[(size_t)f]];
    }
    sc.cellFaceOffsets.assign((size_t)nc + 1, 0);
    for (int64_t c = 0; c < nc; ++c) sc.cellFaceOffsets[(size_t)c + 1] = sc.cellFaceOffsets[(size_t)c] + cnt[(size_t)c];
    sc.cellFaces.resize((size_t)sc.cellFaceOffsets.back());
    sc.cellFaceSign.resize((size_t)sc.cellFaceOffsets.back());
    std::vector<int64_t> fill(sc.cellFaceOffsets.begin(), sc.cellFaceOffsets.end() - 1);
    for (int64_t f = 0; f < nf; ++f) {
        const int64_t p = sc.faceP[(size_t)f], n = sc.faceN[(size_t)f];
        sc.cellFaces[(size_t)fill[(size_t)p]] = f;
        sc.cellFaceSign[(size_t)fill[(size_t)p]++] = 1;
        if (n < nc) {
            sc.cellFaces[(size_t)fill[(size_t)n]] = f;
            sc.cellFaceSign[(size_t)fill[(size_t)n]++] = -1;
        }
    }

    // -- per cell S of every valid face in the reordered slot order --------------
    sc.cellSOffsets.assign((size_t)nc + 1, 0);
    for (int64_t c = 0; c < nc; ++c)
        sc.cellSOffsets[(size_t)c + 1] = sc.cellSOffsets[(size_t)c] + (int64_t)slots[(size_t)c].size();
    sc.cellS.assign((size_t)(sc.cellSOffsets.back() * D), 0.0);
    for (int64_t c = 0; c < nc; ++c) {
        const std::vector<Slot>& cs = slots[(size_t)c];
        std::vector<const Slot*> order;
        for (const Slot& sl : cs)
            if (sl.owned) order.push_back(&sl);
        for (size_t k = cs.size(); k-- > 0;)
            if (!cs[k].owned) order.push_back(&cs[k]);
        for (size_t k = 0; k < order.size(); ++k)
            for (int dd = 0; dd < D; ++dd)
                sc.cellS[(size_t)((sc.cellSOffsets[(size_t)c] + (int64_t)k) * D + dd)] = order[k]->S[dd];
    }

    // -- constants and initial state (src/cfd_v0.cpp:866-967) --------------------
    sc.solver = prm.solver;
    sc.rkOrder = prm.rkOrder;
    sc.minmod = prm.minmod;
    sc.residuals = prm.residuals;
    rkCoefficients(prm.rkOrder, sc.rkA, sc.rkB);
    sc.pInf = prm.pInf;
    sc.TInf = prm.TInf;
    for (int dd = 0; dd < 3; ++dd) sc.UInf[dd] = (dd < D) ? prm.UInf[dd] : 0.0;
    sc.mu = prm.mu;
    sc.Cp = prm.Cp;
    sc.Rgas = 8.31447 / prm.molWeight * 1000;
    const double Cv = prm.Cp - sc.Rgas;
    sc.gamma = prm.Cp / Cv;
    sc.rhoInf = prm.pInf / (sc.Rgas * prm.TInf);
    const double gm1 = sc.gamma - 1.0;
    double u2 = 0;
    for (int dd = 0; dd < D; ++dd) u2 += sc.UInf[dd] * sc.UInf[dd];
    sc.EInf = prm.pInf / (sc.rhoInf * gm1) + 0.5 * u2;
    sc.PrInv = 1.0 / prm.Pr;

    sc.volInv.resize((size_t)nc);
    sc.sponge.assign((size_t)nc, 0.0);
    for (int64_t c = 0; c < nc; ++c) sc.volInv[(size_t)c] = 1.0 / r.getCellVolume((int)sc.cellId[(size_t)c]);
    if (!prm.laminar) {
        // Smagorinsky model constant of each cell, -2 (Cs Delta)^2 with
        // Cs = 0.16 and Delta = V^(1/3), evaluated as calc_VIS_Smagorinsky
        // does (src/cfd_v0.cpp:1601)
        sc.smagC.resize((size_t)nc);
        for (int64_t c = 0; c < nc; ++c)
            sc.smagC[(size_t)c] = -(double)2.0 * std::pow((double)0.16 * std::pow(1.0 / sc.volInv[(size_t)c], 1. / 3.), 2);
    }
    if (prm.Ls > 0) {
        const double sigma0 = 3.0 * (1.0 - prm.mach * prm.mach) / (prm.kSponge * prm.Ls);
        const int ia = r.readScalarField("alpha");
        for (int64_t c = 0; c < nc; ++c) {
            const double dist = r.getCellScalar((int)sc.cellId[(size_t)c], ia);
            if (dist < prm.Ls) {
                const double x = (prm.Ls - dist) / prm.Ls;
                sc.sponge[(size_t)c] = sigma0 * (x * x);
            }
        }
    }
    const int ip = r.readScalarField("p");
    const int it = r.readScalarField("T");
    const int iu = r.readVectorField("U");
    sc.q0.assign((size_t)(sc.nq * nc), 0.0);
    for (int64_t c = 0; c < nc; ++c) {
        const int cell = (int)sc.cellId[(size_t)c];
        double U[3];
        r.getCellVector(cell, iu, U);
        const double p = r.getCellScalar(cell, ip);
        const double T = r.getCellScalar(cell, it);
        double um2 = 0;
        for (int dd = 0; dd < D; ++dd) um2 += U[dd] * U[dd];
        const double rho = p / (sc.Rgas * T);
        const double E = p / (rho * gm1) + 0.5 * um2;
        sc.q0[(size_t)c] = rho;
        for (int dd = 0; dd < D; ++dd) sc.q0[(size_t)((dd + 1) * nc + c)] = rho * U[dd];
        sc.q0[(size_t)((D + 1) * nc + c)] = rho * E;
    }
    return sc;
}


void resolveHalos(std::vector<SolverCase>& parts) {
    // (partition across, face id) -> halo index, per partition
    std::vector<std::map<std::pair<int, int64_t>, int64_t>> index(parts.size());
    for (size_t p = 0; p < parts.size(); ++p)
        for (int64_t h = 0; h < parts[p].nHalos; ++h)
            index[p][{parts[p].haloProc[(size_t)h], parts[p].haloFaceId[(size_t)h]}] = h;
    for (size_t p = 0; p < parts.size(); ++p) {
        SolverCase& sc = parts[p];
        sc.haloSrcPart.assign((size_t)sc.nHalos, -1);
        sc.haloSrcCell.assign((size_t)sc.nHalos, -1);
        for (int64_t h = 0; h < sc.nHalos; ++h) {
            const int q = sc.haloProc[(size_t)h];
            if (q < 0 || q >= (int)parts.size())
                throw std::runtime_error("processor patch refers to partition " + std::to_string(q) + " of " +
                                         std::to_string(parts.size()));
            auto it = index[(size_t)q].find({(int)p, sc.haloFaceId[(size_t)h]});
            if (it == index[(size_t)q].end())
                throw std::runtime_error("processor face " + std::to_string(sc.haloFaceId[(size_t)h]) + " of partition " +
                                         std::to_string(p) + " has no partner in partition " + std::to_string(q));
            sc.haloSrcPart[(size_t)h] = q;
            sc.haloSrcCell[(size_t)h] = parts[(size_t)q].haloCell[(size_t)it->second];
        }
    }
}

void describeSolverCase(const SolverCase& s, lfm_solver_desc* d) {
    std::memset(d, 0, sizeof(*d));
    d->dim = s.dim;
    d->nq = s.nq;
    d->solver = s.solver;
    d->rk_order = s.rkOrder;
    d->minmod = s.minmod;
    d->residuals = s.residuals;
    d->n_cells = s.nCells;
    d->n_cells0 = s.nCells0;
    d->n_ghosts = s.nGhosts;
    d->n_faces = s.nFaces;
    d->face_p = s.faceP.data();
    d->face_n = s.faceN.data();
    d->face_ghost = s.faceGhost.data();
    d->S = s.S.data();
    d->d = s.d.data();
    d->w = s.w.data();
    d->smag = s.Smag.data();
    d->dmag_inv = s.dmagInv.data();
    d->dnorm = s.dnorm.data();
    d->delta_mag = s.deltaMag.data();
    d->K = s.K.data();
    d->vol_inv = s.volInv.data();
    d->sponge = s.sponge.data();
    d->ghost_cell = s.ghostCell.data();
    d->ghost_kind = s.ghostKind.data();
    d->cell_face_offsets = s.cellFaceOffsets.data();
    d->cell_faces = s.cellFaces.data();
    d->cell_face_sign = s.cellFaceSign.data();
    d->cell_s_offsets = s.cellSOffsets.data();
    d->cell_s = s.cellS.data();
    d->q0 = s.q0.data();
    d->gamma = s.gamma;
    d->Rgas = s.Rgas;
    d->rhoInf = s.rhoInf;
    d->EInf = s.EInf;
    d->pInf = s.pInf;
    d->TInf = s.TInf;
    for (int k = 0; k < 3; ++k) d->UInf[k] = s.UInf[k];
    d->mu = s.mu;
    d->Cp = s.Cp;
    d->PrInv = s.PrInv;
    d->rkA = s.rkA.data();
    d->rkB = s.rkB.data();
    d->n_halos = s.nHalos;
    d->halo_src_part = s.haloSrcPart.empty() ? nullptr : s.haloSrcPart.data();
    d->halo_src_cell = s.haloSrcCell.empty() ? nullptr : s.haloSrcCell.data();
    d->ghost_patch = s.ghostPatch.data();
    d->smag_c = s.smagC.empty() ? nullptr : s.smagC.data();
}

namespace {

// Offsets (cell centre - face centre) of the processor faces of every
// partition, keyed by (partition, partition across, face id).
class OffsetTable : public HaloLookup {
public:
    std::map<std::tuple<int, int, int64_t>, std::array<double, 3>> offsets;
    int self = 0;
    bool neighbourOffset(int nbr, int64_t faceId, double* x) const override {
        auto it = offsets.find(std::make_tuple(nbr, self, faceId));
        if (it == offsets.end()) return false;
        for (int k = 0; k < 3; ++k) x[k] = it->second[(size_t)k];
        return true;
    }
};

}  // namespace

std::vector<SolverCase> buildPartitionCases(const std::vector<IMeshReader*>& readers, const CaseParams& prm) {
    OffsetTable table;
    for (size_t p = 0; p < readers.size(); ++p) {
        IMeshReader& r = *readers[p];
        for (int b = 0; b < r.getBoundaryCount(); ++b) {
            const int q = r.getBoundaryProcessorRank(b);
            if (q < 0) continue;
            for (int f = r.getBoundaryFaceStart(b); f <= r.getBoundaryFaceEnd(b); ++f) {
                double xc[3], xf[3];
                r.getCellCenter(r.getFaceOwner(f), xc);
                r.getFaceCenter(f, xf);
                table.offsets[std::make_tuple((int)p, q, (int64_t)r.getFaceId(f))] = {xc[0] - xf[0], xc[1] - xf[1],
                                                                                       xc[2] - xf[2]};
            }
        }
    }
    std::vector<SolverCase> parts;
    for (size_t p = 0; p < readers.size(); ++p) {
        table.self = (int)p;
        parts.push_back(buildSolverCase(*readers[p], prm, &table));
        SolverCase& sc = parts.back();
        sc.cellGlobal.resize(sc.cellId.size());
        for (size_t c = 0; c < sc.cellId.size(); ++c) sc.cellGlobal[c] = readers[p]->getCellProcAddressing((int)sc.cellId[c]);
    }
    resolveHalos(parts);
    return parts;
}

}  // namespace lfm
