// C ABI, case half: case input and the flattened solver description
// (declarations and the reference interfaces they replace: include/lfm_gpu.h).
#include <array>
#include <cstring>
#include <exception>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "capi_internal.h"
#include "case_setup.h"
#include "foam_case.h"
#include "inputReader.h"
#include "lfm_gpu.h"
#include "dictReaderOF.h"
#include "polyMeshReaderOF.h"
#include "renumber.h"
#include "tiles.h"

struct lfm_case {
    lfm::SolverCase sc;
    double deltaT = 0, startTime = 0, endTime = 0, maxCo = 1;
    bool adjust = false;
};

namespace lfm {
thread_local std::string g_lastError;
int setError(int code, const std::string& msg) {
    g_lastError = msg;
    return code;
}
}  // namespace lfm

extern "C" const char* lfm_last_error(void) { return lfm::g_lastError.c_str(); }
extern "C" const char* lfm_version(void) { return "lfm_public_gb300 0.1 (sm_103a)"; }

static lfm::CaseParams paramsFromInput(const CInputReader& in) {
    lfm::CaseParams p;
    p.solver = in.m_nSolver;
    p.dimension = in.m_nDimension;
    p.rkOrder = in.m_nRkStepCount;
    p.minmod = in.m_bMinmodInterpolation;
    p.laminar = in.m_bisLaminar;
    p.residuals = in.m_bHaveResidual;
    p.pInf = in.m_dPInf;
    p.TInf = in.m_dTInf;
    for (int k = 0; k < 3; ++k) p.UInf[k] = in.m_dUInf[k];
    p.Ls = in.m_dLs;
    p.mach = in.m_dMach;
    p.kSponge = in.m_dK;
    p.Cp = in.m_dCp;
    p.molWeight = in.m_dMolWeight;
    p.mu = in.m_dMu0;
    p.Pr = in.m_dPrandtl;
    return p;
}

// controlDict lfm/renumber (none | rcm | hilbert): an extension of the
// reference's controlDict, which the reference ignores.
static int renumberOption(const std::string& root) {
    CDictReaderOF controlDict("controlDict", root + "/system");
    return lfm::renumberFromName(controlDict.readDictWord("renumber", "lfm", "none", true));
}

static int validateParams(const lfm::CaseParams& p) {
    if (p.solver < 0 || p.solver > 2) return lfm::setError(LFM_ERR_INVALID, "unknown solver type " + std::to_string(p.solver));
    if (p.dimension != 2 && p.dimension != 3)
        return lfm::setError(LFM_ERR_INVALID, "invalid dimension " + std::to_string(p.dimension));
    if (p.rkOrder < 0 || p.rkOrder > 5) return lfm::setError(LFM_ERR_INVALID, "rkOrder must be 0..5");
    if (p.renumber < LFM_RENUMBER_NONE || p.renumber > LFM_RENUMBER_HPATH)
        return lfm::setError(LFM_ERR_INVALID, "unknown renumbering (none, rcm, hilbert or hpath)");
    return LFM_OK;
}

extern "C" int lfm_case_open(const char* root, int rank, lfm_case** out) {
    if (!root || !out) return lfm::setError(LFM_ERR_INVALID, "lfm_case_open: null argument");
    *out = nullptr;
    try {
        CInputReader in;
        in.readCase(root);
        lfm::CaseParams prm = paramsFromInput(in);
        prm.renumber = renumberOption(root);
        int rc = validateParams(prm);
        if (rc) return rc;
        const std::string caseName = rank >= 0 ? "processor" + std::to_string(rank) : ".";
        std::unique_ptr<lfm::FoamTime> rt(lfm::newFoamTime(root, caseName));
        std::unique_ptr<lfm_case> c(new lfm_case);
        {
            CPolyMeshReaderOF reader(rt.get());
            c->sc = lfm::buildSolverCase(reader, prm);
        }
        c->deltaT = rt->deltaT;
        c->startTime = rt->startTime;
        c->endTime = rt->endTime;
        c->adjust = rt->adjustTimeStep;
        c->maxCo = in.m_dCFLMax;
        *out = c.release();
        return LFM_OK;
    } catch (const lfm::foam::FoamError& e) {
        return lfm::setError(LFM_ERR_IO, e.what());
    } catch (const std::exception& e) {
        return lfm::setError(LFM_ERR_INVALID, e.what());
    }
}

extern "C" int lfm_case_from_polymesh(const lfm_polymesh* mesh, const lfm_params* params, const lfm_fields* fields,
                                      lfm_case** out) {
    if (!mesh || !params || !fields || !out) return lfm::setError(LFM_ERR_INVALID, "lfm_case_from_polymesh: null argument");
    *out = nullptr;
    try {
        lfm::CaseParams prm;
        prm.solver = params->solver;
        prm.dimension = params->dimension;
        prm.rkOrder = params->rk_order;
        prm.minmod = params->minmod != 0;
        prm.laminar = params->laminar != 0;
        prm.residuals = params->residuals != 0;
        prm.pInf = params->p_inf;
        prm.TInf = params->T_inf;
        for (int k = 0; k < 3; ++k) prm.UInf[k] = params->U_inf[k];
        prm.Ls = params->Ls;
        prm.mach = params->mach;
        prm.kSponge = params->k_sponge;
        prm.Cp = params->Cp;
        prm.molWeight = params->mol_weight;
        prm.mu = params->mu;
        prm.Pr = params->Pr;
        prm.renumber = params->renumber;
        int rc = validateParams(prm);
        if (rc) return rc;
        if (mesh->n_faces <= 0 || mesh->n_cells <= 0 || !mesh->points || !mesh->face_offsets || !mesh->face_points ||
            !mesh->owner || (mesh->n_internal_faces > 0 && !mesh->neighbour))
            return lfm::setError(LFM_ERR_INVALID, "lfm_case_from_polymesh: incomplete mesh");
        if (!fields->p || !fields->T || !fields->U || (prm.Ls > 0 && !fields->alpha))
            return lfm::setError(LFM_ERR_INVALID, "lfm_case_from_polymesh: missing initial field");

        auto mc = std::make_shared<lfm::MemoryCase>();
        lfm::FoamMesh& m = mc->mesh;
        m.points.assign(mesh->points, mesh->points + 3 * mesh->n_points);
        m.faceOffsets.assign(mesh->face_offsets, mesh->face_offsets + mesh->n_faces + 1);
        m.facePoints.assign(mesh->face_points, mesh->face_points + m.faceOffsets.back());
        m.owner.assign(mesh->owner, mesh->owner + mesh->n_faces);
        m.neighbour.assign(mesh->neighbour, mesh->neighbour + mesh->n_internal_faces);
        m.nCells = mesh->n_cells;
        for (int p = 0; p < mesh->n_patches; ++p) {
            lfm::foam::Patch pt;
            pt.name = mesh->patch_name[p];
            pt.type = mesh->patch_type[p];
            pt.startFace = mesh->patch_start[p];
            pt.nFaces = mesh->patch_size[p];
            if (mesh->patch_neighbour && mesh->patch_neighbour[p]) pt.neighbourPatch = mesh->patch_neighbour[p];
            m.patches.push_back(pt);
        }
        if (mesh->cell_submesh) m.cellSubmesh.assign(mesh->cell_submesh, mesh->cell_submesh + mesh->n_cells);
        m.finalize();
        auto addField = [&](const char* name, const double* v, bool vec) {
            lfm::foam::VolField f;
            f.name = name;
            f.isVector = vec;
            f.values.assign(v, v + mesh->n_cells * (vec ? 3 : 1));
            mc->fields.push_back(std::move(f));
        };
        addField("p", fields->p, false);
        addField("T", fields->T, false);
        addField("U", fields->U, true);
        if (fields->alpha) addField("alpha", fields->alpha, false);

        lfm::FoamTime rt;
        rt.memory = mc;
        std::unique_ptr<lfm_case> c(new lfm_case);
        {
            CPolyMeshReaderOF reader(&rt);
            c->sc = lfm::buildSolverCase(reader, prm);
        }
        *out = c.release();
        return LFM_OK;
    } catch (const lfm::foam::FoamError& e) {
        return lfm::setError(LFM_ERR_INVALID, e.what());
    } catch (const std::exception& e) {
        return lfm::setError(LFM_ERR_INVALID, e.what());
    }
}

extern "C" int lfm_case_describe(const lfm_case* c, lfm_solver_desc* d) {
    if (!c || !d) return lfm::setError(LFM_ERR_INVALID, "lfm_case_describe: null argument");
    lfm::describeSolverCase(c->sc, d);
    return LFM_OK;
}

extern "C" int lfm_case_time(const lfm_case* c, double* delta_t, double* start_time, double* end_time,
                             int* adjust_time_step, double* max_co) {
    if (!c) return lfm::setError(LFM_ERR_INVALID, "lfm_case_time: null case");
    if (delta_t) *delta_t = c->deltaT;
    if (start_time) *start_time = c->startTime;
    if (end_time) *end_time = c->endTime;
    if (adjust_time_step) *adjust_time_step = c->adjust ? 1 : 0;
    if (max_co) *max_co = c->maxCo;
    return LFM_OK;
}

extern "C" int lfm_case_cell_ids(const lfm_case* c, int64_t* out) {
    if (!c || !out) return lfm::setError(LFM_ERR_INVALID, "lfm_case_cell_ids: null argument");
    std::memcpy(out, c->sc.cellId.data(), c->sc.cellId.size() * sizeof(int64_t));
    return LFM_OK;
}

extern "C" void lfm_case_free(lfm_case* c) { delete c; }

extern "C" int lfm_tiles_stats(const lfm_solver_desc* d, int tile_cells, int max_local, int64_t* out) {
    if (!d || !out) return lfm::setError(LFM_ERR_INVALID, "lfm_tiles_stats: null argument");
    try {
        const lfm::TileSet ts = lfm::buildTiles(d, tile_cells, max_local);
        out[0] = (int64_t)ts.tiles.size();
        out[1] = ts.maxL;
        out[2] = ts.maxLF;
        out[3] = ts.localCells;
        out[4] = ts.fluxFaces;
        return LFM_OK;
    } catch (const std::exception& e) {
        return lfm::setError(LFM_ERR_INVALID, e.what());
    }
}

// ---- decomposed cases: all processor partitions of a case at once ----------

struct lfm_pcase {
    std::vector<lfm::SolverCase> parts;
    double deltaT = 0, startTime = 0, endTime = 0, maxCo = 1;
    bool adjust = false;
};

extern "C" int lfm_pcase_open(const char* root, int nparts, lfm_pcase** out) {
    if (!root || !out || nparts < 1) return lfm::setError(LFM_ERR_INVALID, "lfm_pcase_open: bad argument");
    *out = nullptr;
    try {
        CInputReader in;
        in.readCase(root);
        lfm::CaseParams prm = paramsFromInput(in);
        prm.renumber = renumberOption(root);
        int rc = validateParams(prm);
        if (rc) return rc;
        std::vector<std::unique_ptr<lfm::FoamTime>> rts;
        std::vector<std::unique_ptr<CPolyMeshReaderOF>> readers;
        std::vector<IMeshReader*> rs;
        for (int p = 0; p < nparts; ++p) {
            rts.emplace_back(lfm::newFoamTime(root, "processor" + std::to_string(p)));
            readers.emplace_back(new CPolyMeshReaderOF(rts.back().get()));
            rs.push_back(readers.back().get());
        }
        std::unique_ptr<lfm_pcase> pc(new lfm_pcase);
        pc->parts = lfm::buildPartitionCases(rs, prm);
        pc->deltaT = rts[0]->deltaT;
        pc->startTime = rts[0]->startTime;
        pc->endTime = rts[0]->endTime;
        pc->adjust = rts[0]->adjustTimeStep;
        pc->maxCo = in.m_dCFLMax;
        readers.clear();
        *out = pc.release();
        return LFM_OK;
    } catch (const lfm::foam::FoamError& e) {
        return lfm::setError(LFM_ERR_IO, e.what());
    } catch (const std::exception& e) {
        return lfm::setError(LFM_ERR_INVALID, e.what());
    }
}

extern "C" int lfm_pcase_parts(const lfm_pcase* pc, int* nparts) {
    if (!pc || !nparts) return lfm::setError(LFM_ERR_INVALID, "lfm_pcase_parts: null argument");
    *nparts = (int)pc->parts.size();
    return LFM_OK;
}

extern "C" int lfm_pcase_describe(const lfm_pcase* pc, int part, lfm_solver_desc* d) {
    if (!pc || !d || part < 0 || part >= (int)pc->parts.size())
        return lfm::setError(LFM_ERR_INVALID, "lfm_pcase_describe: bad argument");
    lfm::describeSolverCase(pc->parts[(size_t)part], d);
    return LFM_OK;
}

extern "C" int lfm_pcase_cell_global(const lfm_pcase* pc, int part, int64_t* out) {
    if (!pc || !out || part < 0 || part >= (int)pc->parts.size())
        return lfm::setError(LFM_ERR_INVALID, "lfm_pcase_cell_global: bad argument");
    const lfm::SolverCase& sc = pc->parts[(size_t)part];
    std::memcpy(out, sc.cellGlobal.data(), sc.cellGlobal.size() * sizeof(int64_t));
    return LFM_OK;
}

extern "C" int lfm_pcase_time(const lfm_pcase* pc, double* delta_t, double* start_time, double* end_time,
                              int* adjust_time_step, double* max_co) {
    if (!pc) return lfm::setError(LFM_ERR_INVALID, "lfm_pcase_time: null case");
    if (delta_t) *delta_t = pc->deltaT;
    if (start_time) *start_time = pc->startTime;
    if (end_time) *end_time = pc->endTime;
    if (adjust_time_step) *adjust_time_step = pc->adjust ? 1 : 0;
    if (max_co) *max_co = pc->maxCo;
    return LFM_OK;
}

extern "C" void lfm_pcase_free(lfm_pcase* pc) { delete pc; }
