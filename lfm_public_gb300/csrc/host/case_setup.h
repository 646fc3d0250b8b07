// Solver setup: from a polyMesh (IMeshReader) and the case parameters to the
// structure-of-arrays description the device kernels and the CPU oracle use.
//
// Restates the reference's per-submesh setup:
//   src/mesh_reader.cpp:90-260   cell / face / neighbour lists per submesh
//   src/mesh_reader.cpp:263-371  face area normals and owner sign
//   src/mesh_reader.cpp:374-460  neighbour-centre vectors (cyclic translated,
//                                boundary ghosts mirrored)
//   src/cfd_v0.cpp:759-861       S, d, linear weight, 1/V per cell-face
//   src/cfd_v0.cpp:277-339       reorder_faces: a face belongs to the side with
//                                the smaller (submesh, index)
//   src/cfd_v0.cpp:344-420       one boundary ghost per boundary face
//   src/cfd_v0.cpp:866-967       free stream, sponge and initial state
//   src/cfd_v0.cpp:972-1005      patch -> boundary-condition kind
//   src/cfd_v0.cpp:86-128        low-storage RK coefficients
#pragma once

#include <cstdint>
#include <string>
#include <vector>

class IMeshReader;
struct lfm_solver_desc;

namespace lfm {

enum GhostKind { GHOST_NONE = 0, GHOST_WALL = 1, GHOST_INLET = 2, GHOST_OUTLET = 3, GHOST_FARFIELD = 4 };

// Parameters the reference reads through CInputReader (src/inputReader.cpp:13-64).
struct CaseParams {
    int solver = 0;            // 0 M1, 1 M2, 2 M2AUSM (api/fastmesh.h:38-41)
    int dimension = 2;
    int rkOrder = 5;
    bool minmod = false;
    bool laminar = true;
    bool residuals = false;
    double pInf = 0, TInf = 0, UInf[3] = {0, 0, 0};
    double Ls = 0, mach = 0, kSponge = 4.34294481903252e-01;
    double Cp = 0, molWeight = 0, mu = 0, Pr = 1;
    int renumber = 0;          // solver order inside each submesh: Renumber (renumber.h)
};

// Other side of a processor face, for a partition built alongside its
// neighbours (the reference exchanges these over MPI, src/mesh_reader.cpp:481-611):
// the neighbour's cell centre relative to its face centre, keyed by the
// face's global id (getFaceId).
class HaloLookup {
public:
    virtual ~HaloLookup() = default;
    virtual bool neighbourOffset(int nbrProc, int64_t faceId, double* x) const = 0;
};

struct SolverCase {
    int dim = 2;
    int nq = 4;                  // dim + 2 conserved variables
    int64_t nCells = 0;          // interior cells, submesh 0 first then submesh 1
    int64_t nCells0 = 0;         // cells of submesh 0
    int64_t nGhosts = 0;         // boundary ghosts, stored after the cells
    int64_t nHalos = 0;          // processor-face halos, stored after the ghosts
    int64_t nFaces = 0;          // flux faces, in the reference's processing order
    int maxFacesPerCell = 0;

    // cells (solver order) -----------------------------------------------------
    std::vector<int64_t> cellId;         // polyMesh cell label
    std::vector<double> volInv, sponge;  // per cell
    std::vector<double> smagC;           // per cell, Smagorinsky LES only (see lfm_solver_desc)
    std::vector<double> q0;              // initial state, nq x nCells (SoA)

    // boundary ghosts ------------------------------------------------------------
    std::vector<int64_t> ghostCell;      // interior cell next to the ghost
    std::vector<int> ghostKind;          // GhostKind
    std::vector<int64_t> ghostFace;      // flux face of the ghost
    std::vector<int> ghostPatch;

    // processor-face halos (partitioned cases) ------------------------------------
    // Halo h is the N side of flux face haloFace[h]: the cell across a processor
    // patch, owned by partition haloProc[h]; it is matched to that partition's
    // copy of the face by haloFaceId[h], and its source cell there (solver
    // order) is filled in by resolveHalos.
    std::vector<int64_t> haloFace;
    std::vector<int> haloProc;
    std::vector<int64_t> haloFaceId;
    std::vector<int64_t> haloCell;       // the local cell P of the face
    std::vector<int64_t> haloSrcPart, haloSrcCell;
    std::vector<int64_t> cellGlobal;     // cellProcAddressing of each solver cell (partitioned cases)

    // flux faces (owner side = reference processing side) ------------------------
    std::vector<int64_t> faceP, faceN;   // N >= nCells: ghost N - nCells, halo N - nCells - nGhosts
    std::vector<uint8_t> faceGhost;      // neighbour is a boundary ghost
    std::vector<double> S, d;            // dim x nFaces (SoA)
    std::vector<double> w;               // linear weight of P
    // per-face constants precomputed with the reference's own expressions
    // (src/cfd_v0.cpp:2687-2766): |S|, 1/|d|, d/|d|, |delta|, K = S - delta.
    std::vector<double> Smag, dmagInv, dnorm, deltaMag, K;

    // cell -> face incidence, ascending face index (= the order in which the
    // reference accumulates into a cell); sign +1 when the cell is P.
    std::vector<int64_t> cellFaceOffsets;
    std::vector<int64_t> cellFaces;
    std::vector<int8_t> cellFaceSign;
    // all valid faces of a cell with S seen from that cell (compute_dt / cfl)
    std::vector<int64_t> cellSOffsets;
    std::vector<double> cellS;           // dim values per entry

    // constants ------------------------------------------------------------------
    int solver = 0, rkOrder = 5;
    bool minmod = false, residuals = false;
    double gamma = 1.4, Rgas = 287, rhoInf = 1, EInf = 0, pInf = 0, TInf = 0, UInf[3] = {0, 0, 0};
    double mu = 0, Cp = 0, PrInv = 1;
    std::vector<double> rkA, rkB;
};

// Builds the case from a mesh reader that already holds the fields p, T, U and
// (when Ls > 0) alpha at the start time. Throws std::runtime_error on bad input.
// Processor patches need `halos` (the neighbouring partitions' geometry).
SolverCase buildSolverCase(IMeshReader& reader, const CaseParams& params, const HaloLookup* halos = nullptr);

// Matches every halo of every partition to its source cell in the partition
// across the processor face (by face id). Throws when a face has no partner.
void resolveHalos(std::vector<SolverCase>& parts);

// Every partition of a decomposed case from its readers (processor0..N-1):
// the processor faces' neighbour offsets exchanged between the readers (what
// each rank of the reference sends its neighbours, src/mesh_reader.cpp:520-552),
// each partition's solver case with its halos, cellGlobal from
// cellProcAddressing, and the halos matched to their source cells.
std::vector<SolverCase> buildPartitionCases(const std::vector<IMeshReader*>& readers, const CaseParams& params);

// Fills the flattened C description with pointers into `sc` (valid while sc lives).
void describeSolverCase(const SolverCase& sc, lfm_solver_desc* out);

// RK coefficients for rkOrder (src/cfd_v0.cpp:86-128).
void rkCoefficients(int rkOrder, std::vector<double>& A, std::vector<double>& B);

}  // namespace lfm
