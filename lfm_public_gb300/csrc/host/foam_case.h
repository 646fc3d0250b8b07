// Internal objects behind the OpenFOAM-free plugin classes.
//
// The reference's plugins hide Foam::Time, Foam::fvMesh and the vol fields
// behind void pointers (runTimeManagerOF.h m_pRunTime, polyMeshReaderOF.h
// m_pMesh / m_pVolScalarFieldList, dictReaderOF.h m_pIODict). These are the
// objects this build stores behind the same pointers.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "foam_io.h"

namespace lfm {

// A polyMesh plus the geometry OpenFOAM derives from it (faceAreas,
// faceCentres, cellVolumes, cellCentres) and the cell->face lists.
struct FoamMesh {
    std::vector<double> points;                 // 3 per point
    std::vector<int64_t> faceOffsets, facePoints;  // CSR face->points
    std::vector<int64_t> owner;                 // per face
    std::vector<int64_t> neighbour;             // per internal face
    std::vector<foam::Patch> patches;
    std::vector<int64_t> cellSubmesh;           // optional polyMesh/cellSubmesh
    std::vector<int64_t> pointProcAddressing, faceProcAddressing, cellProcAddressing,
        boundaryProcAddressing;
    int64_t nCells = 0;

    // Derived.
    std::vector<double> faceAreas, faceCentres, cellVolumes, cellCentres;
    std::vector<int64_t> cellOffsets, cellFaces;  // CSR cell->faces (OpenFOAM order)

    int64_t nFaces() const { return (int64_t)owner.size(); }
    int64_t nInternalFaces() const { return (int64_t)neighbour.size(); }
    int64_t nPoints() const { return (int64_t)points.size() / 3; }
    int whichPatch(int64_t face) const;   // -1 for internal faces

    void finalize();   // validates and computes the derived data
};

// Builds the geometry with OpenFOAM's published construction
// (primitiveMeshFaceCentresAndAreas / primitiveMeshCellCentresAndVols):
//   face  : triangles directly; other polygons by a fan of triangles about the
//           point average, centre = area-weighted triangle centroids;
//   cell  : pyramids from each face to the average of the cell's face centres,
//           centre = volume-weighted pyramid centroids.
void computeGeometry(FoamMesh& m);

// In-memory case: a mesh plus initial fields, used instead of case files.
struct MemoryCase {
    FoamMesh mesh;
    std::vector<foam::VolField> fields;   // by name (p, T, U, alpha, ...)
};

struct FieldObject {
    foam::VolField data;
    bool autoWrite = true;
};

// Foam::Time restated: controlDict-driven start/end/deltaT, time index, write
// control and the registry of fields written by write().
struct FoamTime {
    std::string rootPath = ".";
    std::string caseName = ".";
    bool processorCase = false;
    foam::Dict controlDict;

    double startTime = 0, endTime = 0, deltaT = 0, value = 0;
    int64_t timeIndex = 0, startTimeIndex = 0;
    std::string writeControl = "timeStep";
    double writeInterval = 1;
    int64_t writeTimeIndex = 0;
    int writePrecision = 6;
    bool writeBinary = false;
    std::string timeFormat = "general";
    int timePrecision = 6;
    bool adjustTimeStep = false;
    double maxCo = 1, maxDeltaT = 1e300;
    bool writeTime = false;

    std::shared_ptr<MemoryCase> memory;   // non-null: no case files are read or written
    std::vector<FieldObject*> registry;   // fields written by write()

    std::string casePath() const;                 // rootPath/caseName
    std::string dictPath(const std::string& dir, const std::string& name) const;
    std::string timeName() const { return timeName(value); }
    std::string timeName(double t) const;
    bool running() const { return value < endTime - 0.5 * deltaT; }
    void increment();
    void write();
    void loadControlDict();
};

// Builds a FoamTime for `case` under `root` (caseName "." or "processorN").
FoamTime* newFoamTime(const std::string& root, const std::string& caseName);

}  // namespace lfm
