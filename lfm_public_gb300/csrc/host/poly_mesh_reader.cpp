// CPolyMeshReaderOF without OpenFOAM.
//
// Follows polyMeshReaderOF/polyMeshReaderOF.cpp. The mesh is
// <case>/constant/polyMesh (points, faces, owner, neighbour, boundary and the
// optional cellSubmesh / *ProcAddressing label lists, :15-45) or an in-memory
// lfm::MemoryCase. Faces of 'empty' patches are invalid (:47-64). Geometry comes
// from lfm::computeGeometry, which restates OpenFOAM's faceAreas / faceCentres /
// cellVolumes / cellCentres. Cyclic faces see the owner of their partner face as
// neighbour (:140-151, :226-248). The submesh split (:501-610) puts every cell
// that touches a point of a non-empty patch in submesh 0 and the rest in
// submesh 1, unless polyMesh/cellSubmesh gives the split. Fields are read from
// the current time directory with AUTO_WRITE and created fields get
// zeroGradient patches (:687-789).
#include "polyMeshReaderOF.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <iostream>
#include <memory>

#include "foam_case.h"

using lfm::FieldObject;
using lfm::FoamMesh;
using lfm::FoamTime;
namespace foam = lfm::foam;

namespace {
struct MeshHolder {
    std::shared_ptr<FoamMesh> mesh;
    int nNonProcessor = 0;
};

const FoamMesh& M(void* p) { return *static_cast<MeshHolder*>(p)->mesh; }
const MeshHolder& H(void* p) { return *static_cast<MeshHolder*>(p); }

std::vector<int> toInt(const std::vector<int64_t>& v) { return std::vector<int>(v.begin(), v.end()); }

bool isCoupledCyclic(const foam::Patch& p) { return p.type == "cyclic"; }
}  // namespace

CPolyMeshReaderOF::CPolyMeshReaderOF(void* pRunTime) {
    m_pRunTime = pRunTime;
    m_nTimeIndex = 0;
    FoamTime& rt = *static_cast<FoamTime*>(pRunTime);
    MeshHolder* h = new MeshHolder;
    if (rt.memory) {
        h->mesh = std::shared_ptr<FoamMesh>(rt.memory, &rt.memory->mesh);
    } else {
        auto m = std::make_shared<FoamMesh>();
        const std::string dir = rt.casePath() + "/constant/polyMesh/";
        m->points = foam::readVectorList(dir + "points");
        foam::readFaceList(dir + "faces", m->faceOffsets, m->facePoints);
        m->owner = foam::readLabelList(dir + "owner");
        m->neighbour = foam::readLabelList(dir + "neighbour");
        m->patches = foam::readBoundary(dir + "boundary");
        if (foam::fileExists(dir + "cellSubmesh")) m->cellSubmesh = foam::readLabelList(dir + "cellSubmesh");
        if (foam::fileExists(dir + "pointProcAddressing"))
            m->pointProcAddressing = foam::readLabelList(dir + "pointProcAddressing");
        if (foam::fileExists(dir + "faceProcAddressing"))
            m->faceProcAddressing = foam::readLabelList(dir + "faceProcAddressing");
        if (foam::fileExists(dir + "cellProcAddressing"))
            m->cellProcAddressing = foam::readLabelList(dir + "cellProcAddressing");
        if (foam::fileExists(dir + "boundaryProcAddressing"))
            m->boundaryProcAddressing = foam::readLabelList(dir + "boundaryProcAddressing");
        m->finalize();
        h->mesh = m;
    }
    const FoamMesh& mesh = *h->mesh;
    if (mesh.cellVolumes.size() != (size_t)mesh.nCells)
        throw foam::FoamError("mesh geometry has not been computed");
    h->nNonProcessor = (int)mesh.patches.size();
    for (size_t p = 0; p < mesh.patches.size(); ++p)
        if (mesh.patches[p].type == "processor" || mesh.patches[p].type == "processorCyclic") {
            h->nNonProcessor = (int)p;
            break;
        }
    m_pMesh = h;

    m_nPointProcAddressingList = toInt(mesh.pointProcAddressing);
    m_nFaceProcAddressingList = toInt(mesh.faceProcAddressing);
    m_nCellProcAddressingList = toInt(mesh.cellProcAddressing);
    m_nBoundaryProcAddressingList = toInt(mesh.boundaryProcAddressing);
    m_nCellSubmeshList = toInt(mesh.cellSubmesh);

    m_bValidFaceFlagList.assign((size_t)mesh.nFaces(), true);
    for (const foam::Patch& p : mesh.patches)
        if (p.type == "empty")
            for (int64_t f = p.startFace; f < p.startFace + p.nFaces; ++f) m_bValidFaceFlagList[(size_t)f] = false;

    initializeSubmesh();
}

CPolyMeshReaderOF::~CPolyMeshReaderOF() {
    FoamTime* rt = static_cast<FoamTime*>(m_pRunTime);
    auto unregister = [rt](FieldObject* f) {
        if (!rt) return;
        auto& reg = rt->registry;
        reg.erase(std::remove(reg.begin(), reg.end(), f), reg.end());
    };
    for (void* p : m_pVolScalarFieldList) {
        unregister(static_cast<FieldObject*>(p));
        delete static_cast<FieldObject*>(p);
    }
    for (void* p : m_pVolVectorFieldList) {
        unregister(static_cast<FieldObject*>(p));
        delete static_cast<FieldObject*>(p);
    }
    delete static_cast<MeshHolder*>(m_pMesh);
}

// -- points ------------------------------------------------------------------
int CPolyMeshReaderOF::getPointCount() const { return (int)M(m_pMesh).nPoints(); }

void CPolyMeshReaderOF::getPoint(const int nPointIndex, double* pXYZ) const {
    const double* p = &M(m_pMesh).points[(size_t)nPointIndex * 3];
    pXYZ[0] = p[0];
    pXYZ[1] = p[1];
    pXYZ[2] = p[2];
}

int CPolyMeshReaderOF::getPointProcAddressing(const int nPointIndex) const {
    return (nPointIndex < (int)m_nPointProcAddressingList.size()) ? m_nPointProcAddressingList[nPointIndex]
                                                                  : nPointIndex;
}

// -- faces -------------------------------------------------------------------
int CPolyMeshReaderOF::getFaceCount() const { return (int)M(m_pMesh).nFaces(); }

void CPolyMeshReaderOF::getFaceAreaNormal(const int nFaceIndex, double* pN) const {
    const double* a = &M(m_pMesh).faceAreas[(size_t)nFaceIndex * 3];
    pN[0] = a[0];
    pN[1] = a[1];
    pN[2] = a[2];
}

void CPolyMeshReaderOF::getFaceCenter(const int nFaceIndex, double* pXYZ) const {
    const double* c = &M(m_pMesh).faceCentres[(size_t)nFaceIndex * 3];
    pXYZ[0] = c[0];
    pXYZ[1] = c[1];
    pXYZ[2] = c[2];
}

int CPolyMeshReaderOF::getFaceOwner(const int nFaceIndex) const { return (int)M(m_pMesh).owner[(size_t)nFaceIndex]; }

int CPolyMeshReaderOF::getFaceNeighbour(const int nFaceIndex) const {
    const FoamMesh& m = M(m_pMesh);
    if (nFaceIndex < m.nInternalFaces()) return (int)m.neighbour[(size_t)nFaceIndex];
    const int cyc = getCyclicFaceIndex(nFaceIndex);
    return (cyc == nFaceIndex) ? -1 : (int)m.owner[(size_t)cyc];
}

int CPolyMeshReaderOF::getFaceBoundary(const int nFaceIndex) const { return M(m_pMesh).whichPatch(nFaceIndex); }

int CPolyMeshReaderOF::getFaceIndexInsideBoundary(const int nFaceIndex) const {
    const int b = getFaceBoundary(nFaceIndex);
    return nFaceIndex - ((b == -1) ? 0 : (int)M(m_pMesh).patches[(size_t)b].startFace);
}

int CPolyMeshReaderOF::getFacePointCount(const int nFaceIndex) const {
    const FoamMesh& m = M(m_pMesh);
    return (int)(m.faceOffsets[(size_t)nFaceIndex + 1] - m.faceOffsets[(size_t)nFaceIndex]);
}

int CPolyMeshReaderOF::getFaceProcAddressing(const int nFaceIndex) const {
    return (nFaceIndex < (int)m_nFaceProcAddressingList.size()) ? m_nFaceProcAddressingList[nFaceIndex] : nFaceIndex;
}

int CPolyMeshReaderOF::getFacePointIndex(const int nFaceIndex, const int nIndex) const {
    const FoamMesh& m = M(m_pMesh);
    return (int)m.facePoints[(size_t)(m.faceOffsets[(size_t)nFaceIndex] + nIndex)];
}

std::vector<int> CPolyMeshReaderOF::getFacePointIndexList(const int nFaceIndex) const {
    const FoamMesh& m = M(m_pMesh);
    return std::vector<int>(m.facePoints.begin() + m.faceOffsets[(size_t)nFaceIndex],
                            m.facePoints.begin() + m.faceOffsets[(size_t)nFaceIndex + 1]);
}

int CPolyMeshReaderOF::getCyclicFaceIndex(const int nFaceIndex) const {
    const FoamMesh& m = M(m_pMesh);
    const int b = m.whichPatch(nFaceIndex);
    if (b == -1 || !isCoupledCyclic(m.patches[(size_t)b])) return nFaceIndex;
    const std::string& nbrName = m.patches[(size_t)b].neighbourPatch;
    for (size_t q = 0; q < m.patches.size(); ++q)
        if (m.patches[q].name == nbrName)
            return nFaceIndex - (int)m.patches[(size_t)b].startFace + (int)m.patches[q].startFace;
    return nFaceIndex;
}

int CPolyMeshReaderOF::getFaceId(const int nFaceIndex) const {
    const int tag = getBoundaryTag(getFaceBoundary(nFaceIndex));
    if (tag >= -1 && tag <= 1) return std::abs(getFaceProcAddressing(nFaceIndex));
    return getFaceIndexInsideBoundary(nFaceIndex);
}

// -- cells -------------------------------------------------------------------
int CPolyMeshReaderOF::getCellCount() const { return (int)M(m_pMesh).nCells; }

double CPolyMeshReaderOF::getCellVolume(const int nCellIndex) const {
    return M(m_pMesh).cellVolumes[(size_t)nCellIndex];
}

void CPolyMeshReaderOF::getCellCenter(const int nCellIndex, double* pXYZ) const {
    const double* c = &M(m_pMesh).cellCentres[(size_t)nCellIndex * 3];
    pXYZ[0] = c[0];
    pXYZ[1] = c[1];
    pXYZ[2] = c[2];
}

int CPolyMeshReaderOF::getCellFaceCount(const int nCellIndex) const {
    const FoamMesh& m = M(m_pMesh);
    return (int)(m.cellOffsets[(size_t)nCellIndex + 1] - m.cellOffsets[(size_t)nCellIndex]);
}

int CPolyMeshReaderOF::getCellFaceIndex(const int nCellIndex, const int nIndex) const {
    const FoamMesh& m = M(m_pMesh);
    return (int)m.cellFaces[(size_t)(m.cellOffsets[(size_t)nCellIndex] + nIndex)];
}

bool CPolyMeshReaderOF::getCellFaceOwner(const int nCellIndex, const int nIndex) const {
    return getFaceOwner(getCellFaceIndex(nCellIndex, nIndex)) == nCellIndex;
}

int CPolyMeshReaderOF::getCellProcAddressing(const int nCellIndex) const {
    return (nCellIndex < (int)m_nCellProcAddressingList.size()) ? m_nCellProcAddressingList[nCellIndex] : nCellIndex;
}

std::vector<int> CPolyMeshReaderOF::getCellPointList(const int nCellIndex) const {
    std::vector<int> out;
    const int nf = getCellFaceCount(nCellIndex);
    for (int i = 0; i < nf; ++i) {
        for (int p : getFacePointIndexList(getCellFaceIndex(nCellIndex, i)))
            if (std::find(out.begin(), out.end(), p) == out.end()) out.push_back(p);
    }
    return out;
}

int CPolyMeshReaderOF::getCellValidFaceCount(const int nCellIndex) const {
    int n = 0;
    const int nf = getCellFaceCount(nCellIndex);
    for (int i = 0; i < nf; ++i)
        if (m_bValidFaceFlagList[(size_t)getCellFaceIndex(nCellIndex, i)]) ++n;
    return n;
}

int CPolyMeshReaderOF::getCellValidFaceIndex(const int nCellIndex, const int nIndex) const {
    int k = 0;
    const int nf = getCellFaceCount(nCellIndex);
    for (int i = 0; i < nf; ++i) {
        const int f = getCellFaceIndex(nCellIndex, i);
        if (!m_bValidFaceFlagList[(size_t)f]) continue;
        if (k == nIndex) return f;
        ++k;
    }
    return -1;
}

double CPolyMeshReaderOF::getCellScalar(const int nCellIndex, const int nFieldIndex) const {
    return static_cast<const FieldObject*>(m_pVolScalarFieldList[(size_t)nFieldIndex])->data.values[(size_t)nCellIndex];
}

void CPolyMeshReaderOF::getCellVector(const int nCellIndex, const int nFieldIndex, double* pVec) const {
    const FieldObject* f = static_cast<const FieldObject*>(m_pVolVectorFieldList[(size_t)nFieldIndex]);
    for (int k = 0; k < 3; ++k) pVec[k] = f->data.values[(size_t)nCellIndex * 3 + k];
}

// -- boundary ----------------------------------------------------------------
int CPolyMeshReaderOF::getBoundaryCount() const { return (int)M(m_pMesh).patches.size(); }
std::string CPolyMeshReaderOF::getBoundaryName(const int b) const { return M(m_pMesh).patches[(size_t)b].name; }
std::string CPolyMeshReaderOF::getBoundaryType(const int b) const { return M(m_pMesh).patches[(size_t)b].type; }
int CPolyMeshReaderOF::getBoundaryFaceStart(const int b) const { return (int)M(m_pMesh).patches[(size_t)b].startFace; }

int CPolyMeshReaderOF::getBoundaryFaceEnd(const int b) const {
    const foam::Patch& p = M(m_pMesh).patches[(size_t)b];
    return (int)(p.startFace + p.nFaces - 1);
}

std::vector<int> CPolyMeshReaderOF::getBoundaryFaceCellList(const int b) const {
    const FoamMesh& m = M(m_pMesh);
    const foam::Patch& p = m.patches[(size_t)b];
    std::vector<int> out;
    for (int64_t f = p.startFace; f < p.startFace + p.nFaces; ++f) out.push_back((int)m.owner[(size_t)f]);
    return out;
}

int CPolyMeshReaderOF::getBoundaryProcAddressing(const int b) const {
    return (b < (int)m_nBoundaryProcAddressingList.size()) ? m_nBoundaryProcAddressingList[b] : b;
}

int CPolyMeshReaderOF::getBoundaryProcessorRank(const int b) const {
    if (b < H(m_pMesh).nNonProcessor) return -1;
    return M(m_pMesh).patches[(size_t)b].neighbProcNo;
}

int CPolyMeshReaderOF::getBoundaryTag(const int b) const {
    if (b < H(m_pMesh).nNonProcessor) return 0;
    // Plain processor patches carry tag -1; the sign marks the owner side.
    const foam::Patch& p = M(m_pMesh).patches[(size_t)b];
    const int ownerSide = (p.myProcNo < p.neighbProcNo) ? 1 : 0;
    return -1 * (2 * ownerSide - 1);
}

int CPolyMeshReaderOF::getBoundaryCyclicPairIndex(const int /*b*/) const { return -1; }

std::vector<int> CPolyMeshReaderOF::getNeighbourCellList(const int b) const {
    const FoamMesh& m = M(m_pMesh);
    const foam::Patch& p = m.patches[(size_t)b];
    std::vector<int> out;
    if (!isCoupledCyclic(p)) return out;
    for (int64_t f = p.startFace; f < p.startFace + p.nFaces; ++f) out.push_back(getFaceNeighbour((int)f));
    return out;
}

// -- submeshes ---------------------------------------------------------------
void CPolyMeshReaderOF::initializeSubmesh() {
    const FoamMesh& m = M(m_pMesh);
    const int nCells = (int)m.nCells;
    if ((int)m_nCellSubmeshList.size() != nCells) {
        std::vector<bool> interiorPoint((size_t)m.nPoints(), true);
        for (const foam::Patch& p : m.patches) {
            if (p.type == "empty") continue;
            for (int64_t f = p.startFace; f < p.startFace + p.nFaces; ++f)
                for (int64_t k = m.faceOffsets[(size_t)f]; k < m.faceOffsets[(size_t)f + 1]; ++k)
                    interiorPoint[(size_t)m.facePoints[(size_t)k]] = false;
        }
        m_nCellSubmeshList.assign((size_t)nCells, 1);
        for (int c = 0; c < nCells; ++c) {
            bool interior = true;
            for (int64_t i = m.cellOffsets[(size_t)c]; i < m.cellOffsets[(size_t)c + 1] && interior; ++i) {
                const int64_t f = m.cellFaces[(size_t)i];
                for (int64_t k = m.faceOffsets[(size_t)f]; k < m.faceOffsets[(size_t)f + 1] && interior; ++k)
                    interior = interiorPoint[(size_t)m.facePoints[(size_t)k]];
            }
            m_nCellSubmeshList[(size_t)c] = interior ? 1 : 0;
        }
    }
    m_nPointMaskList.assign((size_t)m.nPoints(), 0);
    m_nFaceMaskList.assign((size_t)m.nFaces(), 0);
    m_nCellMaskList.assign((size_t)nCells, 0);
    m_nSubmeshCount = 0;
    for (int c = 0; c < nCells; ++c) {
        const int sm = m_nCellSubmeshList[(size_t)c];
        if (sm >= m_nSubmeshCount) m_nSubmeshCount = sm + 1;
        const int mask = getMask(sm);
        m_nCellMaskList[(size_t)c] |= mask;
        for (int64_t i = m.cellOffsets[(size_t)c]; i < m.cellOffsets[(size_t)c + 1]; ++i) {
            const int64_t f = m.cellFaces[(size_t)i];
            m_nFaceMaskList[(size_t)f] |= mask;
            for (int64_t k = m.faceOffsets[(size_t)f]; k < m.faceOffsets[(size_t)f + 1]; ++k)
                m_nPointMaskList[(size_t)m.facePoints[(size_t)k]] |= mask;
        }
    }
    m_nSubmeshPointMappingList.assign((size_t)m_nSubmeshCount, {});
    m_nSubmeshFaceMappingList.assign((size_t)m_nSubmeshCount, {});
    m_nSubmeshCellMappingList.assign((size_t)m_nSubmeshCount, {});
    // The index lists are ascending: appending at the end of each map is
    // amortised constant time.
    auto fill = [](std::map<int, int>& m, const std::vector<int>& ids) {
        for (size_t i = 0; i < ids.size(); ++i) m.emplace_hint(m.end(), ids[i], (int)i);
    };
    for (int s = 0; s < m_nSubmeshCount; ++s) {
        fill(m_nSubmeshPointMappingList[(size_t)s], getSubmeshPointIndexList(s));
        fill(m_nSubmeshFaceMappingList[(size_t)s], getSubmeshFaceIndexList(s));
        fill(m_nSubmeshCellMappingList[(size_t)s], getSubmeshCellIndexList(s));
    }
}

std::vector<double> CPolyMeshReaderOF::getCellDistanceFromBoundary(const int nSubmeshIndex,
                                                                   const std::vector<int> nBoundaryIndexList) const {
    const FoamMesh& m = M(m_pMesh);
    const std::vector<int> cells = getSubmeshCellIndexList(nSubmeshIndex);
    std::vector<double> dist(cells.size(), (double)INT64_MAX);
    for (int b : nBoundaryIndexList) {
        const foam::Patch& p = m.patches[(size_t)b];
        for (size_t i = 0; i < cells.size(); ++i) {
            const double* cc = &m.cellCentres[(size_t)cells[i] * 3];
            for (int64_t f = p.startFace; f < p.startFace + p.nFaces; ++f) {
                const double* a = &m.faceAreas[(size_t)f * 3];
                const double* fc = &m.faceCentres[(size_t)f * 3];
                const double mag = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
                double v[3];
                for (int k = 0; k < 3; ++k) v[k] = (a[k] / mag) * (fc[k] - cc[k]);
                const double d2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
                if (d2 < dist[i]) dist[i] = d2;
            }
            dist[i] = std::sqrt(dist[i]);
        }
    }
    return dist;
}

double CPolyMeshReaderOF::getLocalityScore(const int nMethod) const {
    const FoamMesh& m = M(m_pMesh);
    double score = 0;
    for (int64_t c = 0; c < m.nCells; ++c) {
        double cellScore = 0;
        int n = 0;
        for (int64_t i = m.cellOffsets[(size_t)c]; i < m.cellOffsets[(size_t)c + 1]; ++i) {
            const int64_t f = m.cellFaces[(size_t)i];
            if (f >= m.nInternalFaces()) continue;
            const double d = std::fabs((double)(m.neighbour[(size_t)f] - c)) / (double)m.nCells;
            cellScore += (nMethod == 0) ? d : d * d;
            ++n;
        }
        score += cellScore / n;
    }
    return score / (double)m.nCells;
}

// -- fields ------------------------------------------------------------------
static FieldObject* loadField(FoamTime& rt, const FoamMesh& m, const std::string& name, bool isVector) {
    FieldObject* f = new FieldObject;
    if (rt.memory) {
        bool found = false;
        for (const foam::VolField& v : rt.memory->fields)
            if (v.name == name) {
                f->data = v;
                found = true;
            }
        if (!found) {
            delete f;
            throw foam::FoamError("field '" + name + "' is not part of the in-memory case");
        }
        if (f->data.values.size() != (size_t)m.nCells * (isVector ? 3 : 1)) {
            delete f;
            throw foam::FoamError("field '" + name + "' has the wrong size");
        }
    } else {
        f->data = foam::readVolField(rt.casePath() + "/" + rt.timeName() + "/" + name, m.nCells, isVector);
    }
    f->data.name = name;
    f->data.isVector = isVector;
    f->autoWrite = true;
    rt.registry.push_back(f);
    return f;
}

int CPolyMeshReaderOF::readScalarField(const std::string sFieldName) {
    int idx = getScalarFieldIndex(sFieldName);
    if (idx != -1) return idx;
    FieldObject* f = loadField(*static_cast<FoamTime*>(m_pRunTime), M(m_pMesh), sFieldName, false);
    m_pVolScalarFieldList.push_back(f);
    m_sScalarFieldList.push_back(sFieldName);
    return (int)m_pVolScalarFieldList.size() - 1;
}

int CPolyMeshReaderOF::readVectorField(const std::string sFieldName) {
    int idx = getVectorFieldIndex(sFieldName);
    if (idx != -1) return idx;
    FieldObject* f = loadField(*static_cast<FoamTime*>(m_pRunTime), M(m_pMesh), sFieldName, true);
    m_pVolVectorFieldList.push_back(f);
    m_sVectorFieldList.push_back(sFieldName);
    return (int)m_pVolVectorFieldList.size() - 1;
}

int CPolyMeshReaderOF::createScalarField(const std::string sFieldName) {
    int idx = getScalarFieldIndex(sFieldName);
    if (idx != -1) return idx;
    const FoamMesh& m = M(m_pMesh);
    FieldObject* f = new FieldObject;
    f->data.name = sFieldName;
    f->data.values.assign((size_t)m.nCells, 0.0);
    std::string b = "\n";
    for (const foam::Patch& p : m.patches) {
        std::string t = "zeroGradient";
        if (p.type == "empty" || p.type == "cyclic" || p.type == "processor" || p.type == "processorCyclic" ||
            p.type == "symmetryPlane" || p.type == "wedge")
            t = p.type;
        b += "    " + p.name + "\n    {\n        type            " + t + ";\n    }\n";
    }
    f->data.boundaryText = b;
    static_cast<FoamTime*>(m_pRunTime)->registry.push_back(f);
    m_pVolScalarFieldList.push_back(f);
    m_sScalarFieldList.push_back(sFieldName);
    return (int)m_pVolScalarFieldList.size() - 1;
}

static std::vector<double>& SV(const std::vector<void*>& l, int i) {
    return static_cast<FieldObject*>(l[(size_t)i])->data.values;
}

template <typename T>
static void updateScalarImpl(CPolyMeshReaderOF* r, std::vector<double>& field, const std::vector<T>& v, int sm,
                             T factor, bool takeSqrt, const std::vector<int>& cells) {
    (void)r;
    auto val = [&](size_t i) {
        const double x = (double)(v[i] * factor);
        return takeSqrt ? std::sqrt(x) : x;
    };
    if (sm == -1) {
        for (size_t c = 0; c < field.size(); ++c) field[c] = val(c);
    } else {
        for (size_t i = 0; i < cells.size(); ++i) field[(size_t)cells[i]] = val(i);
    }
}

void CPolyMeshReaderOF::updateScalarField(const int nFieldIndex, const std::vector<double>& dScalarList,
                                          const int nSubmeshIndex, const double dFactor) {
    updateScalarImpl<double>(this, SV(m_pVolScalarFieldList, nFieldIndex), dScalarList, nSubmeshIndex, dFactor, false,
                             nSubmeshIndex == -1 ? std::vector<int>() : getSubmeshCellIndexList(nSubmeshIndex));
}

void CPolyMeshReaderOF::updateScalarField(const int nFieldIndex, const std::vector<float>& fScalarList,
                                          const int nSubmeshIndex, const float fFactor) {
    updateScalarImpl<float>(this, SV(m_pVolScalarFieldList, nFieldIndex), fScalarList, nSubmeshIndex, fFactor, false,
                            nSubmeshIndex == -1 ? std::vector<int>() : getSubmeshCellIndexList(nSubmeshIndex));
}

void CPolyMeshReaderOF::updateScalarFieldSqrt(const int nFieldIndex, const std::vector<double>& dScalarList,
                                              const int nSubmeshIndex, const double dFactor) {
    updateScalarImpl<double>(this, SV(m_pVolScalarFieldList, nFieldIndex), dScalarList, nSubmeshIndex, dFactor, true,
                             nSubmeshIndex == -1 ? std::vector<int>() : getSubmeshCellIndexList(nSubmeshIndex));
}

void CPolyMeshReaderOF::updateScalarFieldSqrt(const int nFieldIndex, const std::vector<float>& fScalarList,
                                              const int nSubmeshIndex, const float fFactor) {
    updateScalarImpl<float>(this, SV(m_pVolScalarFieldList, nFieldIndex), fScalarList, nSubmeshIndex, fFactor, true,
                            nSubmeshIndex == -1 ? std::vector<int>() : getSubmeshCellIndexList(nSubmeshIndex));
}

void CPolyMeshReaderOF::updateScalarField(const int nFieldIndex, const double dValue, const int nCellIndex) {
    SV(m_pVolScalarFieldList, nFieldIndex)[(size_t)nCellIndex] = dValue;
}

void CPolyMeshReaderOF::updateScalarField(const int nFieldIndex, const float fValue, const int nCellIndex) {
    SV(m_pVolScalarFieldList, nFieldIndex)[(size_t)nCellIndex] = fValue;
}

template <typename T>
static void updateVectorImpl(std::vector<double>& field, const std::vector<T>& v, const std::vector<int>& cells,
                             bool all) {
    if (all) {
        for (size_t i = 0; i < field.size(); ++i) field[i] = v[i];
    } else {
        for (size_t i = 0; i < cells.size(); ++i)
            for (int k = 0; k < 3; ++k) field[(size_t)cells[i] * 3 + k] = v[i * 3 + k];
    }
}

void CPolyMeshReaderOF::updateVectorField(const int nFieldIndex, const std::vector<double>& dVectorList,
                                          const int nSubmeshIndex) {
    updateVectorImpl<double>(SV(m_pVolVectorFieldList, nFieldIndex), dVectorList,
                             nSubmeshIndex == -1 ? std::vector<int>() : getSubmeshCellIndexList(nSubmeshIndex),
                             nSubmeshIndex == -1);
}

void CPolyMeshReaderOF::updateVectorField(const int nFieldIndex, const std::vector<float>& fVectorList,
                                          const int nSubmeshIndex) {
    updateVectorImpl<float>(SV(m_pVolVectorFieldList, nFieldIndex), fVectorList,
                            nSubmeshIndex == -1 ? std::vector<int>() : getSubmeshCellIndexList(nSubmeshIndex),
                            nSubmeshIndex == -1);
}

void CPolyMeshReaderOF::updateVectorField(const int nFieldIndex, const double* pVec, const int nCellIndex) {
    std::vector<double>& f = SV(m_pVolVectorFieldList, nFieldIndex);
    for (int k = 0; k < 3; ++k) f[(size_t)nCellIndex * 3 + k] = pVec[k];
}

void CPolyMeshReaderOF::updateVectorField(const int nFieldIndex, const float* pVec, const int nCellIndex) {
    std::vector<double>& f = SV(m_pVolVectorFieldList, nFieldIndex);
    for (int k = 0; k < 3; ++k) f[(size_t)nCellIndex * 3 + k] = pVec[k];
}

int CPolyMeshReaderOF::getScalarFieldIndex(const std::string& sFieldName) const {
    for (size_t i = 0; i < m_sScalarFieldList.size(); ++i)
        if (m_sScalarFieldList[i] == sFieldName) return (int)i;
    return -1;
}

int CPolyMeshReaderOF::getVectorFieldIndex(const std::string& sFieldName) const {
    for (size_t i = 0; i < m_sVectorFieldList.size(); ++i)
        if (m_sVectorFieldList[i] == sFieldName) return (int)i;
    return -1;
}
