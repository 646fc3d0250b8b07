// Internal case objects: mesh geometry and time control (see foam_case.h).
#include "foam_case.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <dirent.h>
#include <sys/stat.h>

namespace lfm {

// ----------------------------------------------------------------------------
int FoamMesh::whichPatch(int64_t face) const {
    if (face < nInternalFaces()) return -1;
    for (size_t p = 0; p < patches.size(); ++p)
        if (face >= patches[p].startFace && face < patches[p].startFace + patches[p].nFaces)
            return (int)p;
    return -1;
}

void FoamMesh::finalize() {
    const int64_t nf = nFaces();
    if ((int64_t)faceOffsets.size() != nf + 1)
        throw foam::FoamError("faces and owner lists differ in length");
    if (nInternalFaces() > nf) throw foam::FoamError("more neighbours than faces");
    int64_t maxCell = -1;
    for (int64_t c : owner) maxCell = std::max(maxCell, c);
    for (int64_t c : neighbour) maxCell = std::max(maxCell, c);
    if (nCells <= 0) nCells = maxCell + 1;
    for (int64_t c : owner)
        if (c < 0 || c >= nCells) throw foam::FoamError("owner label out of range");
    for (int64_t c : neighbour)
        if (c < 0 || c >= nCells) throw foam::FoamError("neighbour label out of range");
    for (int64_t p : facePoints)
        if (p < 0 || p >= nPoints()) throw foam::FoamError("face point label out of range");

    // Cell -> faces in OpenFOAM's order (primitiveMesh::calcCells): every face
    // is appended to its owner's list in face order, then every internal face
    // to its neighbour's list in face order.
    std::vector<int64_t> count((size_t)nCells, 0);
    for (int64_t f = 0; f < nf; ++f) ++count[(size_t)owner[(size_t)f]];
    for (int64_t f = 0; f < nInternalFaces(); ++f) ++count[(size_t)neighbour[(size_t)f]];
    cellOffsets.assign((size_t)nCells + 1, 0);
    for (int64_t c = 0; c < nCells; ++c) cellOffsets[(size_t)c + 1] = cellOffsets[(size_t)c] + count[(size_t)c];
    cellFaces.assign((size_t)cellOffsets.back(), 0);
    std::vector<int64_t> fill(cellOffsets.begin(), cellOffsets.end() - 1);
    for (int64_t f = 0; f < nf; ++f) cellFaces[(size_t)fill[(size_t)owner[(size_t)f]]++] = f;
    for (int64_t f = 0; f < nInternalFaces(); ++f)
        cellFaces[(size_t)fill[(size_t)neighbour[(size_t)f]]++] = f;

    computeGeometry(*this);
}

// ----------------------------------------------------------------------------
void computeGeometry(FoamMesh& m) {
    const int64_t nf = m.nFaces();
    const double* p = m.points.data();
    m.faceAreas.assign((size_t)nf * 3, 0.0);
    m.faceCentres.assign((size_t)nf * 3, 0.0);
    const double kRootVSmall = 1.0e-150, kVSmall = 1.0e-300;

    for (int64_t f = 0; f < nf; ++f) {
        const int64_t* fp = m.facePoints.data() + m.faceOffsets[(size_t)f];
        const int64_t np = m.faceOffsets[(size_t)f + 1] - m.faceOffsets[(size_t)f];
        double* ctr = &m.faceCentres[(size_t)(3 * f)];
        double* area = &m.faceAreas[(size_t)(3 * f)];
        if (np == 3) {
            const double* a = p + 3 * fp[0];
            const double* b = p + 3 * fp[1];
            const double* c = p + 3 * fp[2];
            for (int k = 0; k < 3; ++k) ctr[k] = (1.0 / 3.0) * (a[k] + b[k] + c[k]);
            const double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
            const double v[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
            area[0] = 0.5 * (u[1] * v[2] - u[2] * v[1]);
            area[1] = 0.5 * (u[2] * v[0] - u[0] * v[2]);
            area[2] = 0.5 * (u[0] * v[1] - u[1] * v[0]);
            continue;
        }
        double fc[3] = {p[3 * fp[0]], p[3 * fp[0] + 1], p[3 * fp[0] + 2]};
        for (int64_t i = 1; i < np; ++i)
            for (int k = 0; k < 3; ++k) fc[k] += p[3 * fp[i] + k];
        for (int k = 0; k < 3; ++k) fc[k] /= (double)np;
        double sumN[3] = {0, 0, 0}, sumAc[3] = {0, 0, 0}, sumA = 0.0;
        for (int64_t i = 0; i < np; ++i) {
            const double* t = p + 3 * fp[i];
            const double* nx = p + 3 * fp[(i == np - 1) ? 0 : i + 1];
            const double c[3] = {t[0] + nx[0] + fc[0], t[1] + nx[1] + fc[1], t[2] + nx[2] + fc[2]};
            const double u[3] = {nx[0] - t[0], nx[1] - t[1], nx[2] - t[2]};
            const double v[3] = {fc[0] - t[0], fc[1] - t[1], fc[2] - t[2]};
            const double n[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2],
                                 u[0] * v[1] - u[1] * v[0]};
            const double a = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            for (int k = 0; k < 3; ++k) {
                sumN[k] += n[k];
                sumAc[k] += a * c[k];
            }
            sumA += a;
        }
        if (sumA < kRootVSmall) {
            for (int k = 0; k < 3; ++k) {
                ctr[k] = fc[k];
                area[k] = 0.0;
            }
        } else {
            for (int k = 0; k < 3; ++k) {
                ctr[k] = (1.0 / 3.0) * sumAc[k] / sumA;
                area[k] = 0.5 * sumN[k];
            }
        }
    }

    const int64_t nc = m.nCells;
    m.cellCentres.assign((size_t)nc * 3, 0.0);
    m.cellVolumes.assign((size_t)nc, 0.0);
    std::vector<double> est((size_t)nc * 3, 0.0);
    std::vector<int64_t> nFacesOf((size_t)nc, 0);
    const int64_t ni = m.nInternalFaces();
    for (int64_t f = 0; f < nf; ++f) {
        const int64_t c = m.owner[(size_t)f];
        for (int k = 0; k < 3; ++k) est[(size_t)(3 * c + k)] += m.faceCentres[(size_t)(3 * f + k)];
        ++nFacesOf[(size_t)c];
    }
    for (int64_t f = 0; f < ni; ++f) {
        const int64_t c = m.neighbour[(size_t)f];
        for (int k = 0; k < 3; ++k) est[(size_t)(3 * c + k)] += m.faceCentres[(size_t)(3 * f + k)];
        ++nFacesOf[(size_t)c];
    }
    for (int64_t c = 0; c < nc; ++c)
        for (int k = 0; k < 3; ++k) est[(size_t)(3 * c + k)] /= (double)nFacesOf[(size_t)c];

    auto accumulate = [&](int64_t f, int64_t c, bool isOwner) {
        const double* fc = &m.faceCentres[(size_t)(3 * f)];
        const double* fa = &m.faceAreas[(size_t)(3 * f)];
        const double* ce = &est[(size_t)(3 * c)];
        double pyr3 = 0.0;
        if (isOwner)
            pyr3 = fa[0] * (fc[0] - ce[0]) + fa[1] * (fc[1] - ce[1]) + fa[2] * (fc[2] - ce[2]);
        else
            pyr3 = fa[0] * (ce[0] - fc[0]) + fa[1] * (ce[1] - fc[1]) + fa[2] * (ce[2] - fc[2]);
        for (int k = 0; k < 3; ++k) {
            const double pc = (3.0 / 4.0) * fc[k] + (1.0 / 4.0) * ce[k];
            m.cellCentres[(size_t)(3 * c + k)] += pyr3 * pc;
        }
        m.cellVolumes[(size_t)c] += pyr3;
    };
    for (int64_t f = 0; f < nf; ++f) accumulate(f, m.owner[(size_t)f], true);
    for (int64_t f = 0; f < ni; ++f) accumulate(f, m.neighbour[(size_t)f], false);
    for (int64_t c = 0; c < nc; ++c) {
        if (std::fabs(m.cellVolumes[(size_t)c]) > kVSmall) {
            for (int k = 0; k < 3; ++k) m.cellCentres[(size_t)(3 * c + k)] /= m.cellVolumes[(size_t)c];
        } else {
            for (int k = 0; k < 3; ++k) m.cellCentres[(size_t)(3 * c + k)] = est[(size_t)(3 * c + k)];
        }
        m.cellVolumes[(size_t)c] *= (1.0 / 3.0);
    }
}

// ----------------------------------------------------------------------------
std::string FoamTime::casePath() const {
    if (caseName.empty() || caseName == ".") return rootPath;
    return rootPath + "/" + caseName;
}

// Dictionaries of a processor case live in the parent case (OpenFOAM reads
// system/ and constant/ dictionaries of processorN from the global case).
std::string FoamTime::dictPath(const std::string& dir, const std::string& name) const {
    const std::string local = casePath() + "/" + dir + "/" + name;
    if (!processorCase || foam::fileExists(local)) return local;
    return rootPath + "/" + dir + "/" + name;
}

std::string FoamTime::timeName(double t) const {
    if (timeFormat == "fixed") {
        char buf[64];
        std::snprintf(buf, sizeof(buf), "%.*f", timePrecision, t);
        return buf;
    }
    if (timeFormat == "scientific") {
        char buf[64];
        std::snprintf(buf, sizeof(buf), "%.*e", timePrecision, t);
        return buf;
    }
    return foam::formatGeneral(t, timePrecision);
}

static double dictScalar(const foam::Dict& d, const char* key, double dflt) {
    const foam::Entry* e = d.find(key);
    if (!e || e->tokens.empty()) return dflt;
    return foam::tokenToScalar(e->tokens[0], key);
}

static std::string dictWord(const foam::Dict& d, const char* key, const std::string& dflt) {
    const foam::Entry* e = d.find(key);
    if (!e || e->tokens.empty()) return dflt;
    return e->tokens[0].text;
}

static bool isTimeDir(const std::string& name, double* t) {
    char* e = nullptr;
    const double v = std::strtod(name.c_str(), &e);
    if (e == name.c_str() || *e != '\0') return false;
    *t = v;
    return true;
}

void FoamTime::loadControlDict() {
    const foam::Dict& d = controlDict;
    startTime = dictScalar(d, "startTime", 0.0);
    endTime = dictScalar(d, "endTime", 0.0);
    deltaT = dictScalar(d, "deltaT", 1.0);
    writeControl = dictWord(d, "writeControl", "timeStep");
    writeInterval = dictScalar(d, "writeInterval", 1.0);
    writePrecision = (int)dictScalar(d, "writePrecision", 6);
    writeBinary = dictWord(d, "writeFormat", "ascii") == "binary";
    timeFormat = dictWord(d, "timeFormat", "general");
    timePrecision = (int)dictScalar(d, "timePrecision", 6);
    bool ok = true;
    adjustTimeStep = foam::wordToBool(dictWord(d, "adjustTimeStep", "no"), &ok);
    maxCo = dictScalar(d, "maxCo", 1.0);
    maxDeltaT = dictScalar(d, "maxDeltaT", 1e300);
    const std::string startFrom = dictWord(d, "startFrom", "startTime");
    if (!memory && (startFrom == "latestTime" || startFrom == "firstTime")) {
        // Pick the largest (or smallest) time directory of the case.
        DIR* dir = opendir(casePath().c_str());
        bool found = false;
        double best = 0;
        if (dir) {
            while (dirent* ent = readdir(dir)) {
                double t = 0;
                if (!isTimeDir(ent->d_name, &t)) continue;
                if (!found || (startFrom == "latestTime" ? t > best : t < best)) best = t;
                found = true;
            }
            closedir(dir);
        }
        if (found) startTime = best;
    }
    value = startTime;
    timeIndex = startTimeIndex = 0;
    writeTimeIndex = 0;
    writeTime = false;
}

// Foam::Time::operator++: advance by deltaT and decide whether this is a write
// time (timeStep control: every writeInterval steps; runTime control: when
// the time passes the next multiple of writeInterval after startTime).
void FoamTime::increment() {
    value += deltaT;
    ++timeIndex;
    writeTime = false;
    if (writeControl == "timeStep") {
        const int64_t every = std::max<int64_t>(1, (int64_t)writeInterval);
        writeTime = (timeIndex % every) == 0;
    } else if (writeControl == "runTime" || writeControl == "adjustableRunTime") {
        const int64_t idx = (int64_t)(((value - startTime) + 0.5 * deltaT) / writeInterval);
        if (idx > writeTimeIndex) {
            writeTime = true;
            writeTimeIndex = idx;
        }
    }
}

void FoamTime::write() {
    if (memory) return;
    const std::string dir = casePath() + "/" + timeName();
    mkdir(dir.c_str(), 0777);
    for (FieldObject* f : registry) {
        if (!f->autoWrite) continue;
        foam::writeVolField(dir + "/" + f->data.name, f->data, timeName(), writePrecision,
                            writeBinary);
    }
}

FoamTime* newFoamTime(const std::string& root, const std::string& caseName) {
    FoamTime* t = new FoamTime;
    t->rootPath = root;
    t->caseName = caseName;
    t->processorCase = caseName.rfind("processor", 0) == 0;
    t->controlDict = foam::parseDictFile(t->dictPath("system", "controlDict"));
    t->loadControlDict();
    return t;
}

}  // namespace lfm
