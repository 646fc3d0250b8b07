// Hamiltonian-path cell order (renumber.h, RENUMBER_HPATH).
//
// A restatement of the reference's hpath renumbering method, an OpenFOAM
// renumberMesh plug-in (hpathRenumber/hpathRenumber.C:127-180 and the walks
// it calls, :183-1076), over this build's mesh reader instead of OpenFOAM's
// polyMesh. The reference writes the order into the polyMesh (renumberMesh
// -overwrite) before the solver reads it; the solver's submesh lists are then
// ascending in the new numbering. Here the order is computed when the solver
// description is built and each submesh's cells are sorted by their position
// in it, which gives the same solver order; the polyMesh keeps its numbering.
//
// The walk, as the reference takes it:
//  * boundary cells (submesh 0: cells that own a non-empty boundary face, or
//    have an internal face with a point on one) are walked first, each step
//    moving to the nearest unwalked boundary cell found by a breadth-first
//    search of at most ten rings; a neighbour that would become a dead end
//    (no unwalked same-submesh neighbour of its own) is set aside and
//    appended after the walk;
//  * interior cells (submesh 1) follow, walked from each of a few starting
//    cells with two strategies (hugging the submesh boundary, then moving
//    outwards from the mesh centre; or a spiral that keeps next to the oldest
//    walked cells), backing out of dead-end strips; the walk covering the
//    most cells wins, and the cells it left out follow it.
// Its quirks are kept where they shape the order (the boundary walk's
// "last cell" is fixed at the start; the interior boundary flags mark the
// owner side of a submesh interface). Two cases the reference leaves
// undefined are pinned: a cell with no boundary neighbour reads its flag as
// false (the reference indexes its flag array at -1), and meshes above two
// million cells try one interior start per selection stride of one (the
// reference divides by zero there).
#include "renumber.h"

#include <algorithm>
#include <cmath>
#include <queue>
#include <string>

namespace lfm {

namespace {

enum WalkKind { WALK_STANDARD = 0, WALK_SPIRAL = 1 };

class HpathWalker {
public:
    explicit HpathWalker(IMeshReader& r);
    std::vector<int> order();

private:
    int nc = 0, nf = 0;
    std::vector<int> cellOff, cellFace;   // faces of each cell, the reader's (OpenFOAM's) order
    std::vector<int> owner, nbr;          // nbr = -1 on boundary faces
    std::vector<char> valid;              // not on an 'empty' patch
    std::vector<int> sm;                  // 0 boundary submesh, 1 interior
    std::vector<double> cc;               // cell centres [3 * nc]
    double centre[3] = {0, 0, 0};

    int faces(int c) const { return cellOff[(size_t)c + 1] - cellOff[(size_t)c]; }
    int face(int c, int k) const { return cellFace[(size_t)(cellOff[(size_t)c] + k)]; }
    // the cell across face f from c, -1 across a boundary face
    int across(int c, int f) const {
        if (nbr[(size_t)f] < 0) return -1;
        return owner[(size_t)f] == c ? nbr[(size_t)f] : owner[(size_t)f];
    }
    double dist2(int c) const {
        double s = 0;
        for (int k = 0; k < 3; ++k) {
            const double d = cc[(size_t)(3 * c + k)] - centre[k];
            s += d * d;
        }
        return s;
    }
    int countValid(int c) const {
        int n = 0;
        for (int k = 0; k < faces(c); ++k) n += valid[(size_t)face(c, k)] ? 1 : 0;
        return n;
    }

    void splitSubmeshes(IMeshReader& r);
    bool neighbourIsDeadEnd(int cur, int nb, const std::vector<char>& walked) const;
    // boundary walk
    bool boundaryPath(std::vector<int>& out) const;
    bool boundaryPathFrom(int start, std::vector<int>& out) const;
    int nearestBoundaryCell(std::vector<char>& seen, std::vector<int>& seenList, const std::vector<char>& walked,
                            int from, int deadEnd) const;
    int boundaryDeadEnd(int cur, int last, const std::vector<char>& walked) const;
    // interior walk
    bool interiorPath(std::vector<int>& path, std::vector<int>& dead) const;
    std::vector<int> interiorStarts() const;
    void interiorWalk(int start, WalkKind kind, int& walkedCount, std::vector<int>& path,
                      std::vector<int>& dead) const;
    int interiorDeadEnd(int cur, const std::vector<char>& walked) const;
    int outwardStep(int cur, int deadEnd, const std::vector<char>& walked) const;
    int boundaryHugStep(const std::vector<char>& isBnd, const std::vector<char>& nearBnd, int cur, int deadEnd,
                        const std::vector<char>& walked, bool& switchToOutward) const;
    int spiralStep(const std::vector<char>& isBnd, const std::vector<char>& nearBnd, int cur, int deadEnd,
                   const std::vector<char>& walked, const std::vector<int>& pathIndex) const;
};

HpathWalker::HpathWalker(IMeshReader& r) {
    nc = r.getCellCount();
    nf = r.getFaceCount();
    cellOff.assign((size_t)nc + 1, 0);
    for (int c = 0; c < nc; ++c) cellOff[(size_t)c + 1] = cellOff[(size_t)c] + r.getCellFaceCount(c);
    cellFace.resize((size_t)cellOff.back());
    for (int c = 0; c < nc; ++c)
        for (int k = 0; k < faces(c); ++k) cellFace[(size_t)(cellOff[(size_t)c] + k)] = r.getCellFaceIndex(c, k);
    owner.resize((size_t)nf);
    nbr.assign((size_t)nf, -1);
    valid.assign((size_t)nf, 1);
    for (int f = 0; f < nf; ++f) {
        owner[(size_t)f] = r.getFaceOwner(f);
        const int b = r.getFaceBoundary(f);
        if (b < 0) nbr[(size_t)f] = r.getFaceNeighbour(f);
        else if (r.getBoundaryType(b) == "empty") valid[(size_t)f] = 0;
    }
    cc.resize((size_t)3 * nc);
    for (int c = 0; c < nc; ++c) r.getCellCenter(c, &cc[(size_t)3 * c]);
    // getCenter: the mean of the cell centres
    double s[3] = {0, 0, 0};
    for (int c = 0; c < nc; ++c)
        for (int k = 0; k < 3; ++k) s[k] += cc[(size_t)(3 * c + k)];
    for (int k = 0; k < 3; ++k) centre[k] = s[k] / nc;
    splitSubmeshes(r);
}

// getCellSubmeshIndex (hpathRenumber.C:381-420): owners of valid boundary
// faces and cells with an internal face touching a point of one.
void HpathWalker::splitSubmeshes(IMeshReader& r) {
    sm.assign((size_t)nc, 1);
    std::vector<char> bndPoint((size_t)r.getPointCount(), 0);
    for (int f = 0; f < nf; ++f) {
        if (nbr[(size_t)f] >= 0 || !valid[(size_t)f]) continue;
        for (int k = 0; k < r.getFacePointCount(f); ++k) bndPoint[(size_t)r.getFacePointIndex(f, k)] = 1;
        sm[(size_t)owner[(size_t)f]] = 0;
    }
    for (int f = 0; f < nf; ++f) {
        if (nbr[(size_t)f] < 0) continue;
        for (int k = 0; k < r.getFacePointCount(f); ++k)
            if (bndPoint[(size_t)r.getFacePointIndex(f, k)]) {
                sm[(size_t)owner[(size_t)f]] = 0;
                sm[(size_t)nbr[(size_t)f]] = 0;
                break;
            }
    }
}

// isNeighbourDeadend (:264-272): nb has no unwalked neighbour of cur's
// submesh other than cur.
bool HpathWalker::neighbourIsDeadEnd(int cur, int nb, const std::vector<char>& walked) const {
    for (int k = 0; k < faces(nb); ++k) {
        const int x = across(nb, face(nb, k));
        if (x < 0 || x == cur || walked[(size_t)x] || sm[(size_t)x] != sm[(size_t)cur]) continue;
        return false;
    }
    return true;
}

// getBoundaryHpath (:183-230): start from the first boundary cell, else from
// quadrilaterals (four valid faces) with more than one boundary neighbour;
// at most ten starts.
bool HpathWalker::boundaryPath(std::vector<int>& out) const {
    std::vector<int> starts;
    for (int c = 0; c < nc; ++c)
        if (sm[(size_t)c] == 0) {
            starts.push_back(c);
            break;
        }
    for (int c = 0; c < nc && starts.size() < 10; ++c) {
        if (sm[(size_t)c] != 0 || countValid(c) < 4) continue;
        int good = 0;
        for (int k = 0; k < faces(c); ++k) {
            const int f = face(c, k);
            if (!valid[(size_t)f]) continue;
            if (nbr[(size_t)f] >= 0 && sm[(size_t)across(c, f)] == 0 && ++good > 1) break;
        }
        if (good > 1) starts.push_back(c);
    }
    for (int s : starts)
        if (boundaryPathFrom(s, out)) return true;
    return false;
}

// getNextBoundaryHpathCell (:233-262): breadth-first search from `from`, at
// most ten rings, for the nearest unwalked boundary cell other than the dead
// end set aside.
int HpathWalker::nearestBoundaryCell(std::vector<char>& seen, std::vector<int>& seenList,
                                     const std::vector<char>& walked, int from, int deadEnd) const {
    for (int c : seenList) seen[(size_t)c] = 0;
    seenList.clear();
    std::queue<int> q;
    q.push(from);
    q.push(-1);
    int ring = 0;
    while (!q.empty() && ring <= 10) {
        const int c = q.front();
        q.pop();
        if (c == -1) {
            ++ring;
            q.push(-1);
            continue;
        }
        if (seen[(size_t)c]) continue;
        seen[(size_t)c] = 1;
        seenList.push_back(c);
        if (c != from && !walked[(size_t)c] && c != deadEnd && sm[(size_t)c] == 0) return c;
        for (int k = 0; k < faces(c); ++k) {
            const int x = across(c, face(c, k));
            if (x > -1 && !seen[(size_t)x]) q.push(x);
        }
    }
    return -1;
}

// getDeadendNeighbourBnd (:274-292): with more than one way on, a neighbour
// (other than `last`) that would become a dead end.
int HpathWalker::boundaryDeadEnd(int cur, int last, const std::vector<char>& walked) const {
    int left = faces(cur);
    for (int k = 0; k < faces(cur); ++k) {
        const int x = across(cur, face(cur, k));
        if (x < 0 || walked[(size_t)x] || sm[(size_t)x] != sm[(size_t)cur]) --left;
    }
    if (left <= 1) return -1;
    for (int k = 0; k < faces(cur); ++k) {
        const int x = across(cur, face(cur, k));
        if (x < 0 || walked[(size_t)x] || x == last || sm[(size_t)x] != sm[(size_t)cur]) continue;
        if (neighbourIsDeadEnd(cur, x, walked)) return x;
    }
    return -1;
}

// findBoundaryHpath (:294-378).
bool HpathWalker::boundaryPathFrom(int start, std::vector<int>& out) const {
    std::vector<char> walked((size_t)nc, 0), isDead((size_t)nc, 0), seen((size_t)nc, 0);
    std::vector<int> seenList, path, dead;
    int last = -1;
    const int first = nearestBoundaryCell(seen, seenList, walked, start, -1);
    const int nValid = countValid(start);
    for (int k = 0; k < faces(start); ++k) {
        const int f = face(start, k);
        if (nbr[(size_t)f] < 0) continue;
        const int x = across(start, f);
        if (sm[(size_t)x] != 0) continue;
        if (nValid != 3 || x != first) last = x;
    }
    int next = start;
    do {
        const int cur = next;
        walked[(size_t)cur] = 1;
        path.push_back(cur);
        const int d = boundaryDeadEnd(cur, last, walked);
        if (d > -1) {
            dead.push_back(d);
            isDead[(size_t)d] = 1;
        }
        next = nearestBoundaryCell(seen, seenList, walked, cur, d);
    } while (next != -1);
    for (int c = 0; c < nc; ++c)
        if (sm[(size_t)c] == 0 && !walked[(size_t)c] && !isDead[(size_t)c]) dead.push_back(c);
    out = path;
    for (int c : dead)
        if (!walked[(size_t)c]) out.push_back(c);
    int nBoundary = 0;
    for (int c = 0; c < nc; ++c) nBoundary += sm[(size_t)c] == 0 ? 1 : 0;
    return (int)out.size() == nBoundary;
}

// getInteriorStartingCells (:434-600): interior cells next to the boundary
// submesh whose neighbours leave room to walk on, sorted by their angle about
// the mesh centre, thinned to about two million cells of walking in all.
std::vector<int> HpathWalker::interiorStarts() const {
    std::vector<char> isBnd((size_t)nc, 0);
    for (int f = 0; f < nf; ++f) {
        if (nbr[(size_t)f] < 0) continue;
        const int a = owner[(size_t)f], b = nbr[(size_t)f];
        if (sm[(size_t)a] != sm[(size_t)b]) isBnd[(size_t)a] = isBnd[(size_t)b] = 1;
    }
    std::vector<int> bnd;
    for (int c = 0; c < nc; ++c) {
        if (sm[(size_t)c] != 1) isBnd[(size_t)c] = 0;
        if (isBnd[(size_t)c]) bnd.push_back(c);
    }
    auto isBndAt = [&](int c) { return c >= 0 && isBnd[(size_t)c]; };
    // neighbours of "irregular" cells (fewer than two interior neighbours);
    // a cell without any keeps the previous cell's last neighbour, as the
    // reference's loop variable does
    std::vector<char> nearIrregular((size_t)nc, 0);
    int lastRegular = -1;
    for (int b : bnd) {
        int reg = 0;
        for (int k = 0; k < faces(b); ++k) {
            const int f = face(b, k);
            if (!valid[(size_t)f]) continue;
            const int x = across(b, f);
            if (x < 0 || sm[(size_t)x] != 1) continue;
            ++reg;
            lastRegular = x;
        }
        if (reg < 2 && lastRegular >= 0) nearIrregular[(size_t)lastRegular] = 1;
    }
    std::vector<int> cand;
    for (int b : bnd) {
        bool ok = true;
        for (int k = 0; k < faces(b) && ok; ++k) {   // condition 0
            const int f = face(b, k);
            if (!valid[(size_t)f]) continue;
            const int x = across(b, f);
            if (x < 0 || sm[(size_t)x] != 1) continue;
            if (nearIrregular[(size_t)x]) ok = false;
        }
        if (!ok) continue;
        int roomy = 0;   // condition 1: neighbours with two more interior neighbours
        for (int k = 0; k < faces(b); ++k) {
            const int f = face(b, k);
            if (!valid[(size_t)f]) continue;
            const int x = across(b, f);
            if (x < 0 || sm[(size_t)x] != 1) continue;
            int reg = 0;
            for (int j = 0; j < faces(x); ++j) {
                const int g = face(x, j);
                if (!valid[(size_t)g]) continue;
                const int y = across(x, g);
                if (y < 0 || sm[(size_t)y] != 1 || y == b) continue;
                ++reg;
            }
            if (reg > 1) ++roomy;
        }
        if (roomy < 2) continue;
        int touching = 0;   // condition 2: neighbours next to the submesh interface
        for (int k = 0; k < faces(b); ++k) {
            const int x = across(b, face(b, k));
            if (x < 0 || sm[(size_t)x] != 1) continue;
            bool has = false;
            for (int j = 0; j < faces(x) && !has; ++j) has = isBndAt(across(x, face(x, j)));
            if (has) ++touching;
        }
        if (touching >= 2) cand.push_back(b);
    }
    if (cand.empty() && !bnd.empty()) {   // the interface cell farthest from the centre
        int far = bnd[0];
        double dmax = dist2(bnd[0]);
        for (int b : bnd)
            if (dist2(b) > dmax) {
                dmax = dist2(b);
                far = b;
            }
        cand.push_back(far);
    }
    // sort by (angle, index) in single precision, as the reference stores them
    std::vector<std::pair<float, float>> ang(cand.size());
    for (size_t i = 0; i < cand.size(); ++i) {
        const int c = cand[i];
        ang[i] = {(float)std::atan2(cc[(size_t)(3 * c + 1)] - centre[1], cc[(size_t)(3 * c)] - centre[0]), (float)i};
    }
    std::sort(ang.begin(), ang.end());
    const int n = (int)cand.size();
    const int maxIter = std::max(1, 2000000 / std::max(1, nc));
    const int ratio = maxIter > n ? 1 : n / maxIter;
    std::vector<int> out;
    for (int i = 0; i < n; ++i)
        if (i % ratio == 0) out.push_back(cand[(size_t)(int)ang[(size_t)i].second]);
    return out;
}

// getInteriorDeadendNeighbour (:603-633).
int HpathWalker::interiorDeadEnd(int cur, const std::vector<char>& walked) const {
    const int s = sm[(size_t)cur];
    int left = 0;
    for (int k = 0; k < faces(cur); ++k) {
        const int f = face(cur, k);
        if (!valid[(size_t)f]) continue;
        const int x = across(cur, f);
        if (x < 0 || sm[(size_t)x] != s || walked[(size_t)x]) continue;
        ++left;
    }
    if (left <= 1) return -1;
    for (int k = 0; k < faces(cur); ++k) {
        const int f = face(cur, k);
        if (!valid[(size_t)f]) continue;
        const int x = across(cur, f);
        if (x < 0 || sm[(size_t)x] != s || walked[(size_t)x]) continue;
        if (neighbourIsDeadEnd(cur, x, walked)) return x;
    }
    return -1;
}

// getInteriorNextHpathCell (:636-668): the free neighbour farthest from the
// mesh centre (the only one, when there is one).
int HpathWalker::outwardStep(int cur, int deadEnd, const std::vector<char>& walked) const {
    const int s = sm[(size_t)cur];
    std::vector<int> freeCells;
    for (int k = 0; k < faces(cur); ++k) {
        const int x = across(cur, face(cur, k));
        if (x < 0 || sm[(size_t)x] != s || walked[(size_t)x]) continue;
        freeCells.push_back(x);
    }
    if (freeCells.size() == 1) return freeCells[0];
    int next = -1;
    double dmax = 0;
    for (int x : freeCells) {
        if (x == deadEnd) continue;
        const double d = std::sqrt(dist2(x));
        if (dmax < d) {
            dmax = d;
            next = x;
        }
    }
    return next;
}

// getInteriorNextHpathCellBnd (:671-718): interface cells first, then their
// neighbours, then a cell two steps away next to one; otherwise any free
// neighbour, and the walk switches to the outward rule.
int HpathWalker::boundaryHugStep(const std::vector<char>& isBnd, const std::vector<char>& nearBnd, int cur,
                                 int deadEnd, const std::vector<char>& walked, bool& switchToOutward) const {
    const int s = sm[(size_t)cur];
    auto free = [&](int x) { return x >= 0 && sm[(size_t)x] == s && !walked[(size_t)x] && x != deadEnd; };
    for (int k = 0; k < faces(cur); ++k) {
        const int x = across(cur, face(cur, k));
        if (free(x) && isBnd[(size_t)x]) return x;
    }
    for (int k = 0; k < faces(cur); ++k) {
        const int x = across(cur, face(cur, k));
        if (free(x) && nearBnd[(size_t)x]) return x;
    }
    for (int k = 0; k < faces(cur); ++k) {
        const int x = across(cur, face(cur, k));
        if (!free(x)) continue;
        for (int j = 0; j < faces(x); ++j) {
            const int y = across(x, face(x, j));
            if (y < 0 || sm[(size_t)y] != s || walked[(size_t)y]) continue;
            if (nearBnd[(size_t)y]) return y;
        }
    }
    for (int k = 0; k < faces(cur); ++k) {
        const int x = across(cur, face(cur, k));
        if (!free(x)) continue;
        switchToOutward = true;
        return x;
    }
    return -1;
}

// getInteriorNextHpathCellSpiral (:720-846).
int HpathWalker::spiralStep(const std::vector<char>& isBnd, const std::vector<char>& nearBnd, int cur, int deadEnd,
                            const std::vector<char>& walked, const std::vector<int>& pathIndex) const {
    const int s = sm[(size_t)cur];
    std::vector<int> onBnd, nearList, plain;
    for (int k = 0; k < faces(cur); ++k) {
        const int x = across(cur, face(cur, k));
        if (x < 0 || sm[(size_t)x] != s || walked[(size_t)x] || x == deadEnd) continue;
        if (isBnd[(size_t)x]) onBnd.push_back(x);
        else if (nearBnd[(size_t)x]) nearList.push_back(x);
        else plain.push_back(x);
    }
    if (!onBnd.empty()) return onBnd[0];
    if (!nearList.empty()) {   // the one next to the earliest walked interface cell
        int oldest = 2 * nc, best = -1;
        for (int x : nearList)
            for (int j = 0; j < faces(x); ++j) {
                const int y = across(x, face(x, j));
                if (y < 0 || sm[(size_t)y] != s || !isBnd[(size_t)y]) continue;
                if (oldest > pathIndex[(size_t)y]) {
                    oldest = pathIndex[(size_t)y];
                    best = x;
                }
            }
        if (best != -1) return best;
    }
    if (plain.empty()) return -1;
    if (plain.size() == 1) return plain[0];
    // a free neighbour next to the earliest walked cell
    int oldest = 2 * nc, best = -1;
    for (int x : plain)
        for (int j = 0; j < faces(x); ++j) {
            const int y = across(x, face(x, j));
            if (y < 0 || !walked[(size_t)y] || y == cur) continue;
            if (oldest > pathIndex[(size_t)y]) {
                oldest = pathIndex[(size_t)y];
                best = x;
            }
        }
    if (best != -1) return best;
    // two steps away, ignoring the last few cells walked
    oldest = 2 * nc;
    for (int x : plain)
        for (int j = 0; j < faces(x); ++j) {
            const int y = across(x, face(x, j));
            if (y < 0 || y == cur) continue;
            for (int i = 0; i < faces(y); ++i) {
                const int z = across(y, face(y, i));
                if (z < 0 || !walked[(size_t)z]) continue;
                if (pathIndex[(size_t)cur] - pathIndex[(size_t)z] < 3) continue;
                if (oldest > pathIndex[(size_t)z]) {
                    oldest = pathIndex[(size_t)z];
                    best = x;
                }
            }
        }
    if (best > -1) return best;
    oldest = 2 * nc;
    for (int x : plain)
        for (int j = 0; j < faces(x); ++j) {
            const int y = across(x, face(x, j));
            if (y < 0) continue;
            for (int i = 0; i < faces(y); ++i) {
                const int z = across(y, face(y, i));
                if (z < 0 || !walked[(size_t)z]) continue;
                if (oldest > pathIndex[(size_t)z]) {
                    oldest = pathIndex[(size_t)z];
                    best = x;
                }
            }
        }
    return best == -1 ? plain[0] : best;
}

// findInteriorHpathNoDeadend (:874-1023).
void HpathWalker::interiorWalk(int start, WalkKind kind, int& walkedCount, std::vector<int>& path,
                               std::vector<int>& dead) const {
    std::vector<char> isBnd((size_t)nc, 0), nearBnd((size_t)nc, 0);
    int nInterior = 0;
    for (int c = 0; c < nc; ++c) nInterior += sm[(size_t)c] == 1 ? 1 : 0;
    for (int f = 0; f < nf; ++f) {   // the owner side of the submesh interface (the reference's flags)
        if (nbr[(size_t)f] < 0) continue;
        const int a = owner[(size_t)f], b = nbr[(size_t)f];
        if (sm[(size_t)a] != sm[(size_t)b] && (sm[(size_t)a] == 1 || sm[(size_t)b] == 1)) isBnd[(size_t)a] = 1;
    }
    for (int f = 0; f < nf; ++f) {
        if (nbr[(size_t)f] < 0) continue;
        const int a = owner[(size_t)f], b = nbr[(size_t)f];
        if (sm[(size_t)a] != sm[(size_t)b] || sm[(size_t)a] != 1) continue;
        if (isBnd[(size_t)a]) nearBnd[(size_t)b] = 1;
        if (isBnd[(size_t)b]) nearBnd[(size_t)a] = 1;
    }
    std::vector<int> tmp((size_t)nc, -1), pathIndex((size_t)nc, -1);
    std::vector<char> walked((size_t)nc, 0);
    int idx = 0, outside = 0, next = start;
    bool outward = false;
    do {
        const int cur = next;
        pathIndex[(size_t)cur] = idx;
        tmp[(size_t)idx++] = cur;
        walked[(size_t)cur] = 1;
        const int d = interiorDeadEnd(cur, walked);
        if (d > -1) ++outside;
        if (kind == WALK_SPIRAL) next = spiralStep(isBnd, nearBnd, cur, d, walked, pathIndex);
        else if (outward) next = outwardStep(cur, d, walked);
        else next = boundaryHugStep(isBnd, nearBnd, cur, d, walked, outward);
        if (next == -1 && idx + outside < nInterior) {
            // stuck in a dead-end strip: walk back until a cell offers another way
            int back = 1, restart = -1;
            bool found = false;
            do {
                if (idx - back <= 0) break;
                const int blocked = tmp[(size_t)(idx - back)];
                const int from = tmp[(size_t)(idx - back - 1)];
                if (from == -1) break;
                restart = outwardStep(from, blocked, walked);
                if (restart != -1) found = true;
                else ++back;
                if (back == 60) break;
            } while (!found);
            if (restart == -1) break;
            for (int k = 1; k < back - 1; ++k) {
                const int c = tmp[(size_t)(idx - k)];
                walked[(size_t)c] = 0;
                pathIndex[(size_t)c] = -1;
                tmp[(size_t)(idx - k)] = -1;
                ++outside;
            }
            next = restart;
            idx -= back;
        }
        if (next != -1) walked[(size_t)next] = 1;
    } while (next != -1);
    path.assign(tmp.begin(), tmp.begin() + idx);
    // cells left out: first those next to the path, in path order, then the rest
    std::vector<char> onPath((size_t)nc, 0), recorded((size_t)nc, 0);
    for (int c : path) onPath[(size_t)c] = 1;
    dead.clear();
    for (int c : path)
        for (int k = 0; k < faces(c); ++k) {
            const int x = across(c, face(c, k));
            if (x < 0 || sm[(size_t)x] != 1 || onPath[(size_t)x] || recorded[(size_t)x]) continue;
            dead.push_back(x);
            recorded[(size_t)x] = 1;
        }
    for (int c = 0; c < nc; ++c)
        if (sm[(size_t)c] == 1 && !onPath[(size_t)c] && !recorded[(size_t)c]) {
            dead.push_back(c);
            recorded[(size_t)c] = 1;
        }
    walkedCount = idx;
}

// getInteriorHpath (:1026-1076): every start with both walks; the walk
// covering the most cells (first found on ties) is taken.
bool HpathWalker::interiorPath(std::vector<int>& path, std::vector<int>& dead) const {
    const std::vector<int> starts = interiorStarts();
    int nInterior = 0;
    for (int c = 0; c < nc; ++c) nInterior += sm[(size_t)c] == 1 ? 1 : 0;
    int best = -1, bestStart = -1;
    WalkKind bestKind = WALK_STANDARD;
    std::vector<int> p, d;
    for (int kind = WALK_STANDARD; kind <= WALK_SPIRAL; ++kind)
        for (int s : starts) {
            int walkedCount = 0;
            interiorWalk(s, (WalkKind)kind, walkedCount, p, d);
            if ((int)(p.size() + d.size()) != nInterior) continue;
            if (best < walkedCount) {
                best = walkedCount;
                bestStart = s;
                bestKind = (WalkKind)kind;
            }
        }
    if (bestStart < 0) return false;
    int walkedCount = 0;
    interiorWalk(bestStart, bestKind, walkedCount, path, dead);
    return true;
}

// renumber (:127-180): the boundary walk, then the interior walk and the
// cells it left out; a submesh whose walk fails keeps its cells ascending.
std::vector<int> HpathWalker::order() {
    std::vector<int> out;
    out.reserve((size_t)nc);
    std::vector<int> bpath;
    if (boundaryPath(bpath)) {
        out = bpath;
    } else {
        for (int c = 0; c < nc; ++c)
            if (sm[(size_t)c] == 0) out.push_back(c);
    }
    std::vector<int> ipath, idead;
    if (interiorPath(ipath, idead)) {
        out.insert(out.end(), ipath.begin(), ipath.end());
        out.insert(out.end(), idead.begin(), idead.end());
    } else {
        for (int c = 0; c < nc; ++c)
            if (sm[(size_t)c] == 1) out.push_back(c);
    }
    return out;
}

}  // namespace

std::vector<int> hpathCellOrder(IMeshReader& r) {
    HpathWalker w(r);
    std::vector<int> order = w.order();
    // a permutation of the cells, or nothing (the caller keeps its order)
    std::vector<char> seen((size_t)r.getCellCount(), 0);
    if ((int)order.size() != r.getCellCount()) return {};
    for (int c : order) {
        if (c < 0 || c >= r.getCellCount() || seen[(size_t)c]) return {};
        seen[(size_t)c] = 1;
    }
    return order;
}

}  // namespace lfm
