// Tiles of the fused FP32-bulk stage kernel (tiles.h, csrc/cuda/tile_desc.h).
#include "tiles.h"

#include <algorithm>
#include <stdexcept>

namespace lfm {

namespace {

inline int faceOf(int64_t code) { return code >= 0 ? (int)code : (int)~code; }

}  // namespace

TileSet buildTiles(const lfm_solver_desc* d, int tileCells, int maxLocal) {
    if (d->n_halos > 0) throw std::runtime_error("tiles: descriptions with processor halos are not tiled");
    if (tileCells < 1) throw std::runtime_error("tiles: tile size must be positive");
    const int D = d->dim;
    const int nc = (int)d->n_cells, ng = (int)d->n_ghosts, nf = (int)d->n_faces, nt = nc + ng;
    TileSet ts;
    ts.dim = D;
    ts.tileCells = tileCells;
    // cell -> face codes (face index, one's complement when the cell is N)
    auto codesOf = [&](int c, std::vector<int64_t>& out) {
        out.clear();
        for (int64_t e = d->cell_face_offsets[c]; e < d->cell_face_offsets[c + 1]; ++e)
            out.push_back(d->cell_face_sign[e] > 0 ? d->cell_faces[e] : ~d->cell_faces[e]);
    };
    std::vector<int> localOf((size_t)nt, -1), faceLocal((size_t)nf, -1);
    std::vector<int64_t> codes;
    // Builds the tile of cells [c0, c1) and appends it when its local cells
    // fit maxLocal (or it has one cell); otherwise returns false untouched.
    auto tryTile = [&](int c0, int c1) -> bool {
        TileDesc td{};
        td.c0 = c0;
        td.nA = c1 - c0;
        std::vector<int> L, FA, FB, B1, B2, C;
        for (int c = c0; c < c1; ++c) {
            localOf[(size_t)c] = (int)L.size();
            L.push_back(c);
        }
        // faces of A, and what lies across them
        for (int c = c0; c < c1; ++c) {
            codesOf(c, codes);
            for (int64_t code : codes) FA.push_back(faceOf(code));
        }
        std::sort(FA.begin(), FA.end());
        FA.erase(std::unique(FA.begin(), FA.end()), FA.end());
        for (int f : FA)
            for (int x : {(int)d->face_p[f], (int)d->face_n[f]}) {
                if (localOf[(size_t)x] != -1) continue;   // in A, or already seen
                localOf[(size_t)x] = -2;
                (x < nc ? B1 : B2).push_back(x);
            }
        std::sort(B1.begin(), B1.end());
        std::sort(B2.begin(), B2.end());
        for (int x : B1) {
            localOf[(size_t)x] = (int)L.size();
            L.push_back(x);
        }
        for (int x : B2) {
            localOf[(size_t)x] = (int)L.size();
            L.push_back(x);
        }
        // the other faces of B1 cells, and what lies across them
        for (int f : FA) faceLocal[(size_t)f] = -2;
        for (int x : B1) {
            codesOf(x, codes);
            for (int64_t code : codes) {
                const int f = faceOf(code);
                if (faceLocal[(size_t)f] != -1) continue;
                faceLocal[(size_t)f] = -3;
                FB.push_back(f);
            }
        }
        std::sort(FB.begin(), FB.end());
        for (int f : FB)
            for (int x : {(int)d->face_p[f], (int)d->face_n[f]}) {
                if (localOf[(size_t)x] != -1) continue;
                localOf[(size_t)x] = -2;
                C.push_back(x);
            }
        std::sort(C.begin(), C.end());
        for (int x : C) {
            localOf[(size_t)x] = (int)L.size();
            L.push_back(x);
        }
        td.nB1 = (int)B1.size();
        td.nL = (int)L.size();
        td.nV = td.nA + td.nB1;
        td.nFA = (int)FA.size();
        td.nLF = (int)(FA.size() + FB.size());
        std::vector<int> LF(FA);
        LF.insert(LF.end(), FB.begin(), FB.end());
        if (td.nL > maxLocal && td.nA > 1) {
            for (int x : L) localOf[(size_t)x] = -1;
            for (int f : LF) faceLocal[(size_t)f] = -1;
            return false;
        }
        for (int k = 0; k < td.nLF; ++k) faceLocal[(size_t)LF[(size_t)k]] = k;

        // ints: L | fP | fN | cfOff | cfList
        td.iOff = (int64_t)ts.ints.size();
        ts.ints.insert(ts.ints.end(), L.begin(), L.end());
        for (int f : LF) {
            const int lp = localOf[(size_t)d->face_p[f]];
            if (lp < 0 || lp >= td.nL) throw std::runtime_error("tiles: face owner outside its tile");
            ts.ints.push_back(lp);
        }
        for (int f : LF) {
            const int ln = localOf[(size_t)d->face_n[f]];
            if (ln < 0 || ln >= td.nL) throw std::runtime_error("tiles: face neighbour outside its tile");
            ts.ints.push_back(ln);
        }
        std::vector<int> cfList, cfNbr;
        ts.ints.push_back(0);
        for (int v = 0; v < td.nV; ++v) {
            codesOf(L[(size_t)v], codes);
            for (int64_t code : codes) {
                const int f = faceOf(code);
                const int lf = faceLocal[(size_t)f];
                if (lf < 0 || lf >= td.nLF || (v < td.nA && lf >= td.nFA))
                    throw std::runtime_error("tiles: cell face outside its tile");
                cfList.push_back(code >= 0 ? lf : ~lf);
                const int other = localOf[(size_t)(code >= 0 ? d->face_n[f] : d->face_p[f])];
                if (other < 0 || other >= td.nL) throw std::runtime_error("tiles: neighbour outside its tile");
                cfNbr.push_back(other);
            }
            ts.ints.push_back((int)cfList.size());
        }
        td.nE = (int)cfList.size();
        ts.ints.insert(ts.ints.end(), cfList.begin(), cfList.end());
        ts.ints.insert(ts.ints.end(), cfNbr.begin(), cfNbr.end());

        // floats (converted as the solver's device copies are: (float) of the FP64 value)
        td.fOff = (int64_t)ts.floats.size();
        auto pushRows = [&](const double* src, int rows) {
            for (int k = 0; k < rows; ++k)
                for (int f : LF) ts.floats.push_back((float)src[(size_t)k * (size_t)nf + (size_t)f]);
        };
        pushRows(d->S, D);
        pushRows(d->d, D);
        pushRows(d->w, 1);
        pushRows(d->K, D);
        for (int f : LF) ts.floats.push_back((float)(d->delta_mag[f] * d->dmag_inv[f]));
        pushRows(d->dmag_inv, 1);
        pushRows(d->dnorm, D);
        for (int v = 0; v < td.nV; ++v) ts.floats.push_back((float)d->vol_inv[L[(size_t)v]]);

        td.bOff = (int64_t)ts.bytes.size();
        for (int f : LF) ts.bytes.push_back(d->face_ghost[f]);

        ts.maxL = std::max(ts.maxL, td.nL);
        ts.maxLF = std::max(ts.maxLF, td.nLF);
        ts.localCells += td.nL;
        ts.fluxFaces += td.nFA;
        ts.tiles.push_back(td);
        for (int x : L) localOf[(size_t)x] = -1;
        for (int f : LF) faceLocal[(size_t)f] = -1;
        return true;
    };
    // tiles of tileCells cells, halved until their local cells fit
    std::vector<std::pair<int, int>> todo;
    for (int c0 = nc - ((nc - 1) % tileCells + 1); c0 >= 0; c0 -= tileCells) todo.push_back({c0, std::min(nc, c0 + tileCells)});
    while (!todo.empty()) {
        const auto r = todo.back();
        todo.pop_back();
        if (tryTile(r.first, r.second)) continue;
        const int mid = r.first + (r.second - r.first) / 2;
        todo.push_back({mid, r.second});
        todo.push_back({r.first, mid});
    }
    if (ts.ints.size() > 0x7fffffffu || ts.floats.size() > 0x7fffffffu)
        throw std::runtime_error("tiles: tile arrays too large for 32-bit offsets");
    return ts;
}

}  // namespace lfm
