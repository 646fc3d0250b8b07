// Cell renumbering (renumber.h): reverse Cuthill-McKee and Hilbert order.
#include "renumber.h"

#include <algorithm>
#include <cstdlib>
#include <numeric>
#include <queue>
#include <string>

namespace lfm {

int renumberFromName(const std::string& name) {
    if (name == "none" || name.empty()) return RENUMBER_NONE;
    if (name == "rcm" || name == "RCM") return RENUMBER_RCM;
    if (name == "hilbert") return RENUMBER_HILBERT;
    if (name == "hpath") return RENUMBER_HPATH;
    return -1;
}

namespace {

// Adjacency among the listed cells, as local indices (CSR).
struct Graph {
    std::vector<int64_t> off;
    std::vector<int> adj;
    int n = 0;
    int degree(int v) const { return (int)(off[(size_t)v + 1] - off[(size_t)v]); }
};

Graph buildGraph(IMeshReader& r, const std::vector<int>& cells) {
    Graph g;
    g.n = (int)cells.size();
    std::vector<int> local((size_t)r.getCellCount(), -1);
    for (int i = 0; i < g.n; ++i) local[(size_t)cells[(size_t)i]] = i;
    g.off.assign((size_t)g.n + 1, 0);
    std::vector<std::vector<int>> nb((size_t)g.n);
    for (int i = 0; i < g.n; ++i) {
        const int cell = cells[(size_t)i];
        const int nf = r.getCellValidFaceCount(cell);
        for (int k = 0; k < nf; ++k) {
            const int f = r.getCellValidFaceIndex(cell, k);
            const int own = r.getFaceOwner(f), nei = r.getFaceNeighbour(f);
            const int other = own == cell ? nei : own;
            if (other < 0 || other == cell) continue;
            const int j = local[(size_t)other];
            if (j >= 0) nb[(size_t)i].push_back(j);
        }
        std::sort(nb[(size_t)i].begin(), nb[(size_t)i].end());
        nb[(size_t)i].erase(std::unique(nb[(size_t)i].begin(), nb[(size_t)i].end()), nb[(size_t)i].end());
        g.off[(size_t)i + 1] = g.off[(size_t)i] + (int64_t)nb[(size_t)i].size();
    }
    g.adj.reserve((size_t)g.off.back());
    for (auto& v : nb) g.adj.insert(g.adj.end(), v.begin(), v.end());
    return g;
}

// Breadth-first levels from `root` inside the unvisited component; returns
// the last level.
std::vector<int> lastLevel(const Graph& g, int root, std::vector<int>& level, const std::vector<char>& done,
                           int* depth) {
    std::vector<int> cur{root}, next, last;
    level[(size_t)root] = 0;
    std::vector<int> touched{root};
    int d = 0;
    while (!cur.empty()) {
        last = cur;
        next.clear();
        for (int v : cur)
            for (int64_t e = g.off[(size_t)v]; e < g.off[(size_t)v + 1]; ++e) {
                const int w = g.adj[(size_t)e];
                if (done[(size_t)w] || level[(size_t)w] >= 0) continue;
                level[(size_t)w] = d + 1;
                touched.push_back(w);
                next.push_back(w);
            }
        cur.swap(next);
        ++d;
    }
    for (int v : touched) level[(size_t)v] = -1;
    *depth = d;
    return last;
}

std::vector<int> rcmOrder(const Graph& g) {
    std::vector<char> done((size_t)g.n, 0);
    std::vector<int> level((size_t)g.n, -1);
    std::vector<int> order;
    order.reserve((size_t)g.n);
    // components in order of their lowest-numbered cell
    for (int seed = 0; seed < g.n; ++seed) {
        if (done[(size_t)seed]) continue;
        // pseudo-peripheral start (George-Liu): from the seed, move to a
        // minimum-degree cell of the last BFS level while the depth grows
        int root = seed, depth = 0;
        std::vector<int> last = lastLevel(g, root, level, done, &depth);
        for (int it = 0; it < 8; ++it) {
            int cand = last[0];
            for (int v : last)
                if (g.degree(v) < g.degree(cand) || (g.degree(v) == g.degree(cand) && v < cand)) cand = v;
            int d2 = 0;
            std::vector<int> l2 = lastLevel(g, cand, level, done, &d2);
            if (d2 <= depth) break;
            root = cand;
            depth = d2;
            last.swap(l2);
        }
        // Cuthill-McKee from the root: neighbours in increasing degree
        const size_t start = order.size();
        order.push_back(root);
        done[(size_t)root] = 1;
        std::vector<int> nbrs;
        for (size_t h = start; h < order.size(); ++h) {
            const int v = order[h];
            nbrs.clear();
            for (int64_t e = g.off[(size_t)v]; e < g.off[(size_t)v + 1]; ++e) {
                const int w = g.adj[(size_t)e];
                if (!done[(size_t)w]) nbrs.push_back(w);
            }
            std::sort(nbrs.begin(), nbrs.end(), [&](int a, int b) {
                return g.degree(a) != g.degree(b) ? g.degree(a) < g.degree(b) : a < b;
            });
            for (int w : nbrs) {
                done[(size_t)w] = 1;
                order.push_back(w);
            }
        }
    }
    std::reverse(order.begin(), order.end());
    return order;
}

// Hilbert index of (x, y) on a 2^bits grid: the rotate-and-flip construction
// of the curve, quadrant by quadrant from the most significant bit.
uint64_t hilbert2(uint32_t x, uint32_t y, int bits) {
    const uint32_t n = 1u << bits;
    uint64_t d = 0;
    for (uint32_t s = n >> 1; s > 0; s >>= 1) {
        const uint32_t rx = (x & s) ? 1u : 0u, ry = (y & s) ? 1u : 0u;
        d += (uint64_t)s * s * ((3u * rx) ^ ry);
        if (ry == 0) {
            if (rx == 1) {
                x = n - 1 - x;
                y = n - 1 - y;
            }
            std::swap(x, y);
        }
    }
    return d;
}

// Hilbert index of (x, y, z) on a 2^bits grid: Skilling's transform of the
// coordinates to the transposed Hilbert index ("Programming the Hilbert
// curve", AIP Conf. Proc. 707, 2004), then its bits interleaved.
uint64_t hilbert3(uint32_t x, uint32_t y, uint32_t z, int bits) {
    uint32_t X[3] = {x, y, z};
    const uint32_t M = 1u << (bits - 1);
    for (uint32_t Q = M; Q > 1; Q >>= 1) {   // inverse undo
        const uint32_t P = Q - 1;
        for (int i = 0; i < 3; ++i) {
            if (X[i] & Q) {
                X[0] ^= P;
            } else {
                const uint32_t t = (X[0] ^ X[i]) & P;
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    for (int i = 1; i < 3; ++i) X[i] ^= X[i - 1];   // Gray encode
    uint32_t t = 0;
    for (uint32_t Q = M; Q > 1; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1;
    for (int i = 0; i < 3; ++i) X[i] ^= t;
    uint64_t d = 0;
    for (int b = bits - 1; b >= 0; --b)
        for (int i = 0; i < 3; ++i) d = (d << 1) | ((X[i] >> b) & 1u);
    return d;
}

std::vector<int> hilbertOrder(IMeshReader& r, const std::vector<int>& cells, int dim) {
    const size_t n = cells.size();
    std::vector<double> xc(3 * n);
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (size_t i = 0; i < n; ++i) {
        r.getCellCenter(cells[i], &xc[3 * i]);
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], xc[3 * i + (size_t)k]);
            hi[k] = std::max(hi[k], xc[3 * i + (size_t)k]);
        }
    }
    const int bits = dim == 2 ? 31 : 21;   // 62- and 63-bit keys: fine enough for stretched meshes
    const double top = (double)((1ull << bits) - 1);
    std::vector<uint64_t> key(n);
    for (size_t i = 0; i < n; ++i) {
        uint32_t u[3];
        for (int k = 0; k < 3; ++k) {
            const double span = hi[k] - lo[k];
            u[k] = span > 0 ? (uint32_t)((xc[3 * i + (size_t)k] - lo[k]) / span * top) : 0u;
        }
        key[i] = dim == 2 ? hilbert2(u[0], u[1], bits) : hilbert3(u[0], u[1], u[2], bits);
    }
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[(size_t)a] < key[(size_t)b]; });
    return order;
}

}  // namespace

void renumberCells(IMeshReader& r, std::vector<int>& cells, int method, int dim) {
    if (method == RENUMBER_NONE || cells.size() < 2) return;
    std::vector<int> order;
    if (method == RENUMBER_RCM)
        order = rcmOrder(buildGraph(r, cells));
    else
        order = hilbertOrder(r, cells, dim);
    std::vector<int> out(cells.size());
    for (size_t i = 0; i < order.size(); ++i) out[i] = cells[(size_t)order[i]];
    cells.swap(out);
}

int64_t cellBandwidth(IMeshReader& r, const std::vector<int>& cells) {
    const Graph g = buildGraph(r, cells);
    int64_t bw = 0;
    for (int v = 0; v < g.n; ++v)
        for (int64_t e = g.off[(size_t)v]; e < g.off[(size_t)v + 1]; ++e)
            bw = std::max<int64_t>(bw, std::llabs((long long)g.adj[(size_t)e] - v));
    return bw;
}

}  // namespace lfm
