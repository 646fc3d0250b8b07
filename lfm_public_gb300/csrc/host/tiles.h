// Host builder of the tiles of the fused FP32-bulk stage kernel
// (csrc/cuda/tile_desc.h describes a tile).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../cuda/tile_desc.h"
#include "lfm_gpu.h"

namespace lfm {

struct TileSet {
    int dim = 2;
    int tileCells = 0;
    std::vector<TileDesc> tiles;
    std::vector<int> ints;
    std::vector<float> floats;
    std::vector<uint8_t> bytes;
    int maxL = 0, maxLF = 0;   // largest local cell and face counts
    int64_t localCells = 0;    // sum of nL (loads per stage, halos included)
    int64_t fluxFaces = 0;     // sum of nFA (faces whose rhs is computed)
};

// Tiles of up to tileCells consecutive cells over a description without
// processor halos, in cell order; a run whose local cells (with its two
// rings) exceed maxLocal is halved until they fit. Throws
// std::runtime_error when the description has halos or an index is
// inconsistent. Every local index of the result is checked against its
// tile's counts.
TileSet buildTiles(const lfm_solver_desc* d, int tileCells, int maxLocal);

}  // namespace lfm
