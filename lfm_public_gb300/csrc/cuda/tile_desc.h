// Tiles of the fused FP32-bulk stage kernel (plain C++: shared by the host
// builder, csrc/host/tiles.cpp, and the device kernel, tile_kernels.cu).
//
// A tile is a run of consecutive solver cells (the A cells, whose state the
// tile's block updates) together with everything one RK stage reads around
// them, numbered locally:
//   local cells  L = A | B1 | B2 | C
//     B1: the cells (not ghosts) across the faces of A, B2: the ghosts across
//     them, C: the cells and ghosts across the faces of B1 that are not in
//     A or B;
//   local faces  LF = FA | FB
//     FA: every face of an A cell (its rhs is computed), FB: the other faces
//     of the B1 cells (read by their viscous terms and gradients).
// The viscous terms and gradients are computed for V = A | B1, fluxes for
// FA, and the update for A, all from shared memory. A tile's arrays are
// copies of the solver's (same values, same per-cell face order), so the
// fused kernel gives the bits of the separate kernels.
#pragma once

#include <cstdint>

namespace lfm {

struct TileDesc {
    int c0;          // first A cell (solver index); the A cells are c0 .. c0 + nA - 1
    int nA, nB1, nL; // A cells, non-ghost cells across them, all local cells
    int nV;          // nA + nB1
    int nFA, nLF;    // faces of A cells, all local faces
    int nE;          // entries of the local cell -> face lists of the V cells
    int64_t iOff;    // ints:  L[nL] fP[nLF] fN[nLF] cfOff[nV + 1] cfList[nE] cfNbr[nE]
    int64_t fOff;    // floats: S[D][nLF] d[D][nLF] w[nLF] K[D][nLF] lapc[nLF] dinv[nLF]
                     //         dnorm[D][nLF] volInv32[nV]
    int64_t bOff;    // bytes: fGhost[nLF]
};

}  // namespace lfm
