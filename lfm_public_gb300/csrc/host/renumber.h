// Cell renumbering for locality of the device gathers: the solver order of
// the cells inside each submesh, so that the cells a kernel's neighbouring
// threads read lie close together in memory.
//
// The reference leaves cell order to a pre-processing step (its hpath
// renumbering utility, hpathRenumber/hpathRenumber.C:127-180, run on the
// polyMesh before the solver reads it); here the order is chosen when the
// solver description is built, and the polyMesh and the written fields keep
// their own numbering (the solver description maps each solver cell to its
// polyMesh label).
#pragma once

#include <cstdint>
#include <vector>

#include "meshReader.h"

namespace lfm {

enum Renumber { RENUMBER_NONE = 0, RENUMBER_RCM = 1, RENUMBER_HILBERT = 2, RENUMBER_HPATH = 3 };

// "none" / "rcm" / "hilbert" / "hpath" -> Renumber; -1 for anything else.
int renumberFromName(const std::string& name);

// Reorders `cells` (polyMesh labels of one submesh) in place.
//   RCM: reverse Cuthill-McKee over the face adjacency among these cells,
//        each connected component started from a pseudo-peripheral cell
//        (George-Liu), neighbours visited in increasing degree; minimises
//        the bandwidth max |i - j| over faces.
//   Hilbert: cells sorted along a Hilbert curve through their centres (2D
//        on a 2^31 grid of the bounding box, 3D on 2^21 per axis).
void renumberCells(IMeshReader& r, std::vector<int>& cells, int method, int dim);

// The reference's Hamiltonian-path cell order over the whole mesh (its hpath
// renumbering method, hpathRenumber/hpathRenumber.C:127-180; hpath.cpp):
// order[i] = the polyMesh label of the i-th cell, boundary cells first. The
// solver order of a submesh is its cells sorted by their position here.
// Empty when the walk does not give a permutation of the cells.
std::vector<int> hpathCellOrder(IMeshReader& r);

// Bandwidth of an order: max |pos(a) - pos(b)| over faces between cells of
// the list (for tests and diagnostics).
int64_t cellBandwidth(IMeshReader& r, const std::vector<int>& cells);

}  // namespace lfm
