// Cell blocks of a Q2 structure: the element-by-element form of the level-0 operator with the
// per-cell products summed on chip.
//
// The cells are ordered by their interior DoF (the DoF numbering is a Morton order of the DoF
// positions, so this is a Morton order of the cells) and cut into blocks of consecutive cells.
// One CTA applies one block: it gathers x for the block's DoFs into shared memory, forms
// K_e x_e for each cell and sums the products of every DoF in a fixed order. A DoF whose cells
// all lie in the block (complete) is finished there; the others leave one partial sum per
// block in a slot, summed afterwards in ascending block order. The result is deterministic.
#pragma once

#include <cstdint>
#include <vector>

#include "fem.h"

namespace fgb {

struct CellBlocks {
    int n_cells = 0, n_blocks = 0, n_dofs = 0;
    int max_cells = 0, max_dofs = 0;      // largest block (cells, local DoFs)
    std::vector<int32_t> perm;            // position -> cell (blocks are position ranges)
    std::vector<int32_t> cell_start;      // n_blocks + 1, positions
    std::vector<int32_t> dof_start;       // n_blocks + 1, local DoF entries
    std::vector<int32_t> dof_list;        // local DoF -> global DoF (ascending within a block)
    std::vector<uint16_t> item_end;       // local DoF -> end of its items within the block's items
    std::vector<int32_t> slot;            // local DoF -> partial-sum slot, -1 when complete
    std::vector<uint16_t> loc;            // 27 per position: block-local index of the lattice DoF
    std::vector<uint16_t> items;          // 28 per position (block region from 28 x its first
                                          // position, 8-byte aligned): 27 * (position - block
                                          // start) + lattice index, grouped by local DoF
    int n_slots = 0;
    std::vector<int32_t> bnd_dofs;        // DoFs with slots, ascending
    std::vector<int32_t> bnd_ptr;         // their slots: bnd_ptr[j] .. bnd_ptr[j+1]-1, ascending block
    int64_t local_entries() const { return (int64_t)dof_list.size(); }
};

// cells_per_block consecutive cells per block, halved while a block holds more than max_dofs
// DoFs (at most 4096); 27 * cells_per_block must fit 16 bits
CellBlocks build_cell_blocks(const FemStructure& fs, int cells_per_block = 256, int max_dofs = 4096);

// every invariant the kernels rely on (throws fgb::Error naming the first violation): the
// permutation, the block ranges and limits, local DoFs ascending, loc and items mapping back
// to the cells' DoFs, each DoF complete in one block or holding one slot per block in block
// order; returns a 64-bit digest of all arrays
uint64_t validate_cell_blocks(const FemStructure& fs, const CellBlocks& cb, int cells_per_block, int max_dofs);

}  // namespace fgb
