// Q1 Laplace/Poisson system on the vacuum hexes: host-built structure (DoF numbering,
// sparsity, boundary classification) and the device-resident system (matrix, right-hand
// side, solution) with its assembly and solve entry points.
#pragma once

#include <memory>

#include "prepared.h"

namespace fgb {

// Structure that depends only on the mesh (built once on the host).
struct FemStructure {
    int n_dofs = 0, n_cells = 0;
    std::vector<int32_t> dof2node;    // n_dofs -> hex-mesh node
    std::vector<int32_t> node2dof;    // n_nodes -> dof or -1
    std::vector<int32_t> cell_dofs;   // 8 per vacuum cell, femocs local order
    std::vector<int64_t> rowptr;      // CSR, columns ascending, diagonal included
    std::vector<int32_t> col;
    std::vector<int32_t> r2c_ptr, r2c_item;  // row -> 8*cell+local, ascending cell
    std::vector<int32_t> top_faces;   // 4 dofs per top (Neumann/anode) face, cyclic order
    std::vector<int32_t> r2f_ptr, r2f_item;  // row -> 4*face+local
    std::vector<int8_t> bc_kind;      // 0 free, 1 copper (phi=0), 2 top (phi=V0 if anode Dirichlet)
    // SELL-32 layout of the same matrix
    std::vector<int64_t> slice_ptr;   // n_slices+1, element offsets
    std::vector<int32_t> slice_len;   // max row length per slice
    std::vector<int64_t> csr2sell;    // CSR position -> SELL position
    std::vector<int32_t> sell_col;    // padded columns (padding points at the row itself)
    std::vector<int32_t> row_len;     // per row
    int n_top_faces() const { return (int)(top_faces.size() / 4); }
    int64_t nnz() const { return rowptr.empty() ? 0 : rowptr.back(); }
};

FemStructure build_fem_structure(const PreparedMesh& pm);

}  // namespace fgb
