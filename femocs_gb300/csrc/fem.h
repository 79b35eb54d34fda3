// Q1 Laplace/Poisson system on the vacuum hexes: host-built structure (DoF numbering,
// sparsity, boundary classification) and the device-resident system (matrix, right-hand
// side, solution) with its assembly and solve entry points.
#pragma once

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <memory>

#include "prepared.h"

namespace fgb {

// Structure that depends only on the mesh (built once on the host).
//
// order 1: Q1, one DoF per vacuum vertex, cells list 8 DoFs in femocs local order, faces 4.
// order 2: Q2 (27-node hexahedra on the trilinear map): cells list 27 DoFs in lattice order
// L = a + 3b + 9c, (a,b,c) in {0,1,2}^3 along the reference axes (vertex k of the femocs
// order sits at a = 1 + hx[k], b = 1 + hy[k], c = 1 + hz[k]); one DoF per vacuum vertex, hex
// edge, hex face and hex interior; top faces list 9 DoFs (u + 3v on the face lattice). Only
// the SELL-32 form of the sparsity exists for Q2 (no CSR copy).
struct FemStructure {
    int order = 1;                    // 1 or 2
    int npc = 8, nfc = 4;             // DoFs per cell and per boundary face
    int n_dofs = 0, n_cells = 0;
    int64_t n_entries = 0;            // nonzeros (sum of row lengths)
    std::vector<int32_t> dof2node;    // n_dofs -> hex-mesh node (-1 for Q2 edge/face/interior DoFs)
    std::vector<int32_t> node2dof;    // n_nodes -> dof or -1
    std::vector<int32_t> cell_dofs;   // npc per vacuum cell
    std::vector<int64_t> rowptr;      // CSR, columns ascending, diagonal included
    std::vector<int32_t> col;
    std::vector<int32_t> r2c_ptr, r2c_item;  // row -> npc*cell+local, ascending cell
    int region = 0;                   // kRegionVacuum or kRegionBulk
    std::vector<int32_t> top_faces;   // nfc dofs per top (Neumann/anode) face (Q1: cyclic order)
    std::vector<int32_t> top_face_cells;  // Q1: cell of each Neumann face
    std::vector<int8_t> top_face_local;   // Q1: its local face (femocs face numbering)
    std::vector<int32_t> r2f_ptr, r2f_item;  // row -> nfc*face+local
    std::vector<int8_t> bc_kind;      // 0 free, 1 copper (phi=0), 2 top (phi=V0 if anode Dirichlet)
    // SELL-32 layout of the same matrix
    std::vector<int64_t> slice_ptr;   // n_slices+1, element offsets
    std::vector<int32_t> slice_len;   // max row length per slice
    std::vector<int64_t> csr2sell;    // CSR position -> SELL position
    std::vector<int32_t> sell_col;    // padded columns (padding points at the row itself)
    std::vector<int32_t> row_len;     // per row
    std::vector<double> dof_xyz;      // Q2: position of every DoF (3 per DoF)
    std::vector<int32_t> dof_cell;    // Q2: one vacuum cell holding the DoF
    std::vector<int8_t> dof_local;    // Q2: its lattice index in that cell
    int n_top_faces() const { return (int)(top_faces.size() / nfc); }
    int64_t nnz() const { return !rowptr.empty() ? rowptr.back() : n_entries; }
};

// Region of the hex mesh a structure is built on: the vacuum (field solve) or the bulk
// (current and heat, src/CurrentHeatSolver.cpp)
enum : int { kRegionVacuum = 0, kRegionBulk = 1 };
struct RegionCells {
    std::vector<int32_t> cells;        // hex ids of the region, ascending
    std::vector<int32_t> node2vertex;  // hex-mesh node -> compact vertex (ascending node order) or -1
    std::vector<int32_t> vertex2node;
};
RegionCells region_cells(const PreparedMesh& pm, int region);

FemStructure build_fem_structure(const PreparedMesh& pm, int region = kRegionVacuum);

// FGB_SETUP_VERBOSE=1 prints the phases of the structure builders to stderr
class SetupPhases {
public:
    explicit SetupPhases(const char* who) : who_(who), on_(std::getenv("FGB_SETUP_VERBOSE") != nullptr),
                                            t_(std::chrono::steady_clock::now()) {}
    void operator()(const char* what) {
        const auto t = std::chrono::steady_clock::now();
        if (on_)
            std::fprintf(stderr, "%s: %-32s %9.1f ms\n", who_, what,
                         std::chrono::duration<double, std::milli>(t - t_).count());
        t_ = t;
    }

private:
    const char* who_;
    bool on_;
    std::chrono::steady_clock::time_point t_;
};
// Q2 structure of the same vacuum hexahedra (see the order-2 notes above)
// sell_columns = false leaves sell_col empty (slice pointers and lengths are set): the device
// fills it (q2_sell_columns, fem_q2.cu), the host copy would only be uploaded
FemStructure build_q2_structure(const PreparedMesh& pm, bool sell_columns = true);
// lattice coordinates (a,b,c) of local Q2 node L, and the femocs vertex of a lattice corner
inline void q2_lattice(int L, int& a, int& b, int& c) { a = L % 3; b = (L / 3) % 3; c = L / 9; }
int q2_corner_vertex(int a, int b, int c);  // a,b,c in {0,2} -> femocs local vertex 0..7
// femocs local vertices spanning the entity of lattice node L (1 vertex, 2 edge ends, 4 face
// corners or 8 cell corners); returns the count
int q2_entity_corners(int L, int out[8]);

}  // namespace fgb
