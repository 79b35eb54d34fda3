// Host-side mesh preparation: everything the device kernels need that is derived once per
// mesh (tet -> hex split, neighbour lists, barycentric determinant tables, trilinear map
// coefficients, vacuum-node compaction, smoothing stencils).
//
// The layouts mirror what the reference keeps in TetgenMesh / InterpolatorCells so that
// cell indices and interpolated values can be compared one to one:
//   * nodes: tet vertices first, then one node per edge, per face, per tet
//     (src/Tethex.cpp:965-1035), markers 1/2/3/4 (include/Globals.h:53-56);
//   * hex 4t+k is the corner of tet t around its vertex k (src/Tethex.cpp:1037-1102);
//   * hex markers +-(1+tet vertex) for vacuum/bulk (src/TetgenMesh.cpp:353-385).
#pragma once

#include "common.h"

namespace fgb {

struct TetMesh {
    std::vector<double> xyz;        // 3 * n_nodes
    std::vector<int32_t> tets;      // 4 * n_tets
    std::vector<int32_t> marker;    // n_tets, kVacuum or other
    int n_nodes() const { return (int)(xyz.size() / 3); }
    int n_tets() const { return (int)(tets.size() / 4); }
};

// Read a Gmsh 2.2 ASCII tetrahedral mesh; the first element tag is the region marker.
TetMesh read_gmsh(const std::string& path);

struct HexMesh {
    int n_tetnodes = 0, n_edges = 0, n_faces = 0, n_tets = 0;
    std::vector<double> xyz;          // 3 * n_nodes
    std::vector<int8_t> node_marker;  // kTetNode .. kTetCentroid
    std::vector<int32_t> hexs;        // 8 * n_hexs (= 4 * n_tets)
    std::vector<int32_t> hex_marker;  // +(1+v) vacuum, -(1+v) bulk
    // tet vertices a node was made from (itself; edge ends; face corners; tet corners),
    // 4 slots per node, unused slots -1 -- the linear interpolation from the tet mesh
    std::vector<int32_t> parents;
    int n_nodes() const { return (int)(xyz.size() / 3); }
    int n_hexs() const { return (int)(hexs.size() / 8); }
};

// Split every tet into four hexahedra (one per tet vertex).
HexMesh tethex_split(const TetMesh& tm);

// Face neighbours, entry 4t+j = tet across the face opposite to vertex j, or -1.
std::vector<int32_t> tet_face_neighbours(const TetMesh& tm);

// Maximum tet edge length (sqrt of the max squared edge), over all tets.
double tet_edgemax(const TetMesh& tm);

// Per-tet data for point location and barycentric interpolation.
//   det: 17 doubles per tet  = 1/D, then the four minor vectors (4 doubles each)
//   centroid: 3 doubles per tet
//   search: 1 if the tet belongs to the searched (vacuum) region, else 0
//   nbr_ptr/nbr_idx: candidate list used after a failed guess: face neighbours, then the
//                    tets sharing a vertex, duplicates removed (first occurrence kept)
struct TetTables {
    std::vector<double> det;
    std::vector<double> centroid;
    std::vector<int8_t> search;
    std::vector<int32_t> nbr_ptr, nbr_idx;
    std::vector<int32_t> quad_nodes;  // 10 * n_tets, quadratic-tet node list
};
constexpr int kTetDetStride = 17;
TetTables build_tet_tables(const TetMesh& tm, const HexMesh& hm, const std::vector<int32_t>& face_nbr);

// Trilinear map coefficients f0..f7 (3 doubles each) per hex, for the Newton projection
// to natural coordinates.
std::vector<double> build_hex_coeffs(const HexMesh& hm);

// Vacuum bookkeeping: femocs2deal[node] = compact vacuum-vertex id or -1, plus the list
// of vacuum hexes in ascending order.
struct VacuumMap {
    std::vector<int32_t> node2vertex;  // n_nodes
    std::vector<int32_t> vertex2node;  // n_vertices
    std::vector<int32_t> cells;        // hex ids with marker > 0, ascending
};
VacuumMap build_vacuum_map(const HexMesh& hm);

// Pseudo Voronoi stencils of the tet vertices (vacuum hexes), for nodal-field smoothing.
void build_vorocells(const HexMesh& hm, std::vector<int32_t>& ptr, std::vector<int32_t>& idx);

}  // namespace fgb
