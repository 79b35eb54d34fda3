// Surface triangles of the vacuum/metal interface and the tables of surface (2-D) location:
// the GPU counterpart of the reference's TetgenFaces appendices and LinearTriangles
// precompute (src/TetgenCells.cpp:387-412, src/InterpolatorCells.cpp:1585-1637).
#pragma once

#include "common.h"

namespace fgb {

// per triangle: vert0 (3), edge1/D (3), edge2 (3), pvec/D (3), unit normal (3), max distance
// |edge2| (1), centroid (3)
constexpr int kTriGeoStride = 19;

struct SurfaceTables {
    std::vector<int32_t> tris;     // 3 tet-mesh node ids per triangle
    std::vector<int32_t> tri2tet;  // the two tets of each triangle; the first is tried first
    std::vector<double> geo;       // kTriGeoStride per triangle
    // candidates after a failed guess: for each node of the triangle (in triangle order) the
    // other triangles holding that node, ascending, repeats kept (LinearTriangles::precompute)
    std::vector<int32_t> nbr_ptr, nbr_idx;
    int n_tris() const { return (int)(tris.size() / 3); }
};

// The vacuum/metal interface faces of a tet mesh: for every vacuum tet (ascending) its faces
// opposite vertex 0..3 whose neighbour is a non-vacuum tet. Vertices in ascending local order,
// the last two swapped when needed so that the normal (e1 x e2) points into the vacuum tet;
// tri2tet = {vacuum tet, metal tet}.
void interface_triangles(const std::vector<int32_t>& tets, const std::vector<int32_t>& marker,
                         const std::vector<int32_t>& face_nbr, const std::vector<double>& xyz,
                         std::vector<int32_t>& tris, std::vector<int32_t>& tri2tet);

// Location tables of the given triangles over node coordinates xyz (3 per node), in the
// reference's operation order. Node ids must be < n_nodes; tets in tri2tet < n_tets.
SurfaceTables build_surface_tables(const double* xyz, int n_nodes, int n_tets, std::vector<int32_t> tris,
                                   std::vector<int32_t> tri2tet);

}  // namespace fgb
