// A tetrahedral mesh together with every host-derived table the device path uploads.
#pragma once

#include "mesh.h"
#include "surface.h"

namespace fgb {

struct PreparedMesh {
    TetMesh tet;
    HexMesh hex;
    std::vector<int32_t> face_nbr;    // 4 per tet
    TetTables tt;
    std::vector<double> hex_coeffs;   // 24 per hex
    VacuumMap vac;
    std::vector<int32_t> voro_ptr, voro_idx;
    // node -> vacuum hexes (ascending) with the node's local index, for nodal-field recovery
    std::vector<int32_t> n2c_ptr, n2c_item;  // item = 8*hex + local
    double edgemax = 0.0;
    double decay_factor = 0.0;
    double bbox_min[3] = {0, 0, 0}, bbox_max[3] = {0, 0, 0};
    // surface triangles for 2-D location (default: the vacuum/metal interface faces)
    SurfaceTables surf;
};

// the default surface of a prepared mesh: its vacuum/metal interface triangles
void attach_interface_surface(PreparedMesh& pm);

PreparedMesh prepare_mesh(TetMesh&& tm);

}  // namespace fgb
