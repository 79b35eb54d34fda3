#include "prepared.h"

#include <algorithm>

namespace fgb {

PreparedMesh prepare_mesh(TetMesh&& tm) {
    FGB_REQUIRE(tm.n_tets() > 0 && tm.n_nodes() > 0, "empty mesh");
    FGB_REQUIRE(tm.marker.size() == (size_t)tm.n_tets(), "one marker per tet is required");
    for (int32_t v : tm.tets) FGB_REQUIRE(v >= 0 && v < tm.n_nodes(), "tet references a node out of range");
    PreparedMesh pm;
    pm.tet = std::move(tm);
    pm.hex = tethex_split(pm.tet);
    pm.face_nbr = tet_face_neighbours(pm.tet);
    pm.tt = build_tet_tables(pm.tet, pm.hex, pm.face_nbr);
    pm.hex_coeffs = build_hex_coeffs(pm.hex);
    pm.vac = build_vacuum_map(pm.hex);
    build_vorocells(pm.hex, pm.voro_ptr, pm.voro_idx);
    pm.edgemax = tet_edgemax(pm.tet);
    pm.decay_factor = -1.0 / pm.edgemax;

    const int n_nodes = pm.hex.n_nodes();
    pm.n2c_ptr.assign(n_nodes + 1, 0);
    for (int32_t h : pm.vac.cells)
        for (int k = 0; k < 8; ++k) pm.n2c_ptr[pm.hex.hexs[8 * (size_t)h + k] + 1]++;
    for (int i = 0; i < n_nodes; ++i) pm.n2c_ptr[i + 1] += pm.n2c_ptr[i];
    pm.n2c_item.resize(pm.n2c_ptr[n_nodes]);
    {
        std::vector<int32_t> pos(pm.n2c_ptr.begin(), pm.n2c_ptr.end() - 1);
        for (int32_t h : pm.vac.cells)
            for (int k = 0; k < 8; ++k) pm.n2c_item[pos[pm.hex.hexs[8 * (size_t)h + k]]++] = 8 * h + k;
    }
    for (int c = 0; c < 3; ++c) {
        pm.bbox_min[c] = 1e300;
        pm.bbox_max[c] = -1e300;
    }
    for (int i = 0; i < pm.tet.n_nodes(); ++i)
        for (int c = 0; c < 3; ++c) {
            pm.bbox_min[c] = std::min(pm.bbox_min[c], pm.tet.xyz[3 * (size_t)i + c]);
            pm.bbox_max[c] = std::max(pm.bbox_max[c], pm.tet.xyz[3 * (size_t)i + c]);
        }
    attach_interface_surface(pm);
    return pm;
}

void attach_interface_surface(PreparedMesh& pm) {
    std::vector<int32_t> tris, tri2tet;
    interface_triangles(pm.tet.tets, pm.tet.marker, pm.face_nbr, pm.tet.xyz, tris, tri2tet);
    pm.surf = build_surface_tables(pm.tet.xyz.data(), pm.tet.n_nodes(), pm.tet.n_tets(), std::move(tris),
                                   std::move(tri2tet));
}

}  // namespace fgb
