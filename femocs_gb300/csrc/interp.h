// Device-resident interpolator of one mesh: nodal solution (E, charge density, phi per
// hex-mesh node), nodal-field recovery and smoothing, point location and interpolation.
#pragma once

#include <cuda_runtime.h>

#include "device.h"
#include "prepared.h"

namespace fgb {

// Uniform grid over the mesh box: a seed tet per grid cell (start of the location walk) and
// the tets bucketed by centroid (exact nearest-centroid fallback search).
struct SeedGrid {
    int dim[3] = {1, 1, 1};
    double origin[3] = {0, 0, 0};
    double step[3] = {1, 1, 1};
    std::vector<int32_t> seed;       // per grid cell
    std::vector<int32_t> ptr, tets;  // tets bucketed by centroid, ascending within a bucket
    std::vector<double> cxyz;        // centroids in bucket order
};
SeedGrid build_seed_grid(const PreparedMesh& pm);

struct LocateStats {
    int n_points = 0;
    int n_walk_failed = 0;   // located by the exhaustive scan
    int n_fallback = 0;      // no searchable tet contains the point (nearest-centroid result)
    int n_dependent = 0;     // points whose result depends on the previous point's cell
    int longest_run = 0;
};

class DeviceMesh {
public:
    DeviceMesh(const PreparedMesh& pm, cudaStream_t stream);

    // nodal solution from the FEM solution (phi by dof); recovers E (src/Interpolator.cpp:172-190)
    void extract_solution(const double* d_phi_dof, const int32_t* d_dof2node, int n_dofs, bool smoothen,
                          const double* d_charge_dof = nullptr);
    // overwrite the nodal solution (5 doubles per node) from the host
    void set_solution(const double* h_sol5);
    void get_solution(double* h_sol5);
    // max |E| over the nodes (FieldReader::max_field, src/SolutionReader.cpp:558-566)
    double max_field_norm();
    // Locate and interpolate n points (device pointers, xyz interleaved); rank 1 lin-tet,
    // 2 quad-tet, 3 lin-hex; cells and out (5 per point) on the device.
    void locate_interpolate(int n, const double* d_pts, int rank, int32_t* d_cells, double* d_out,
                            LocateStats* stats = nullptr);
    // Same result as locate_interpolate, for callers that cannot allocate device memory: no
    // cudaMalloc/cudaFree, the per-point scratch is a file-scope device array (at most
    // 262144 points per call, shared by all calls; overlapping calls race). Asynchronous on
    // stream(). The first call on a device looks up the array's device address.
    void locate_interpolate_noalloc(int n, const double* d_pts, int rank, int32_t* d_cells, double* d_out);
    // Space charge of n particles in vacuum hexes d_hex (femocs hex ids, < 0: skipped) added to
    // a per-DoF rhs (order 1: through node -> dof; order 2: through hex -> vacuum cell and its
    // 27 cell DoFs); n_skipped (may be null) receives the particles outside the vacuum hexes
    void space_charge(int n, const double* d_pts, const int32_t* d_hex, int order, const int32_t* d_node2dof,
                      const int32_t* d_hex2cell, const int32_t* d_cell_dofs, double charge_factor, double* d_rhs,
                      int* n_skipped);
    // Surface (2-D) location + interpolation on the mesh's surface triangles: the chained
    // triangle search of InterpolatorCells<3>::locate_cell, then the tet reached through the
    // triangle's two tets (LinearTriangles / QuadraticTriangles::interp_solution,
    // src/InterpolatorCells.cpp:1639-1686, 1834-1856), rank 1 linear or 2 quadratic in that tet;
    // rank 3 (LinearQuadrangles, :1922-1993) trilinear in the hex of the point's quadrangle.
    // d_cells: triangle (ranks 1, 2) or quadrangle (rank 3) per point (negative = nearest-
    // centroid fallback); d_out: 5 per point.
    void surface_interpolate(int n, const double* d_pts, int rank, int32_t* d_cells, double* d_out);
    int n_surface_tris() const { return n_stris_; }
    // Interpolate with cells already known (SolutionReader::calc_interpolation with mapped atoms)
    void interpolate_known(int n, const double* d_pts, int rank, const int32_t* d_cells, double* d_out);

    int n_nodes() const { return n_nodes_; }
    int n_tets() const { return n_tets_; }
    double* d_sol() { return sol_.get(); }
    cudaStream_t stream() const { return stream_; }
    const double* d_node_xyz() const { return xyz_.get(); }
    const int32_t* d_hexs() const { return hexs_.get(); }
    const double* d_hex_coeffs() const { return hexf_.get(); }
    // keep the geometry-only factors of the nodal field and the smoothing on the device after
    // the first extraction (112 B per node-hex incidence, 8 B per smoothing neighbour): later
    // extractions only gather and sum, with bit-identical results. On by default.
    void set_geometry_cache(bool on) {
        geo_cache_ = on;
        if (!on) { nodal_ids_.release(); nodal_coef_.release(); smooth_w_.release(); smooth_f_.release(); }
    }

private:
    void ensure_scratch(int n);
    void set_surface(const PreparedMesh& pm);
    cudaStream_t stream_;
    int n_nodes_, n_tets_, n_tetnodes_;
    double decay_;
    double bb_lo_[3], bb_hi_[3];
    SeedGrid grid_;
    DBuf<int32_t> tet_nodes_, face_nbr_, nbr_ptr_, nbr_idx_, quad_;
    DBuf<int8_t> search_;
    DBuf<double> det_, centroid_;
    DBuf<int32_t> hexs_, n2c_ptr_, n2c_item_, voro_ptr_, voro_idx_;
    DBuf<double> hexf_, xyz_;
    DBuf<int32_t> seed_, gptr_, gtets_;
    DBuf<double> gcxyz_;
    DBuf<double> sol_;
    bool geo_cache_ = true;
    DBuf<int32_t> nodal_ids_;
    DBuf<double> nodal_coef_, smooth_w_, smooth_f_;
    // per-point scratch
    DBuf<int32_t> v_, nin_, f_, res_, dep_, counters_;
    int scratch_n_ = 0;
    // surface triangles: tables, candidate grid (triangles whose acceptance region meets a
    // cell), centroid buckets for the nearest-centroid fallback, per-point scratch
    int n_stris_ = 0;
    DBuf<int32_t> stris_, stri2tet_, snbr_ptr_, snbr_idx_, scand_ptr_, scand_idx_, sgptr_, sgtris_;
    DBuf<double> sgeo_, sgcxyz_;
    int scand_dim_[3] = {1, 1, 1}, sg_dim_[3] = {1, 1, 1};
    double scand_org_[3] = {0, 0, 0}, scand_step_[3] = {1, 1, 1}, scand_lo_[3] = {0, 0, 0}, scand_hi_[3] = {0, 0, 0};
    double sg_org_[3] = {0, 0, 0}, sg_step_[3] = {1, 1, 1};
    DBuf<int32_t> s_tv_, s_nin_, s_tf_, s_res_, s_dep_, s_counters_;
    int s_scratch_n_ = 0;
};

}  // namespace fgb
