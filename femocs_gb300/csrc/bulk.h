// Current and heat on the bulk (metal) hexahedra: the GPU counterpart of the reference's
// CurrentHeatSolver (src/CurrentHeatSolver.cpp), on the same Q1 structure, kernels and PCG
// solvers as the vacuum field.
//
//   current (CurrentSolver::assemble, :421-489): Laplace with sigma = 1, the surface current
//     density j_f per copper-surface face as the Neumann value, phi = 0 at the copper bottom;
//   heat (HeatSolver::assemble + assemble_local_cell, :116-153, :347-398), implicit Euler:
//     (gamma M + K_kappa(T_prev)) T = gamma M T_prev + sigma(T_prev) |grad phi|^2 plus the heat
//     flux q_f per surface face, T = T_ambient at the bottom; gamma = rho_cp / dt;
//   material (PhysicalQuantities, src/PhysicalQuantities.cpp:31-64, 173-184): resistivity
//     rho(T) = 10 * linear interpolation of a (T, rho) table, T clamped to the table,
//     sigma = 1 / rho, kappa = lorentz * T * sigma.
// Boundary marking as CurrentHeatSolver::mark_mesh (:535-539): x/y extremes natural, z min
// the copper bottom, the rest copper surface; surface faces are ordered as the reference
// numbers its boundary values (bulk cells ascending, deal.II faces x-, x+, y-, y+, z-, z+).
// The emission model that produces j_f and q_f (GETELEC) is outside this library.
#pragma once

#include <memory>

#include "fem_device.h"

namespace fgb {

class BulkSolver {
public:
    BulkSolver(std::shared_ptr<const PreparedMesh> pm, cudaStream_t stream = nullptr);
    ~BulkSolver();
    BulkSolver(const BulkSolver&) = delete;
    BulkSolver& operator=(const BulkSolver&) = delete;

    void set_resistivity(const std::vector<double>& T, const std::vector<double>& rho);
    // CurrentHeatSolver::setup: T = t_ambient everywhere (and the bottom value), phi = 0;
    // rho_cp = volumetric heat capacity [J/(K A^3)] (CurrentHeatSolver.h:110 uses copper's)
    void setup(double t_ambient, double lorentz, double rho_cp);
    // host arrays of n_faces() values; returns #iterations (< 0: not converged)
    int solve_current(const double* face_j, const SolveOptions& opt, SolveStats* st);
    int solve_heat(double delta_time_s, const double* face_q, const SolveOptions& opt, SolveStats* st);

    int n_dofs() const { return cur_->n_dofs(); }
    int n_faces() const { return cur_->structure().n_top_faces(); }
    int64_t nnz() const { return cur_->structure().nnz(); }
    // surface faces: centroid (3 each, mean of the 4 corners) and (hex id, femocs local face)
    void surface_faces(double* centroid3, int32_t* hex_face2) const;
    // per hex-mesh node (non-bulk nodes: NaN): temperature and current potential
    void export_nodes(double* T_node, double* phi_node);
    // extremes of the temperature (HeatSolver::check_limits)
    void temperature_range(double* tmin, double* tmax);
    FemDevice& current() { return *cur_; }
    FemDevice& heat() { return *heat_; }

private:
    std::shared_ptr<const PreparedMesh> pm_;
    cudaStream_t stream_;
    bool own_stream_ = false;
    std::unique_ptr<FemDevice> cur_, heat_;
    DBuf<double> tab_T_, tab_rho_, face_j_, face_q_, fe_, tmp_;
    int n_tab_ = 0;
    double t_ambient_ = 300.0, lorentz_ = 2.44e-8, rho_cp_ = 3.4496e-24;
};

}  // namespace fgb
