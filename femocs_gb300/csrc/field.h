// One mesh on the device: the Poisson system (FemDevice) and the interpolator (DeviceMesh)
// sharing a CUDA stream. This is the GPU counterpart of the reference's PoissonSolver<3>
// plus the vacuum Interpolator of ProjectRunaway.
#pragma once

#include <memory>

#include "fem_device.h"
#include "interp.h"

namespace fgb {

class Field {
public:
    // order: 1 = Q1 elements (the reference's), 2 = Q2 (27-node hexahedra on the same mesh)
    explicit Field(std::shared_ptr<const PreparedMesh> pm, cudaStream_t stream = nullptr, int order = 1);
    ~Field();

    const PreparedMesh& mesh() const { return *pm_; }
    FemDevice& fem() { return *fem_; }
    DeviceMesh& interp() { return *dm_; }
    cudaStream_t stream() const { return stream_; }

    // ProjectRunaway::solve_laplace (src/ProjectRunaway.cpp:422-447): setup(-E0,V0),
    // assemble(true), solve, extract_solution
    int solve_laplace(double E0, double V0, bool anode_dirichlet, const SolveOptions& opt, bool smoothen, SolveStats* st);

    // host-pointer interpolation through reusable device buffers
    void interpolate_host(int n, const double* xyz, int rank, int32_t* cells, double* out5, LocateStats* ls);
    // surface (2-D) variant: cells are surface triangles (DeviceMesh::surface_interpolate)
    void interpolate_surface_host(int n, const double* xyz, int rank, int32_t* cells, double* out5);
    void extract(bool smoothen);
    // PIC: scatter n particles (device xyz) with charge factor q/eps0 * W_sp into the space-
    // charge rhs of the next assemble; d_hex = their vacuum hexes, or null to locate them
    // first (rank-3 location, as the reference keeps particle.cell). Returns the particles
    // outside the vacuum hexes.
    int space_charge(int n, const double* d_pts, const int32_t* d_hex, double charge_factor, bool accumulate);

private:
    std::shared_ptr<const PreparedMesh> pm_;
    cudaStream_t stream_;
    bool own_stream_ = false;
    std::unique_ptr<FemDevice> fem_;
    std::unique_ptr<DeviceMesh> dm_;
    DBuf<double> pts_, out_;
    DBuf<int32_t> cells_;
};

}  // namespace fgb
