#include "field.h"

#include <future>

namespace fgb {

Field::Field(std::shared_ptr<const PreparedMesh> pm, cudaStream_t stream, int order)
    : pm_(std::move(pm)), stream_(stream) {
    FGB_REQUIRE(order == 1 || order == 2, "element order must be 1 or 2");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        throw Error("no CUDA device available: the femocs_gb300 field path runs on the GPU only");
    if (!stream_) {
        FGB_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
        own_stream_ = true;
    }
    if (order == 2) {
        // the Q1 structure of the same mesh, the coarse level of the Q2 multigrid (needed at
        // the first solve), is built on another host thread while the Q2 structure is built here
        std::shared_ptr<const PreparedMesh> pm = pm_;
        std::future<FemStructure> q1 = std::async(std::launch::async, [pm] { return build_fem_structure(*pm); });
        fem_.reset(new FemDevice(*pm_, build_q2_structure(*pm_, false), stream_));
        fem_->set_q1_structure(std::move(q1));
    } else {
        fem_.reset(new FemDevice(*pm_, build_fem_structure(*pm_), stream_));
    }
    dm_.reset(new DeviceMesh(*pm_, stream_));
}

Field::~Field() {
    fem_.reset();
    dm_.reset();
    if (own_stream_) cudaStreamDestroy(stream_);
}

int Field::solve_laplace(double E0, double V0, bool anode_dirichlet, const SolveOptions& opt, bool smoothen,
                         SolveStats* st) {
    fem_->setup(-E0, V0);
    fem_->assemble(true, anode_dirichlet);
    const int rc = fem_->solve(opt, st);
    extract(smoothen);
    return rc;
}

void Field::extract(bool smoothen) {
    dm_->extract_solution(fem_->d_solution(), fem_->d_dof2node(), fem_->n_dofs(), smoothen);
}

int Field::space_charge(int n, const double* d_pts, const int32_t* d_hex, double charge_factor, bool accumulate) {
    double* rhs = fem_->space_charge_buffer(accumulate);
    if (n <= 0) return 0;
    const int32_t* hex = d_hex;
    if (!hex) {
        if (out_.size() < 5 * (size_t)n) out_.resize(5 * (size_t)n);
        if (cells_.size() < (size_t)n) cells_.resize(n);
        dm_->locate_interpolate(n, d_pts, 3, cells_.get(), out_.get(), nullptr);
        hex = cells_.get();
    }
    int skipped = 0;
    dm_->space_charge(n, d_pts, hex, fem_->order(), fem_->d_node2dof(), fem_->d_hex2cell(), fem_->d_cell_dofs(),
                      charge_factor, rhs, &skipped);
    return skipped;
}

void Field::interpolate_host(int n, const double* xyz, int rank, int32_t* cells, double* out5, LocateStats* ls) {
    if (n <= 0) return;
    if (pts_.size() < 3 * (size_t)n) pts_.resize(3 * (size_t)n);
    if (out_.size() < 5 * (size_t)n) out_.resize(5 * (size_t)n);
    if (cells_.size() < (size_t)n) cells_.resize(n);
    FGB_CUDA(cudaMemcpyAsync(pts_.get(), xyz, 3 * sizeof(double) * n, cudaMemcpyHostToDevice, stream_));
    dm_->locate_interpolate(n, pts_.get(), rank, cells_.get(), out_.get(), ls);
    if (cells) FGB_CUDA(cudaMemcpyAsync(cells, cells_.get(), sizeof(int32_t) * n, cudaMemcpyDeviceToHost, stream_));
    if (out5) FGB_CUDA(cudaMemcpyAsync(out5, out_.get(), 5 * sizeof(double) * n, cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
}

void Field::interpolate_surface_host(int n, const double* xyz, int rank, int32_t* cells, double* out5) {
    if (n <= 0) return;
    if (pts_.size() < 3 * (size_t)n) pts_.resize(3 * (size_t)n);
    if (out_.size() < 5 * (size_t)n) out_.resize(5 * (size_t)n);
    if (cells_.size() < (size_t)n) cells_.resize(n);
    FGB_CUDA(cudaMemcpyAsync(pts_.get(), xyz, 3 * sizeof(double) * n, cudaMemcpyHostToDevice, stream_));
    dm_->surface_interpolate(n, pts_.get(), rank, cells_.get(), out_.get());
    if (cells) FGB_CUDA(cudaMemcpyAsync(cells, cells_.get(), sizeof(int32_t) * n, cudaMemcpyDeviceToHost, stream_));
    if (out5) FGB_CUDA(cudaMemcpyAsync(out5, out_.get(), 5 * sizeof(double) * n, cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
}

}  // namespace fgb
