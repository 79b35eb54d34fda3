// Current and heat on the bulk hexahedra (see bulk.h).
//   k_heat_cell   per bulk cell, 2x2x2 Gauss on the trilinear map: the heat element matrix
//                 JxW (gamma N_i N_j + kappa(T_q) grad N_i . grad N_j) and the element rhs
//                 JxW N_i (gamma T_q + sigma(T_q) |grad phi_q|^2), T_q and grad phi_q from the
//                 nodal T_prev and current potential (HeatSolver::assemble_local_cell)
//   k_sum_rows    element rhs -> per-DoF rhs through the row -> (cell, local) lists
#include "bulk.h"

#include <cmath>
#include <limits>

namespace fgb {

namespace {

constexpr int kB = 256;
__constant__ double c_bx[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
__constant__ double c_by[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
__constant__ double c_bz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};

// PhysicalQuantities::linear_interp (src/PhysicalQuantities.cpp:173-184): table ends outside,
// else the segment found by lower_bound on T
__device__ double table_interp(double x, const double* __restrict__ T, const double* __restrict__ R, int n) {
    if (x <= T[0]) return R[0];
    if (x >= T[n - 1]) return R[n - 1];
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (T[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return R[lo - 1] + (R[lo] - R[lo - 1]) * (x - T[lo - 1]) / (T[lo] - T[lo - 1]);
}
__device__ __forceinline__ double clamp_t(double t, const double* T, int n) {
    if (t < T[0]) t = T[0];
    if (t > T[n - 1]) t = T[n - 1];
    return t;
}
// sigma = 1 / (10 rho(T)), kappa = lorentz T sigma(T), T clamped (PhysicalQuantities::sigma/kappa)
__device__ __forceinline__ double sigma_of(double t, const double* T, const double* R, int n) {
    return 1.0 / (10. * table_interp(clamp_t(t, T, n), T, R, n));
}

__global__ void k_heat_cell(int nc, const int32_t* __restrict__ cd, const double* __restrict__ dxyz,
                            const double* __restrict__ tprev, const double* __restrict__ phi, double gamma,
                            double lorentz, const double* __restrict__ tabT, const double* __restrict__ tabR, int ntab,
                            double* __restrict__ ke, double* __restrict__ fe) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    double X[8][3], tn[8], pn[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int d = cd[8 * (size_t)c + k];
        X[k][0] = dxyz[3 * (size_t)d];
        X[k][1] = dxyz[3 * (size_t)d + 1];
        X[k][2] = dxyz[3 * (size_t)d + 2];
        tn[k] = tprev[d];
        pn[k] = phi[d];
    }
    double K[36], F[8];
#pragma unroll
    for (int i = 0; i < 36; ++i) K[i] = 0.0;
#pragma unroll
    for (int i = 0; i < 8; ++i) F[i] = 0.0;
    const double g = 0.57735026918962576451;
#pragma unroll 1
    for (int q = 0; q < 8; ++q) {
        const double xi = (q & 1) ? g : -g, eta = (q & 2) ? g : -g, zeta = (q & 4) ? g : -g;
        double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        double N[8], dN[8][3];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const double ax = c_bx[k], ay = c_by[k], az = c_bz[k];
            N[k] = (1 + xi * ax) * (1 + eta * ay) * (1 + zeta * az) * 0.125;
            dN[k][0] = ax * (1 + eta * ay) * (1 + zeta * az) * 0.125;
            dN[k][1] = (1 + xi * ax) * ay * (1 + zeta * az) * 0.125;
            dN[k][2] = (1 + xi * ax) * (1 + eta * ay) * az * 0.125;
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) J[a][b] += X[k][a] * dN[k][b];
        }
        const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        const double id = 1.0 / det;
        double inv[3][3];
        inv[0][0] = c00 * id;
        inv[1][0] = c01 * id;
        inv[2][0] = c02 * id;
        inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
        inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
        inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
        inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
        inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
        inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
        double G[8][3];
        double tq = 0.0, gp[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                G[k][a] = inv[0][a] * dN[k][0] + inv[1][a] * dN[k][1] + inv[2][a] * dN[k][2];
                gp[a] += G[k][a] * pn[k];
            }
            tq += N[k] * tn[k];
        }
        const double w = fabs(det);
        const double sig = sigma_of(tq, tabT, tabR, ntab);
        const double kap = lorentz * clamp_t(tq, tabT, ntab) * sig;
        const double src = gamma * tq + sig * (gp[0] * gp[0] + gp[1] * gp[1] + gp[2] * gp[2]);
        int t = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            F[i] += w * N[i] * src;
#pragma unroll
            for (int j = i; j < 8; ++j, ++t)
                K[t] += w * (gamma * N[i] * N[j] + kap * (G[i][0] * G[j][0] + G[i][1] * G[j][1] + G[i][2] * G[j][2]));
        }
    }
    double* o = ke + 64 * (size_t)c;
    int t = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = i; j < 8; ++j, ++t) {
            o[8 * i + j] = K[t];
            o[8 * j + i] = K[t];
        }
#pragma unroll
    for (int i = 0; i < 8; ++i) fe[8 * (size_t)c + i] = F[i];
}

__global__ void k_sum_rows(int n, const int32_t* __restrict__ r2c_ptr, const int32_t* __restrict__ r2c_item,
                           const double* __restrict__ fe, double* __restrict__ out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double acc = 0.0;
    for (int p = r2c_ptr[r]; p < r2c_ptr[r + 1]; ++p) acc += fe[r2c_item[p]];
    out[r] = acc;
}

__global__ void k_fill(int n, double v, double* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = v;
}

}  // namespace

BulkSolver::BulkSolver(std::shared_ptr<const PreparedMesh> pm, cudaStream_t stream) : pm_(std::move(pm)), stream_(stream) {
    if (!stream_) {
        FGB_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
        own_stream_ = true;
    }
    cur_.reset(new FemDevice(*pm_, build_fem_structure(*pm_, kRegionBulk), stream_));
    heat_.reset(new FemDevice(*pm_, build_fem_structure(*pm_, kRegionBulk), stream_));
    fe_.resize(8 * (size_t)cur_->structure().n_cells);
    // bulk copper by default until a table is set: a constant resistivity table
    set_resistivity({300.0, 301.0}, {1.7e-8, 1.7e-8});
    setup(t_ambient_, lorentz_, rho_cp_);
}

BulkSolver::~BulkSolver() {
    cur_.reset();
    heat_.reset();
    if (own_stream_) cudaStreamDestroy(stream_);
}

void BulkSolver::set_resistivity(const std::vector<double>& T, const std::vector<double>& rho) {
    FGB_REQUIRE(T.size() == rho.size() && T.size() >= 2, "resistivity table needs >= 2 (T, rho) pairs");
    for (size_t i = 1; i < T.size(); ++i) FGB_REQUIRE(T[i] > T[i - 1], "resistivity table: T must increase");
    for (double r : rho) FGB_REQUIRE(r > 0, "resistivity must be positive");
    tab_T_.upload(T, stream_);
    tab_rho_.upload(rho, stream_);
    n_tab_ = (int)T.size();
    FGB_CUDA(cudaStreamSynchronize(stream_));
}

void BulkSolver::setup(double t_ambient, double lorentz, double rho_cp) {
    FGB_REQUIRE(rho_cp > 0 && lorentz > 0, "heat capacity and Lorentz number must be positive");
    t_ambient_ = t_ambient;
    lorentz_ = lorentz;
    rho_cp_ = rho_cp;
    cur_->setup(0.0, 0.0);
    heat_->setup(0.0, 0.0);
    heat_->set_dirichlet_value(t_ambient);
    FGB_LAUNCH(k_fill<<<grid_for(n_dofs(), kB), kB, 0, stream_>>>(n_dofs(), t_ambient, heat_->d_solution()));
    FGB_CUDA(cudaGetLastError());
}

int BulkSolver::solve_current(const double* face_j, const SolveOptions& opt, SolveStats* st) {
    const int nf = n_faces();
    face_j_.resize(std::max(nf, 1));
    if (nf) FGB_CUDA(cudaMemcpyAsync(face_j_.get(), face_j, sizeof(double) * nf, cudaMemcpyHostToDevice, stream_));
    cur_->set_face_values(face_j_.get());
    cur_->assemble(true, false);
    return cur_->solve(opt, st);
}

int BulkSolver::solve_heat(double delta_time_s, const double* face_q, const SolveOptions& opt, SolveStats* st) {
    FGB_REQUIRE(delta_time_s > 0, "invalid delta time");
    const int nf = n_faces();
    face_q_.resize(std::max(nf, 1));
    if (nf) FGB_CUDA(cudaMemcpyAsync(face_q_.get(), face_q, sizeof(double) * nf, cudaMemcpyHostToDevice, stream_));
    const FemStructure& fs = heat_->structure();
    const double gamma = rho_cp_ / delta_time_s;
    FGB_LAUNCH(k_heat_cell<<<grid_for(fs.n_cells, 128), 128, 0, stream_>>>(
        fs.n_cells, heat_->d_cell_dofs(), heat_->d_dof_xyz(), heat_->d_solution(), cur_->d_solution(), gamma, lorentz_,
        tab_T_.get(), tab_rho_.get(), n_tab_, heat_->d_ke(), fe_.get()));
    double* rhs = heat_->space_charge_buffer(false);
    FGB_LAUNCH(k_sum_rows<<<grid_for(n_dofs(), kB), kB, 0, stream_>>>(n_dofs(), heat_->d_r2c_ptr(), heat_->d_r2c_item(),
                                                                     fe_.get(), rhs));
    heat_->set_face_values(face_q_.get());
    heat_->set_dirichlet_value(t_ambient_);
    heat_->assemble_from_ke(false);
    FGB_CUDA(cudaGetLastError());
    return heat_->solve(opt, st);
}

void BulkSolver::surface_faces(double* centroid3, int32_t* hex_face2) const {
    const FemStructure& fs = cur_->structure();
    const RegionCells rc = region_cells(*pm_, kRegionBulk);
    const int nf = fs.n_top_faces();
    for (int f = 0; f < nf; ++f) {
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += pm_->hex.xyz[3 * (size_t)fs.dof2node[fs.top_faces[4 * (size_t)f + k]] + c];
            if (centroid3) centroid3[3 * (size_t)f + c] = s / 4.0;
        }
        if (hex_face2) {
            hex_face2[2 * (size_t)f] = rc.cells[fs.top_face_cells[f]];
            hex_face2[2 * (size_t)f + 1] = fs.top_face_local[f];
        }
    }
}

void BulkSolver::export_nodes(double* T_node, double* phi_node) {
    const FemStructure& fs = cur_->structure();
    const int n = n_dofs();
    std::vector<double> t(n), p(n);
    FGB_CUDA(cudaMemcpyAsync(t.data(), heat_->d_solution(), sizeof(double) * n, cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaMemcpyAsync(p.data(), cur_->d_solution(), sizeof(double) * n, cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    const int nn = pm_->hex.n_nodes();
    const double nan = std::numeric_limits<double>::quiet_NaN();
    for (int i = 0; i < nn; ++i) {
        if (T_node) T_node[i] = nan;
        if (phi_node) phi_node[i] = nan;
    }
    for (int d = 0; d < n; ++d) {
        if (T_node) T_node[fs.dof2node[d]] = t[d];
        if (phi_node) phi_node[fs.dof2node[d]] = p[d];
    }
}

void BulkSolver::temperature_range(double* tmin, double* tmax) {
    const int n = n_dofs();
    std::vector<double> t(n);
    FGB_CUDA(cudaMemcpyAsync(t.data(), heat_->d_solution(), sizeof(double) * n, cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    double a = 1e300, b = -1e300;
    for (double v : t) {
        a = std::min(a, v);
        b = std::max(b, v);
    }
    if (tmin) *tmin = a;
    if (tmax) *tmax = b;
}

}  // namespace fgb
