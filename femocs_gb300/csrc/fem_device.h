// Device-resident Poisson system of one mesh and its solvers.
#pragma once

#include <cuda_runtime.h>

#include "device.h"
#include "fem.h"

#include <future>
#include <memory>

#include "cell_blocks.h"

namespace fgb {

// Scalars of one CG run, kept in device memory so that a whole chunk of iterations can be
// replayed from a CUDA graph without host round trips.
struct CgState {
    double rz, rz_new, pq, alpha, beta, rr, rr0, tol2;
    double ff;  // sum of squared row magnitudes |b| + |A||x| of the last compensated residual
    int iter, max_iter, done, status;  // status: 1 converged, 2 at the FP64 floor, -1 max_iter,
                                       // -2 breakdown/NaN, -3 no progress
    unsigned int ticket;
    int pad;
};

// Result block written by the persistent mixed-precision CG kernel.
struct MixedResult {
    int iterations, updates, status, pad;
    double rr;
};

// most values one grid-wide sum of the persistent mixed-precision CG reduces at once
constexpr int kMixedSumMax = 3;

// Arguments of the persistent mixed-precision CG kernel (cg_persistent.cu).
struct MixedArgs {
    int n;
    const int64_t* sptr;
    const int32_t* slen;
    const int32_t* scol;
    const float* s32;
    const double* s64;
    const float* dinv32;
    const double* b;
    double* x;
    float* d;
    float* r;
    float* z;
    float* pa;
    float* pb;
    float* q;
    double* partial;  // 2 buffers x kMixedSumMax values x grid CTAs
    MixedResult* out;
    double tol2;
    double ru2;       // squared reliable-update factor
    int max_iter;
    int comp;         // true residuals compensated (Dot2) when the tolerance nears the FP64 floor
};
void launch_mixed_cg(const MixedArgs& args, cudaStream_t stream);
int mixed_cg_grid(int n);

class AmgDevice;

// start vector of the multigrid setup's level-0 power iteration (amg_setup.cpp lambda_max)
constexpr uint64_t kAmgLambdaSeed = 0x12345678abcdefull;

struct SolveOptions {
    // 0: plain FP64 Jacobi-PCG; 1: FP32 Jacobi-PCG with FP64 reliable refinement (persistent
    // kernel); 2: FP64 CG preconditioned by an FP32 multigrid V-cycle
    int precision = 2;
    double rel_tol = 1e-9;    // on ||b - A x||_2 / ||b||_2 (FP64 true residual)
    double abs_tol = 0.0;     // optional absolute floor (reference field_cgtol semantics)
    int max_iter = 10000;     // total CG iterations (inner + plain)
    double inner_tol = 0.1;   // residual reduction between FP64 refinements (reliable updates)
    int max_outer = 50;
    int chunk = 16;           // iterations per graph launch
};

struct SolveStats {
    int iterations = 0;       // total CG iterations (all refinement sweeps)
    int outer = 0;            // refinement sweeps (0 for plain FP64)
    int status = 0;           // 1 converged, -1 not converged, -2 breakdown
    double rel_residual = 0;  // final ||b-Ax||/||b|| in FP64
    double bnorm = 0;
    double ms = 0;            // device time of the solve (CUDA events)
    double kernel_ms = 0;     // device time of the persistent CG kernel alone (mixed path)
    double setup_ms = 0;      // multigrid hierarchy construction in this call (0 when reused)
    int levels = 0;           // multigrid levels
    // with profiling on (multigrid path): summed device time and count of the level-0
    // Chebyshev smoothing launches and of the outer FP64 SpMV launches
    int smoother_launches = 0, spmv_launches = 0;
    double smoother_ms = 0, spmv_ms = 0;
    double smoother_bytes = 0;  // algorithmic bytes of one level-0 smoothing step
};

class FemDevice {
public:
    FemDevice(const PreparedMesh& pm, FemStructure&& fs, cudaStream_t stream);
    // multigrid hierarchy of the current matrix (built on first use, rebuilt when the anode
    // boundary condition changes the eliminated matrix)
    void ensure_amg(SolveStats* st);
    std::string amg_levels() const;
    // event pairs around the multigrid path's hot launches (see SolveStats)
    void set_profiling(bool on);
    // Chebyshev smoothing of the finest multigrid level: degree (steps before and after the
    // coarse correction) and the lower end of the interval as a fraction of lambda_max;
    // 0 keeps the default (Q1: 4 and 0.04; Q2: 2 and 0.1). Drops the current hierarchy.
    void set_smoothing(int degree, double lo);
    // Q2 element matrices on the tensor cores (q2_ke_tc.cu, default) or the FP32 pipe (FP32
    // hi/lo pairs)
    void set_ke_tensor(bool on);
    // element matrices of the last full assembly (Q1: 64 per cell, Q2: 378 packed per cell)
    void export_element_matrices(double* out);
    size_t element_matrix_values() const { return ke_.size(); }
    // Q2 level 0 by cell blocks: element matrices streamed by bulk copies or loaded by the
    // applying warps (default)
    void set_level0_stream(bool on);
    void set_level0_prefetch(int cells);
    // Q2 level 0 by cell blocks: element matrices (0) or geometric factors in FP32 (1) or
    // FP16 (2), applied by sum factorisation; returns the kind in use (FP16 falls back to FP32
    // when an entry is beyond its range)
    int set_level0_operator(int kind);
    // multigrid: cycles of level+1 per coarse-grid correction at `level` (1 = V-cycle)
    void set_coarse_cycles(int level, int cycles);
    // multigrid: Chebyshev degree and interval of level `level` >= 1 (Q2: level 1 is the Q1
    // system; 0 = the hierarchy's default), applied from the next solve without a rebuild
    void set_level_smoothing(int level, int degree, double lo);
    // Q2: apply the finest multigrid level element by element, by cell blocks (cell_blocks.h;
    // default: 4.3 vs 8.95 GB per smoothing step on the 1.7e7-DoF Q2 nanotip), or through the
    // assembled SELL matrix; the hierarchy is rebuilt at the next solve
    void set_level0_ebe(bool on);
    // Q2: form the assembled SELL matrices at every assembly (false) or only when read (true,
    // the default); results are the same
    void set_lazy_matrix(bool on);
    // outer SpMV of the multigrid PCG: 1 = the SELL matrix as FP32 hi/lo pairs with error-free
    // products (Q1 default; FP64-accurate to ~2^-48 per term, off the FP64 pipe), 2 = the same
    // arithmetic element by element over the cell blocks (Q2 default: half the bytes of the
    // assembled pairs), 0 = the FP64 SELL matrix
    void set_outer_spmv(int mode);
    int outer_spmv() const { return outer_mode_; }
    // limits of the Q2 cell blocks (hexes per block, DoFs per block: at most 256 and 4096);
    // drops the blocks, the converted element matrices and the hierarchy
    void set_cell_blocks(int cells_per_block, int max_dofs);
    // algorithmic bytes of one outer SpMV launch in the current mode
    double outer_spmv_bytes() const;
    ~FemDevice();

    // PoissonSolver::setup + assemble verbs (src/PoissonSolver.cpp:162-210)
    void setup(double applied_field, double applied_potential);   // zeroes the solution
    void assemble(bool full_run, bool anode_dirichlet);
    // Q1 hooks of the bulk (current/heat) systems: element matrices written by the caller into
    // d_ke() (64 per cell, row-major), per-face Neumann values (device, one per Neumann face in
    // the structure's order; null = the applied field), the value of the kind-1 Dirichlet rows
    double* d_ke() { return ke_.get(); }
    void assemble_from_ke(bool anode_dirichlet);
    void set_face_values(const double* d_vals) { face_vals_ = d_vals; }
    void set_dirichlet_value(double v) { dirichlet_value_ = v; }
    const int32_t* d_r2c_ptr() const { return r2c_ptr_.get(); }
    const int32_t* d_r2c_item() const { return r2c_item_.get(); }
    const double* d_dof_xyz() const { return dof_xyz_.get(); }
    // adds a space-charge contribution rhs[dof] += w * N(point) to the unconstrained rhs
    // before Dirichlet application; values given per dof (already summed)
    void set_space_charge(const double* d_rhs_extra);
    // PIC space charge: a zeroed (or kept) per-DoF rhs that particles scatter into; it is
    // added to the rhs at the next assemble, before the Dirichlet values (as the reference's
    // assemble_space_charge). clear_space_charge() drops it.
    double* space_charge_buffer(bool accumulate);
    void clear_space_charge() { has_extra_ = false; }
    const int32_t* d_node2dof();   // hex-mesh node -> DoF (Q1) or -1
    const int32_t* d_hex2cell();   // hex -> vacuum cell index or -1
    const int32_t* d_cell_dofs() const { return cell_dofs_.get(); }
    int solve(const SolveOptions& opt, SolveStats* st);

    // solution by dof / by mesh node
    const double* d_solution() const { return x_.get(); }
    double* d_solution() {  // writable: the solution is no longer known to be zero
        x_zero_ = false;
        return x_.get();
    }
    const FemStructure& structure() const { return fs_; }
    int n_dofs() const { return fs_.n_dofs; }
    int64_t nnz() const { return fs_.nnz(); }
    const int32_t* d_dof2node() const { return dof2node_.get(); }
    double last_spmv_ms(int precision) const { return precision ? spmv32_ms_ : spmv64_ms_; }
    // measure: average device time of one SpMV (64 or 32 bit values) over `reps` launches
    double time_spmv(int precision, int reps);
    void download_matrix(std::vector<double>& vals, std::vector<double>& rhs);
    // CSR pattern of the system (Q1: the host structure; Q2: read back from the SELL layout)
    void download_pattern(std::vector<int64_t>& rowptr, std::vector<int32_t>& col);
    int order() const { return fs_.order; }
    cudaStream_t stream() const { return stream_; }
    // device arrays of the assembled system (SELL-32 layout of the structure), for placing
    // the system into a multi-mesh batch
    const double* d_sell64() const { return sell64_.get(); }
    const float* d_sell32() const { return sell32_.get(); }
    const int32_t* d_sell_col() const { return sell_col_.get(); }
    const float* d_dinv32() const { return dinv32_.get(); }
    const double* d_rhs() const { return rhs_.get(); }

private:
    void spmv64(const double* x, double* y);
    void assemble_q1_rows(bool matrix, bool anode_dirichlet);
    int solve_plain(const SolveOptions& opt, SolveStats* st);
    int solve_mixed(const SolveOptions& opt, SolveStats* st);
    int solve_amg(const SolveOptions& opt, SolveStats* st);
    int solve_amg_mixed(const SolveOptions& opt, SolveStats* st);
    void prepare_amg(SolveStats* st);  // hierarchy on first use, per-level settings
    void run_cg(bool fp32, CgState* d_state, int max_iter, int chunk);

    FemStructure fs_;
    const PreparedMesh* pm_;
    cudaStream_t stream_;
    std::unique_ptr<AmgDevice> amg_;
    int amg_anode_ = -1;
    std::unique_ptr<FemDevice> q1_;   // Q2: the Q1 system of the same mesh, coarse level of the multigrid
    void build_q2_amg(int anode, SolveStats* st);
    // power iteration on D^-1 A (FP64, device) from the pseudo-random start of `seed`
    double estimate_lambda(int iters, uint64_t seed = 0x9e3779b97f4a7c15ull);  // largest eigenvalue of D^-1 A (FP64 power iteration)
    bool profiling_ = false;
    int smooth_degree_ = 0;
    std::vector<int> coarse_cycles_;
    std::vector<std::pair<int, double>> level_smooth_;  // per level (index 0 unused): degree, lo
    bool level0_stream_ = false;
    // L2 prefetch one group ahead (measured best on the 1.7e7-DoF Q2 nanotip)
    int level0_prefetch_ = 1;
    // requested level-0 operator source (set_level0_operator): FP16 geometric factors (0.69 vs
    // 0.89 ms per step on the 1.7e7-DoF Q2 nanotip)
    int level0_geo_ = 2;
    int geo_built_ = 0;           // kind held in geo_ (0: none)
    int geo_for_ = 0;             // kind requested when geo_ was built (2 may hold FP32: fallback)
    DBuf<unsigned char> geo_;     // geometric factors in block order (q2_geometric_factors)
    DBuf<unsigned> geo_max_;
    void ensure_geo();
    bool ke_tensor_ = true;
    DBuf<unsigned char> tc_scratch_;  // tensor-core element matrices: slices per persistent CTA
    DBuf<unsigned> tc_err_;
    double smooth_lo_ = 0;
    int q1_gauss_ = 2;  // Gauss points per direction of the Q1 element integrals
    bool level0_ebe_ = false;
    int outer_mode_ = 1;
    bool split_valid_ = false;
    // Q2: the assembled SELL values (kval_, then sell64_/sell32_) are formed only when a
    // consumer needs them (ensure_sell): with all Dirichlet values zero, D^-1, the right-hand
    // side and x come from the element matrices directly, and the multigrid PCG over the cell
    // blocks reads neither matrix
    bool lazy_matrix_ = true;
    bool kval_valid_ = false;   // kval_ holds the rows of the current element matrices
    bool sell_valid_ = true;    // sell64_/sell32_ hold the current eliminated values
    void ensure_sell();
    // r64 = b - A x from the FP64 element matrices (Q2, no assembled matrix), returns |r|^2
    double cells_true_residual();
    DBuf<CgState> res_state_;
    DBuf<double> cell_y_;       // K_e x_e per cell (27 per cell) for that residual
    bool x_zero_ = true;        // x is the zero vector of setup() (no solve or write since)
    DBuf<float> sell_lo_;  // low FP32 part of the matrix values (high part: sell32_)
    DBuf<float2> p2_;      // p as interleaved FP32 (hi, lo) pairs
    void ensure_split();
    DBuf<float> ke32_;      // Q2: FP32 element matrices in block order, cyclic half (EbeOperator)
    struct CellBlocksDev;
    std::unique_ptr<CellBlocksDev> cb_;
    void ensure_cell_blocks();
    void refresh_ke32();    // element matrices (ke_) into ke32_ (and ke32lo_ for outer mode 2)
    DBuf<float> ke32lo_;    // low FP32 parts of the element matrices, same layout as ke32_
    DBuf<float2> cb_pair_;  // outer mode 2: partial (hi, lo) sums of the split DoFs
    DBuf<double> cb_dot_;   // outer mode 2: p.q partials
    bool cb_spmv_attr_ = false;
    // cell blocks of at most 176 hexes / 2816 DoFs: the largest whose matrix-free smoother
    // shared memory (56.4 KB) lets 4 CTAs of 64 registers share an SM (1.7e7-DoF Q2 nanotip:
    // smoothing step 0.648 ms against 0.685 ms for 256 / 4096, outer product 1.70 against
    // 1.77 ms)
    int cb_cells_ = 176, cb_max_dofs_ = 2816;
    DBuf<int8_t> fixed_;    // 1 on Dirichlet rows of the current anode mode
    LaunchTimer spmv_timer_;
    int n_, nc_;
    double applied_field_ = 0, applied_potential_ = 0;
    bool anode_dirichlet_ = false;
    // structure
    DBuf<int32_t> cell_dofs_, r2c_ptr_, r2c_item_, r2f_ptr_, r2f_item_, top_faces_, dof2node_;
    DBuf<int64_t> rowptr_, slice_ptr_, csr2sell_;
    DBuf<int32_t> col_, slice_len_, sell_col_, row_len_;
    int max_row_ = 0;
    DBuf<int8_t> bc_;
    DBuf<int32_t> node2dof_dev_, hex2cell_dev_;
    DBuf<double> dof_xyz_;
    // values
    DBuf<double> ke_;        // Q1: 64 per cell; Q2: 378 (packed upper triangle)
    DBuf<double> kval_;      // values before Dirichlet (saved matrix): Q1 CSR order, Q2 SELL layout
    DBuf<double> sell64_;    // SELL values after Dirichlet
    DBuf<float> sell32_;
    DBuf<double> dinv64_;
    DBuf<float> dinv32_;
    DBuf<double> rhs_, rhs_extra_, x_;
    const double* face_vals_ = nullptr;
    double dirichlet_value_ = 0.0;
    bool has_extra_ = false;
    // work vectors
    DBuf<double> r64_, p64_, q64_, z64_;
    DBuf<float> r32_, p32_, p32b_, q32_, z32_, d32_;
    DBuf<double> partial_;
    DBuf<CgState> state_;
    DBuf<MixedResult> mixed_;
    MixedResult* h_mixed_ = nullptr;
    CgState* h_state_ = nullptr;  // pinned mirror
    double spmv64_ms_ = 0, spmv32_ms_ = 0;
    cudaEvent_t ev0_, ev1_, kev0_, kev1_;
    // host work started at construction on other threads (declared last: destroyed, that is
    // waited for, before the structure they read): the Q2 cell blocks of the default shape,
    // and the Q1 structure of a Q2 field's coarse level (set_q1_structure)
    std::future<CellBlocks> cb_host_;
    int cb_host_cells_ = 0, cb_host_dofs_ = 0;
    std::future<FemStructure> q1_fs_;

public:
    void set_q1_structure(std::future<FemStructure> f) { q1_fs_ = std::move(f); }
};

}  // namespace fgb
