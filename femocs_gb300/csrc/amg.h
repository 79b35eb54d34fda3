// Multigrid preconditioner for the vacuum Poisson system.
//
// Level 0 is the Q1 system on the hex mesh. Level 1 lives on the free vacuum tet vertices:
// its prolongation is the exact linear (P1) interpolation the tet->hex split used to create
// the hex nodes (edge midpoints 1/2, face centroids 1/3, tet centroids 1/4), so the first
// coarsening is geometric. Deeper levels use smoothed aggregation; the coarsest level is
// solved with a dense inverse. Galerkin coarse operators (R A P) throughout; Chebyshev
// smoothing on D^-1 A. The V-cycle runs in FP32 on the device as the preconditioner of an
// FP64 CG, whose SpMV, residual and solution update stay FP64.
#pragma once

#include <memory>

#include "device.h"
#include "fem.h"

namespace fgb {

struct CsrD {
    int n_rows = 0, n_cols = 0;
    std::vector<int64_t> ptr;
    std::vector<int32_t> col;
    std::vector<double> val;
    int64_t nnz() const { return ptr.empty() ? 0 : ptr.back(); }
};

struct AmgHostLevel {
    CsrD A;        // operator on this level
    CsrD P, R;     // prolongation to this level from the next coarser one, and its transpose
    double lambda = 1.0;  // estimate of the largest eigenvalue of D^-1 A
    int cheb_degree = 3;  // Chebyshev smoothing steps before and after the coarse correction
    double cheb_lo = 0.06; // smoothing interval [cheb_lo, 1.1] x lambda
    // P and R were built on the device and are handed over with AmgDevice::adopt_transfers
    // (P.n_rows / P.n_cols give the shape; the host arrays stay empty)
    bool transfers_on_device = false;
    // operator already on the device as SELL-32 with 4-wide chunks (FP32 values, the
    // eliminated FP64 matrix rounded, and its FP32 inverse diagonal), owned by the caller and
    // alive as long as the hierarchy: used instead of packing and uploading A
    const int64_t* dev_sptr = nullptr;
    const int32_t* dev_slen = nullptr;
    const int32_t* dev_scol = nullptr;
    const float* dev_val = nullptr;
    const float* dev_dinv = nullptr;
};

struct AmgHost {
    std::vector<AmgHostLevel> levels;  // levels[0] = fine; last level has no P/R
    std::vector<double> coarse_inv;    // dense inverse of the coarsest operator (row major)
    int n_coarse = 0;
    double setup_ms = 0;
};

struct AmgOptions {
    double strength = 0.08;  // aggregation strength threshold
    int max_coarse = 1500;   // dense solve below this size
    int max_dense = 4096;    // largest dense coarsest level accepted
    int max_levels = 10;
    double level0_lambda = 0.0;  // > 0: lambda_max of D^-1 A on level 0, already estimated (device)
};

// fixed: 1 for Dirichlet rows (copper, and the anode when it is a Dirichlet boundary)
AmgHost build_amg(const PreparedMesh& pm, const FemStructure& fs, const std::vector<double>& a0_val,
                  const std::vector<int8_t>& fixed, const AmgOptions& opt = AmgOptions());

struct AmgDevLevel;

// Element-by-element form of a level-0 operator (Q2), applied by cell blocks (cell_blocks.h):
// y = sum over cells of K_e x_e, rows of Dirichlet DoFs replaced by diag * x -- the eliminated
// operator on vectors that vanish on the Dirichlet DoFs, which every V-cycle vector does
struct EbeOperator {
    int n_cells = 0, n_blocks = 0, max_cells = 0, max_dofs = 0, n_bnd = 0, n_slots = 0;
    int64_t n_local = 0;
    // 378 per block position, cyclic half of K_e: K_e(i, (i + t) mod 27) for t = 0..13 (27 is
    // odd, so every off-diagonal pair appears exactly once), stored at 54 (t / 2) + 2 i + t % 2
    const float* ke = nullptr;
    const int32_t* cell_start = nullptr;  // block -> first position
    const int32_t* dof_start = nullptr;   // block -> first local DoF entry
    const int32_t* dof_list = nullptr;    // local entry -> global DoF
    const uint16_t* item_end = nullptr;   // local entry -> end of its items (block-relative)
    const int32_t* slot = nullptr;        // local entry -> partial slot, -1 when complete
    const uint16_t* loc = nullptr;        // 27 per position: local entry of each lattice DoF
    const uint16_t* items = nullptr;      // 28 per position: products grouped by local entry
    const int32_t* bnd_dofs = nullptr;    // DoFs split over blocks
    const int32_t* bnd_ptr = nullptr;     // their slots bnd_ptr[j] .. bnd_ptr[j+1]-1, ascending block
    float* partial = nullptr;             // n_slots
    const int8_t* fixed = nullptr;        // 1 on Dirichlet rows
    int64_t n_ke = 0;                     // floats in ke (378 per cell)
    unsigned* err = nullptr;              // bounded waits of the streamed kernel that timed out
    int prefetch = 0;                     // element matrices prefetched into L2, cells ahead per warp
    // geometric factors instead of the element matrices (0: element matrices; 1: FP32, 2: FP16):
    // per position 81 pairs at [(qx, m), pencil] = 9 (3 qx + m) + qy + 3 qz, pair m = (C00, C11),
    // (C22, C01), (C02, C12) of C_q = w_q |det J_q| J_q^-1 J_q^-T at Gauss point (qx, qy, qz)
    const void* geo = nullptr;
    int geo_kind = 0;
};

// Device side of the hierarchy and the V-cycle (amg.cu).
class AmgDevice {
public:
    AmgDevice(const AmgHost& h, cudaStream_t stream, const int64_t* l0_sptr, const int32_t* l0_slen,
              const int32_t* l0_scol, const float* l0_val, const float* l0_dinv);
    ~AmgDevice();
    // z = V(r) on level 0 (FP32, length n0); z is the hierarchy's own buffer, valid until the
    // next cycle
    const float* vcycle(const float* r);
    // y = b - A0 x with the level-0 operator the smoother applies (FP32: the SELL matrix, or
    // for Q2 the element matrices or geometric factors by cell blocks); b may be all zeros
    void level0_residual(const float* b, const float* x, float* y);
    int n_levels() const;
    // "rows:nnz" per level, coarsest marked dense
    std::string describe() const;
    // average device time [ms] of one level-0 Chebyshev smoothing step (one FP32 SpMV plus
    // the vector update), timed back to back on the solver stream with the current buffers
    double time_smoother(int reps);
    // event pairs around every level-0 Chebyshev step of the V-cycles (when enabled)
    LaunchTimer smoother_timer;
    // largest eigenvalue of D^-1 A on level 0 (the smoothing interval): refreshed when the
    // level-0 matrix changes under a kept hierarchy
    void set_level0_lambda(double lambda);
    // apply level 0 element by element over cell blocks (null operator: back to the SELL matrix)
    void set_level0_ebe(const EbeOperator* op);
    // level-0 element matrices streamed into a shared-memory ring by bulk copies (1) or loaded
    // by the warps that apply them (0, default: measured faster, see the design notes)
    void set_level0_stream(bool on) { stream_ke_ = on; }
    void set_level0_prefetch(int cells) { ebe_.prefetch = cells; }
    void set_level0_geo(const void* geo, int kind) {
        ebe_.geo = geo;
        ebe_.geo_kind = geo ? kind : 0;
    }
    // nonzero when a bounded wait of the streamed kernel ran out (the result is then invalid)
    unsigned level0_errors();
    bool level0_ebe() const { return ebe_on_; }
    // algorithmic bytes of one level-0 smoothing step (SELL: nnz*8 + 24 n; cell blocks: the
    // element matrices, the block tables, x per block-local DoF, the vectors, the partial sums)
    double smoother_bytes() const;
    // coarse-grid correction of level `level` by `cycles` stationary cycles of the next level
    // (1: V-cycle; 2 at level 0: two Q1 cycles per Q2 correction). Each further cycle starts
    // from the residual of the sum so far, so the preconditioner stays symmetric.
    void set_coarse_cycles(int level, int cycles);
    // Chebyshev degree and interval of one level's smoother (0: the hierarchy's own choice);
    // only the polynomial changes, nothing is rebuilt (the coarsest level is solved densely)
    void set_level_smoothing(int level, int degree, double lo);
    // prolongation P (rows of this level) and restriction R (rows of the next) of `level`,
    // built on the device in CSR with FP32 values; the hierarchy takes ownership
    void adopt_transfers(int level, DBuf<int64_t>&& p_ptr, DBuf<int32_t>&& p_col, DBuf<float>&& p_val,
                         DBuf<int64_t>&& r_ptr, DBuf<int32_t>&& r_col, DBuf<float>&& r_val, int64_t nnz);

private:
    void cycle(int l);
    void level0_apply(int kind, const float* xin, float* xout, float c1, float c2);  // 0 cheb, 1 residual
    EbeOperator ebe_;
    bool ebe_on_ = false;
    bool stream_ke_ = false;
    DBuf<unsigned> ebe_err_;
    int64_t nnz0_ = 0;
    cudaStream_t stream_;
    std::vector<std::unique_ptr<AmgDevLevel>> lv_;
    DBuf<float> coarse_inv_;
    int n_coarse_ = 0;
    std::vector<int> coarse_cycles_;
    std::string desc_;
};

}  // namespace fgb
