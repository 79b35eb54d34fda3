// Launchers of the Q2 assembly kernels (fem_q2.cu); the structure is built by
// build_q2_structure (fem_q2_setup.cpp).
#pragma once

#include "device.h"
#include "fem.h"

namespace fgb {

// 378 packed upper-triangle entries per cell
void q2_cell_stiffness(int nc, const int32_t* cell_dofs, const double* dof_xyz, double* ke, cudaStream_t s);
// the same 378 entries per cell on the tensor cores (q2_ke_tc.cu): per-point factors in
// double-float arithmetic, error-free BF16 slices, tcgen05 products with FP32 accumulators in
// tensor memory, levels combined into FP64; scratch (per persistent CTA) and err are the
// caller's reusable buffers
void q2_cell_stiffness_tc(int nc, const int32_t* cell_dofs, const double* dof_xyz, double* ke,
                          DBuf<unsigned char>& scratch, DBuf<unsigned>& err, cudaStream_t s);
// geometric factors of the matrix-free level-0 smoother, block order (position p = cell
// perm[p]): 81 pairs per position, FP32 (float2) or FP16 (half2); with half, *cmax (device)
// receives the largest |entry| as float bits
void q2_geometric_factors(long long n_pos, const int32_t* perm, const int32_t* cell_dofs, const double* dof_xyz,
                          void* out, bool half, unsigned* cmax, cudaStream_t s);
// one 128 x 48 x 32 BF16 tensor-core product of small integers on the device against the
// host's: the largest absolute difference (0 when descriptors and TMEM layout are right)
double tc_selftest();
// SELL-32 columns of the Q2 rows: per row the sorted, unique DoFs of its cells (one warp per
// row, bitonic sort in shared memory); padding = the row itself (0 past the last row).
// max_cells = the longest row -> cell list. Returns the number of rows whose column count
// differed from row_len (0 when the structure is consistent).
int q2_sell_columns(int n, int n_slices, const int64_t* sptr, const int32_t* slen, const int32_t* row_len,
                    const int32_t* r2c_ptr, const int32_t* r2c_item, const int32_t* cell_dofs, int max_cells,
                    int32_t* scol, cudaStream_t s);
// saved (pre-Dirichlet) matrix in the SELL layout of the structure
void q2_assemble_rows(int n, int max_len, const int64_t* sptr, const int32_t* scol, const int32_t* row_len,
                      const int32_t* r2c_ptr, const int32_t* r2c_item, const int32_t* cell_dofs, const double* ke,
                      double* kval, cudaStream_t s);
void q2_neumann_rows(int n, const int32_t* r2f_ptr, const int32_t* r2f_item, const int32_t* top, const double* dof_xyz,
                     double bc, const double* extra, double* rhs, cudaStream_t s);
// CSR matrix with FP32 values on the device
struct DeviceCsr32 {
    DBuf<int64_t> ptr;
    DBuf<int32_t> col;
    DBuf<float> val;
    int n_rows = 0, n_cols = 0;
    int64_t nnz = 0;
};
// Q2 -> Q1 embedding on the device: row d of P holds the free Q1 DoFs at the corners of the
// entity of Q2 DoF d (corners in the lattice order of its cell dof_cell[d], weight
// 1 / #corners); rows of fixed Q2 DoFs are empty. cq1 = the Q1 DoF of each cell corner (8 per
// cell, -1: none). R = P^T with each row in ascending P-row order.
void q2_embedding(int n, int n1, const int32_t* dof_cell, const int8_t* dof_local, const int32_t* cq1,
                  const int8_t* fixed2, const int8_t* fixed1, DeviceCsr32& P, DeviceCsr32& R, cudaStream_t s);
// symmetric Dirichlet elimination on a SELL-layout matrix (any element order); rhs == nullptr
// writes the eliminated values s64/s32 only (rhs, x and D^-1 untouched)
void sell_dirichlet(int n, const int64_t* sptr, const int32_t* scol, const int32_t* row_len, const double* kval,
                    const int8_t* bc, int anode, double v0, double* s64, float* s32, double* dinv64, float* dinv32,
                    double* rhs, double* x, cudaStream_t s);
// r = b - A x of the eliminated Q2 system from the FP64 element matrices (no assembled
// matrix): y (27 per cell, scratch) = K_e x_e per cell, then per row the sum over its cells
void q2_residual_cells(int n, int nc, const int32_t* r2c_ptr, const int32_t* r2c_item, const int32_t* cd,
                       const double* ke, const int8_t* fixed, const double* dinv, const double* x, const double* b,
                       double* y, double* r, cudaStream_t s);
// D^-1, right-hand side and x of the eliminated Q2 system when every Dirichlet value is zero,
// without the matrix: the diagonal from the element matrices in the assembled summation order
void q2_dirichlet_zero(int n, const int32_t* r2c_ptr, const int32_t* r2c_item, const double* ke, const int8_t* bc,
                       int anode, double* dinv64, float* dinv32, double* rhs, double* x, cudaStream_t s);

}  // namespace fgb
