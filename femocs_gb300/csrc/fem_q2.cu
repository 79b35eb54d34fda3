// Q2 (27-node hexahedron) assembly on the device (sm_103a); structure from fem_q2_setup.cpp.
//
//   k_q2_cell_stiffness  K_e[i][j] = sum_q w_q |det J_q| grad N_i . grad N_j over 3x3x3 Gauss
//                        points on the trilinear (Q1) map of the hex, one warp per cell: lanes
//                        0..26 own the quadrature points for the Jacobians (FP64) and the nodes
//                        for the physical gradients, every lane accumulates 11-12 of the 378
//                        upper-triangle entries. Gradients and the ~31k products per cell are
//                        carried as FP32 hi/lo pairs with error-free products (FMA split) and
//                        sums (Knuth's TwoSum): ~2^-48 relative per operation, run on the FP32
//                        pipe (GB300's FP64 rate is 1/64 of FP32)
//   k_q2_assemble_rows   row-owned gather of the element matrices into the saved SELL-layout
//                        matrix, one warp per row: the row's columns in shared memory, one
//                        cell at a time, lanes 0..26 place the cell's 27 contributions by binary
//                        search (fixed order: deterministic)
//   k_q2_neumann_rows    3x3 Gauss on the bilinear top faces, biquadratic face shape functions
//   k_sell_dirichlet     symmetric elimination on the SELL layout (FP64 + FP32 copies, D^-1)
//   k_q2_geo             geometric factors w |det J| J^-1 J^-T per Gauss point for the
//                        matrix-free level-0 smoother (FP32 or FP16, block order)
// Lattice: node L = a + 3b + 9c at reference coordinates (a-1, b-1, c-1); 1-D quadratic
// Lagrange l0(t) = t(t-1)/2, l1(t) = 1 - t^2, l2(t) = t(t+1)/2.
#include <climits>
#include <cmath>
#include <mutex>

#include <cuda_fp16.h>

#include "fem_q2.h"
#include "dprim.cuh"

namespace fgb {

namespace {

constexpr int kQ2Warps = 4;  // warps (cells or rows) per 128-thread block

__constant__ double c_q2_dN[27 * 27 * 3];   // [qp][node][dir] reference gradients
__constant__ double c_q1_dN[27 * 8 * 3];    // [qp][corner][dir] trilinear-map gradients
__constant__ double c_q2_w[27];             // tensor Gauss weights
__constant__ unsigned char c_q2_ij[378 * 2];
__constant__ int c_q2_corner[8];            // lattice index of femocs corner k

const double kG3[3] = {-0.77459666924148337704, 0.0, 0.77459666924148337704};  // +-sqrt(3/5)
const double kW3[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
const int kHx[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
const int kHy[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
const int kHz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};

double l1d(int a, double t) { return a == 0 ? 0.5 * t * (t - 1.0) : (a == 1 ? 1.0 - t * t : 0.5 * t * (t + 1.0)); }
double dl1d(int a, double t) { return a == 0 ? t - 0.5 : (a == 1 ? -2.0 * t : t + 0.5); }

void upload_tables() {
    static std::once_flag once;
    static std::string err;
    std::call_once(once, [] {
        std::vector<double> dn(27 * 27 * 3), d1(27 * 8 * 3), w(27);
        for (int q = 0; q < 27; ++q) {
            const int qa = q % 3, qb = (q / 3) % 3, qc = q / 9;
            const double x = kG3[qa], y = kG3[qb], z = kG3[qc];
            w[q] = kW3[qa] * kW3[qb] * kW3[qc];
            for (int L = 0; L < 27; ++L) {
                const int a = L % 3, b = (L / 3) % 3, c = L / 9;
                dn[(q * 27 + L) * 3 + 0] = dl1d(a, x) * l1d(b, y) * l1d(c, z);
                dn[(q * 27 + L) * 3 + 1] = l1d(a, x) * dl1d(b, y) * l1d(c, z);
                dn[(q * 27 + L) * 3 + 2] = l1d(a, x) * l1d(b, y) * dl1d(c, z);
            }
            for (int k = 0; k < 8; ++k) {
                d1[(q * 8 + k) * 3 + 0] = 0.125 * kHx[k] * (1 + y * kHy[k]) * (1 + z * kHz[k]);
                d1[(q * 8 + k) * 3 + 1] = 0.125 * (1 + x * kHx[k]) * kHy[k] * (1 + z * kHz[k]);
                d1[(q * 8 + k) * 3 + 2] = 0.125 * (1 + x * kHx[k]) * (1 + y * kHy[k]) * kHz[k];
            }
        }
        unsigned char ij[378 * 2];
        int e = 0;
        for (int i = 0; i < 27; ++i)
            for (int j = i; j < 27; ++j, ++e) {
                ij[2 * e] = (unsigned char)i;
                ij[2 * e + 1] = (unsigned char)j;
            }
        int corner[8];
        for (int k = 0; k < 8; ++k) corner[k] = (kHx[k] + 1) + 3 * (kHy[k] + 1) + 9 * (kHz[k] + 1);
        cudaMemcpyToSymbol(c_q2_dN, dn.data(), sizeof(double) * dn.size());
        cudaMemcpyToSymbol(c_q1_dN, d1.data(), sizeof(double) * d1.size());
        cudaMemcpyToSymbol(c_q2_w, w.data(), sizeof(double) * w.size());
        cudaMemcpyToSymbol(c_q2_ij, ij, sizeof(ij));
        const cudaError_t rc = cudaMemcpyToSymbol(c_q2_corner, corner, sizeof(corner));
        if (rc != cudaSuccess) err = cudaGetErrorString(rc);
    });
    if (!err.empty()) throw Error("Q2 tables: " + err);
}

// index of (i, j) in the packed upper triangle of a 27x27 symmetric matrix
__device__ __forceinline__ int sym27(int i, int j) {
    if (i > j) { const int t = i; i = j; j = t; }
    return i * 27 - (i * (i - 1)) / 2 + (j - i);
}

// ---- FP32 hi/lo pairs (value = hi + lo, |lo| <= ulp(hi)/2); explicit _rn intrinsics so that
// no product or sum is ever contracted or reassociated
struct DF {
    float h, l;
};
__device__ __forceinline__ DF df_of(double x) {
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ DF df_norm(float s, float e) {  // Fast2Sum, |s| >= |e|
    const float h = __fadd_rn(s, e);
    return {h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ DF df_mul(DF a, DF b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);  // exact rounding error of the leading product
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return df_norm(p, e);
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
    float s, e;
    two_sum(a.h, b.h, s, e);
    e = __fadd_rn(e, __fadd_rn(a.l, b.l));
    return df_norm(s, e);
}

__global__ void __launch_bounds__(32 * kQ2Warps) k_q2_cell_stiffness(int nc, const int32_t* __restrict__ cd,
                                                                     const double* __restrict__ dxyz,
                                                                     double* __restrict__ ke) {
    __shared__ double sX[kQ2Warps][8][3];
    __shared__ DF sInv[kQ2Warps][27][10];  // J^-1 (row major) and w |det J| per point
    __shared__ DF sG[kQ2Warps][27][3];
    __shared__ DF sGw[kQ2Warps][27][3];    // w |det J| times the gradients
    // shape-gradient tables in shared memory: lanes read them at different addresses, which
    // the constant cache would serialise
    __shared__ DF sDN[27 * 27 * 3];
    __shared__ double sD1[27 * 8 * 3];
    for (int i = threadIdx.x; i < 27 * 27 * 3; i += blockDim.x) sDN[i] = df_of(c_q2_dN[i]);
    for (int i = threadIdx.x; i < 27 * 8 * 3; i += blockDim.x) sD1[i] = c_q1_dN[i];
    __syncthreads();
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = blockIdx.x * kQ2Warps + wid;
    if (c >= nc) return;  // whole warp leaves together
    if (lane < 8) {
        const int d = cd[27 * (size_t)c + c_q2_corner[lane]];
        sX[wid][lane][0] = dxyz[3 * (size_t)d];
        sX[wid][lane][1] = dxyz[3 * (size_t)d + 1];
        sX[wid][lane][2] = dxyz[3 * (size_t)d + 2];
    }
    __syncwarp();
    if (lane < 27) {
        double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int k = 0; k < 8; ++k)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) J[a][b] += sX[wid][k][a] * sD1[(lane * 8 + k) * 3 + b];
        const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        const double id = 1.0 / det;
        DF* o = sInv[wid][lane];
        o[0] = df_of(c00 * id);
        o[3] = df_of(c01 * id);
        o[6] = df_of(c02 * id);
        o[1] = df_of((J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id);
        o[4] = df_of((J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id);
        o[7] = df_of((J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id);
        o[2] = df_of((J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id);
        o[5] = df_of((J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id);
        o[8] = df_of((J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id);
        o[9] = df_of(c_q2_w[lane] * fabs(det));
    }
    DF acc[12];
    int ei[12], ej[12];  // this lane's packed entries e = lane + 32 t, held in registers (a
                         // table read per entry would diverge across the warp)
#pragma unroll
    for (int t = 0; t < 12; ++t) {
        acc[t] = {0.0f, 0.0f};
        const int e = min(lane + 32 * t, 377);
        ei[t] = c_q2_ij[2 * e];
        ej[t] = c_q2_ij[2 * e + 1];
    }
    for (int q = 0; q < 27; ++q) {
        __syncwarp();
        if (lane < 27) {
            const DF* inv = sInv[wid][q];
            const DF* g = sDN + (q * 27 + lane) * 3;
            // physical gradient: (J^-T g)_a = sum_k inv[k][a] g_k; the weight folded into one copy
            const DF w = inv[9];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const DF ga = df_add(df_add(df_mul(inv[a], g[0]), df_mul(inv[3 + a], g[1])), df_mul(inv[6 + a], g[2]));
                sG[wid][lane][a] = ga;
                sGw[wid][lane][a] = df_mul(w, ga);
            }
        }
        __syncwarp();
#pragma unroll
        for (int t = 0; t < 12; ++t) {
            const DF* gi = sGw[wid][ei[t]];
            const DF* gj = sG[wid][ej[t]];
            acc[t] = df_add(acc[t], df_mul(gi[0], gj[0]));
            acc[t] = df_add(acc[t], df_mul(gi[1], gj[1]));
            acc[t] = df_add(acc[t], df_mul(gi[2], gj[2]));
        }
    }
    double* o = ke + 378 * (size_t)c;
#pragma unroll
    for (int t = 0; t < 12; ++t) {
        const int e = lane + 32 * t;
        if (e < 378) o[e] = (double)acc[t].h + (double)acc[t].l;
    }
}

// one warp per row: gather the DoFs of the row's cells, bitonic sort (padded to a power of two
// with INT_MAX), then keep the first of each run of equal values
__global__ void __launch_bounds__(32) k_q2_sell_cols(int n, const int64_t* __restrict__ sptr,
                                                     const int32_t* __restrict__ slen, const int32_t* __restrict__ row_len,
                                                     const int32_t* __restrict__ r2c_ptr,
                                                     const int32_t* __restrict__ r2c_item,
                                                     const int32_t* __restrict__ cd, int32_t* __restrict__ scol,
                                                     int* __restrict__ bad) {
    extern __shared__ int32_t sc_buf[];
    const int lane = threadIdx.x;
    const int r = blockIdx.x;  // rows n.. only pad the last slice
    const int s = r >> 5, rl = r & 31;
    const int64_t base = sptr[s] + (int64_t)rl * 4;
    const int len_s = slen[s];
    int cnt = 0;
    if (r < n) {
        const int p0 = r2c_ptr[r], nc = r2c_ptr[r + 1] - p0;
        const int m = 27 * nc;
        int cap = 32;
        while (cap < m) cap <<= 1;
        for (int i = lane; i < cap; i += 32) {
            int v = INT_MAX;
            if (i < m) v = cd[27 * (size_t)(r2c_item[p0 + i / 27] / 27) + i % 27];
            sc_buf[i] = v;
        }
        __syncwarp();
        for (int k = 2; k <= cap; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = lane; i < cap; i += 32) {
                    const int ixj = i ^ j;
                    if (ixj > i) {
                        const int a = sc_buf[i], b = sc_buf[ixj];
                        const bool up = (i & k) == 0;
                        if ((a > b) == up) {
                            sc_buf[i] = b;
                            sc_buf[ixj] = a;
                        }
                    }
                }
                __syncwarp();
            }
        for (int b0 = 0; b0 < cap; b0 += 32) {
            const int i = b0 + lane;
            const int v = sc_buf[i];
            const bool keep = v != INT_MAX && (i == 0 || sc_buf[i - 1] != v);
            const unsigned msk = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                const int jj = cnt + __popc(msk & ((1u << lane) - 1u));
                if (jj < len_s) scol[base + (int64_t)(jj >> 2) * 128 + (jj & 3)] = v;
            }
            cnt += __popc(msk);
        }
        if (lane == 0 && cnt != row_len[r]) atomicAdd(bad, 1);
    }
    const int pad = r < n ? r : 0;
    for (int jj = (r < n ? cnt : 0) + lane; jj < len_s; jj += 32) scol[base + (int64_t)(jj >> 2) * 128 + (jj & 3)] = pad;
}

__global__ void __launch_bounds__(32 * kQ2Warps) k_q2_assemble_rows(int n, int max_len, const int64_t* __restrict__ sptr,
                                                                    const int32_t* __restrict__ scol,
                                                                    const int32_t* __restrict__ row_len,
                                                                    const int32_t* __restrict__ r2c_ptr,
                                                                    const int32_t* __restrict__ r2c_item,
                                                                    const int32_t* __restrict__ cd,
                                                                    const double* __restrict__ ke,
                                                                    double* __restrict__ kval) {
    extern __shared__ unsigned char q2_smem[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* vals = reinterpret_cast<double*>(q2_smem) + (size_t)wid * max_len;
    int32_t* cols = reinterpret_cast<int32_t*>(reinterpret_cast<double*>(q2_smem) + (size_t)kQ2Warps * max_len) +
                    (size_t)wid * max_len;
    const int r = blockIdx.x * kQ2Warps + wid;
    if (r >= n) return;  // whole warp leaves together
    const int len = row_len[r];
    const int64_t base = sptr[r >> 5] + (int64_t)(r & 31) * 4;
    for (int j = lane; j < len; j += 32) {
        cols[j] = scol[base + (int64_t)(j >> 2) * 128 + (j & 3)];
        vals[j] = 0.0;
    }
    __syncwarp();
    for (int p = r2c_ptr[r]; p < r2c_ptr[r + 1]; ++p) {
        const int item = r2c_item[p];
        const int c = item / 27, li = item - 27 * c;
        if (lane < 27) {
            const int cj = cd[27 * (size_t)c + lane];
            int lo = 0, hi = len - 1;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (cols[mid] < cj) lo = mid + 1; else hi = mid;
            }
            vals[lo] += ke[378 * (size_t)c + sym27(li, lane)];
        }
        __syncwarp();
    }
    for (int j = lane; j < len; j += 32) kval[base + (int64_t)(j >> 2) * 128 + (j & 3)] = vals[j];
}

__global__ void k_q2_neumann_rows(int n, const int32_t* __restrict__ r2f_ptr, const int32_t* __restrict__ r2f_item,
                                  const int32_t* __restrict__ top, const double* __restrict__ dxyz, double bc,
                                  const double* __restrict__ extra, double* __restrict__ rhs) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const double g3[3] = {-0.77459666924148337704, 0.0, 0.77459666924148337704};
    const double w3[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
    double acc = 0.0;
    for (int p = r2f_ptr[r]; p < r2f_ptr[r + 1]; ++p) {
        const int f = r2f_item[p] / 9, q = r2f_item[p] - 9 * (r2f_item[p] / 9);
        const int qu = q % 3, qv = q / 3;
        // corners (u,v) = (0,0), (2,0), (2,2), (0,2) of the face lattice
        const int cl[4] = {0, 2, 8, 6};
        double P[4][3];
        for (int k = 0; k < 4; ++k)
            for (int a = 0; a < 3; ++a) P[k][a] = dxyz[3 * (size_t)top[9 * (size_t)f + cl[k]] + a];
        for (int iv = 0; iv < 3; ++iv)
            for (int iu = 0; iu < 3; ++iu) {
                const double s = g3[iu], t = g3[iv];
                const double lu = qu == 0 ? 0.5 * s * (s - 1.0) : (qu == 1 ? 1.0 - s * s : 0.5 * s * (s + 1.0));
                const double lv = qv == 0 ? 0.5 * t * (t - 1.0) : (qv == 1 ? 1.0 - t * t : 0.5 * t * (t + 1.0));
                double ds[3], dt[3];
                for (int a = 0; a < 3; ++a) {
                    ds[a] = 0.25 * (-(1 - t) * P[0][a] + (1 - t) * P[1][a] + (1 + t) * P[2][a] - (1 + t) * P[3][a]);
                    dt[a] = 0.25 * (-(1 - s) * P[0][a] - (1 + s) * P[1][a] + (1 + s) * P[2][a] + (1 - s) * P[3][a]);
                }
                const double cx = ds[1] * dt[2] - ds[2] * dt[1], cy = ds[2] * dt[0] - ds[0] * dt[2],
                             cz = ds[0] * dt[1] - ds[1] * dt[0];
                acc += w3[iu] * w3[iv] * lu * lv * bc * sqrt(cx * cx + cy * cy + cz * cz);
            }
    }
    if (extra) acc += extra[r];
    rhs[r] = acc;
}

__device__ __forceinline__ bool fixed_kind(int8_t k, bool anode) { return k == 1 || (k == 2 && anode); }

__global__ void k_sell_dirichlet(int n, const int64_t* __restrict__ sptr, const int32_t* __restrict__ scol,
                                 const int32_t* __restrict__ row_len, const double* __restrict__ kval,
                                 const int8_t* __restrict__ bc, int anode, double v0, double* __restrict__ s64,
                                 float* __restrict__ s32, double* __restrict__ dinv64, float* __restrict__ dinv32,
                                 double* __restrict__ rhs, double* __restrict__ x) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int len = row_len[r];
    const int64_t base = sptr[r >> 5] + (int64_t)(r & 31) * 4;
    auto pos = [&](int j) { return base + (int64_t)(j >> 2) * 128 + (j & 3); };
    double diag = 1.0;
    for (int j = 0; j < len; ++j)
        if (scol[pos(j)] == r) diag = kval[pos(j)];
    if (fixed_kind(bc[r], anode)) {
        const double gr = bc[r] == 2 ? v0 : 0.0;
        for (int j = 0; j < len; ++j) {
            const int64_t q = pos(j);
            const double a = scol[q] == r ? kval[q] : 0.0;
            s64[q] = a;
            s32[q] = (float)a;
        }
        if (rhs) {
            rhs[r] = gr * diag;
            x[r] = gr;
        }
    } else {
        double acc = rhs ? rhs[r] : 0.0;
        for (int j = 0; j < len; ++j) {
            const int64_t q = pos(j);
            const int c = scol[q];
            double a = kval[q];
            if (fixed_kind(bc[c], anode)) {
                acc -= a * (bc[c] == 2 ? v0 : 0.0);
                a = 0.0;
            }
            s64[q] = a;
            s32[q] = (float)a;
        }
        if (rhs) rhs[r] = acc;
    }
    if (!rhs) return;  // values only: the right-hand side, x and D^-1 are already in place
    dinv64[r] = 1.0 / diag;
    dinv32[r] = (float)(1.0 / diag);
}

// r = b - A x of the eliminated system without the assembled matrix, in FP64, in two passes.
// Cells: y_e = K_e x_e, one warp per cell with the cell's 378 packed entries and its 27 x
// values (zero for fixed DoFs: their columns are zero in the eliminated matrix) staged in
// shared memory, lane i < 27 forming row i. Rows: r = b - the sum of the row's y entries over
// its cells (r2c order; item 27 c + L indexes y directly); a fixed row's residual is b - diag x.
__global__ void __launch_bounds__(32 * kQ2Warps) k_q2_cell_products(int nc, const int32_t* __restrict__ cd,
                                                                    const double* __restrict__ ke,
                                                                    const int8_t* __restrict__ fixed,
                                                                    const double* __restrict__ x,
                                                                    double* __restrict__ y) {
    __shared__ double sk[kQ2Warps][378];
    __shared__ double sx[kQ2Warps][27];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = blockIdx.x * kQ2Warps + wid;
    if (c >= nc) return;  // whole warp leaves together
    const double* K = ke + 378 * (size_t)c;
    for (int k = lane; k < 378; k += 32) sk[wid][k] = K[k];
    if (lane < 27) {
        const int d = cd[27 * (size_t)c + lane];
        sx[wid][lane] = fixed[d] ? 0.0 : x[d];
    }
    __syncwarp();
    if (lane < 27) {
        double acc = 0.0;
        for (int j = 0; j < 27; ++j) acc = fma(sk[wid][sym27(lane, j)], sx[wid][j], acc);
        y[27 * (size_t)c + lane] = acc;
    }
}

__global__ void k_q2_residual_rows(int n, const int32_t* __restrict__ r2c_ptr, const int32_t* __restrict__ r2c_item,
                                   const double* __restrict__ y, const int8_t* __restrict__ fixed,
                                   const double* __restrict__ dinv, const double* __restrict__ x,
                                   const double* __restrict__ b, double* __restrict__ r) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    if (fixed[row]) {
        r[row] = b[row] - x[row] / dinv[row];
        return;
    }
    double acc = 0.0;
    for (int p = r2c_ptr[row]; p < r2c_ptr[row + 1]; ++p) acc += y[r2c_item[p]];
    r[row] = b[row] - acc;
}

// The eliminated system's D^-1, right-hand side and x without the matrix, when every
// Dirichlet value is zero: the diagonal is the same sum of element-matrix diagonals, in the
// same cell order, as the assembled one (k_q2_assemble_rows); fixed rows get rhs = x = 0; the
// lift of the boundary values onto the free rows vanishes
__global__ void k_q2_dirichlet_zero(int n, const int32_t* __restrict__ r2c_ptr, const int32_t* __restrict__ r2c_item,
                                    const double* __restrict__ ke, const int8_t* __restrict__ bc, int anode,
                                    double* __restrict__ dinv64, float* __restrict__ dinv32, double* __restrict__ rhs,
                                    double* __restrict__ x) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double diag = 0.0;
    for (int p = r2c_ptr[r]; p < r2c_ptr[r + 1]; ++p) {
        const int item = r2c_item[p];
        const int c = item / 27, li = item - 27 * c;
        diag += ke[378 * (size_t)c + sym27(li, li)];
    }
    if (r2c_ptr[r] == r2c_ptr[r + 1]) diag = 1.0;
    if (fixed_kind(bc[r], anode)) {
        rhs[r] = 0.0;
        x[r] = 0.0;
    }
    dinv64[r] = 1.0 / diag;
    dinv32[r] = (float)(1.0 / diag);
}

// geometric factors of the cell-block smoother: thread (p, q) takes cell perm[p], its corners
// relative to corner 0 (FP64 differences, then FP32), J_q of the trilinear map, and writes
// C_q = w_q |det J_q| J_q^-1 J_q^-T as pairs m = (C00, C11), (C22, C01), (C02, C12) at
// [81 p + 9 (3 qx + m) + qy + 3 qz] (q = qx + 3 qy + 9 qz; the smoother's lane for pencil
// (qy, qz) reads its three Gauss points' pairs 9 apart), in FP32 (T = float2) or FP16 (T = __half2; the largest |entry| is kept
// in *cmax as float bits so that the host can refuse values beyond the FP16 range)
template <typename T>
__global__ void k_q2_geo(long long total, const int32_t* __restrict__ perm, const int32_t* __restrict__ cd,
                         const double* __restrict__ dxyz, T* __restrict__ out, unsigned* __restrict__ cmax) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const long long p = idx / 27;
    const int q = (int)(idx - 27 * p);
    const int32_t* c = cd + 27 * (size_t)perm[p];
    const double* x0 = dxyz + 3 * (size_t)c[c_q2_corner[0]];
    float J[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    for (int k = 1; k < 8; ++k) {  // corner 0 contributes nothing relative to itself
        const double* xk = dxyz + 3 * (size_t)c[c_q2_corner[k]];
        for (int a = 0; a < 3; ++a) {
            const float xa = (float)(xk[a] - x0[a]);
            for (int b = 0; b < 3; ++b) J[a][b] = fmaf(xa, (float)c_q1_dN[(q * 8 + k) * 3 + b], J[a][b]);
        }
    }
    // adjugate rows: J^-1 = adj / det
    float A[3][3];
    A[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    A[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    A[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    A[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    A[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    A[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
    A[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    A[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
    A[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const float det = J[0][0] * A[0][0] + J[0][1] * A[1][0] + J[0][2] * A[2][0];
    const float s = (float)c_q2_w[q] / fabsf(det);
    auto C = [&](int r, int t) { return s * (A[r][0] * A[t][0] + A[r][1] * A[t][1] + A[r][2] * A[t][2]); };
    const float v[6] = {C(0, 0), C(1, 1), C(2, 2), C(0, 1), C(0, 2), C(1, 2)};
    T* o = out + 81 * (size_t)p + 27 * (q % 3) + q / 3;
    if constexpr (sizeof(T) == sizeof(float2)) {
        for (int m = 0; m < 3; ++m) o[9 * m] = make_float2(v[2 * m], v[2 * m + 1]);
    } else {
        float mx = 0.f;
        for (int m = 0; m < 6; ++m) mx = fmaxf(mx, fabsf(v[m]));
        if (!(mx <= 3.0e38f)) mx = 3.0e38f;  // NaN or inf: report as out of range
        atomicMax(cmax, __float_as_uint(mx));
        for (int m = 0; m < 3; ++m) o[9 * m] = __floats2half2_rn(v[2 * m], v[2 * m + 1]);
    }
}

// lattice corners of each local node's entity (1, 2, 4 or 8) as a by-value kernel argument
struct CornerTab {
    int8_t c[27][8];
    int8_t n[27];
};

// one Q2 DoF per thread: count pass (ptr == nullptr: cnt[d] = entries of row d) or fill pass
__global__ void k_embed_rows(int n, const int32_t* __restrict__ dof_cell, const int8_t* __restrict__ dof_local,
                             const int32_t* __restrict__ cq1, const int8_t* __restrict__ fixed2,
                             const int8_t* __restrict__ fixed1, CornerTab tab, const int64_t* __restrict__ ptr,
                             int64_t* __restrict__ cnt, int32_t* __restrict__ col, float* __restrict__ val,
                             int32_t* __restrict__ rowof) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    int m = 0;
    if (!fixed2[d]) {
        const int L = dof_local[d];
        const int64_t c = dof_cell[d];
        const int nk = tab.n[L];
        for (int q = 0; q < nk; ++q) {
            const int v = cq1[8 * c + tab.c[L][q]];
            if (v >= 0 && !fixed1[v]) {
                if (ptr) {
                    const int64_t k = ptr[d] + m;
                    col[k] = v;
                    val[k] = 1.f / (float)nk;  // nk is 1, 2, 4 or 8: exact
                    rowof[k] = d;
                }
                ++m;
            }
        }
    }
    if (!ptr) cnt[d] = m;
}

__global__ void k_iota32(int64_t n, int32_t* __restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (int32_t)i;
}

__global__ void k_count_cols(int64_t n, const int32_t* __restrict__ col, int64_t* __restrict__ cnt) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(reinterpret_cast<unsigned long long*>(cnt + col[i]), 1ull);
}

// R entry j: the P entry idx[j] (sorted by column, ascending P position within a column)
__global__ void k_transpose_fill(int64_t n, const int32_t* __restrict__ idx, const int32_t* __restrict__ rowof,
                                 const float* __restrict__ pval, int32_t* __restrict__ rcol, float* __restrict__ rval) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int32_t k = idx[j];
    rcol[j] = rowof[k];
    rval[j] = pval[k];
}

}  // namespace

void q2_geometric_factors(long long n_pos, const int32_t* perm, const int32_t* cell_dofs, const double* dof_xyz,
                          void* out, bool half, unsigned* cmax, cudaStream_t s) {
    upload_tables();
    const long long total = 27 * n_pos;
    if (half) {
        FGB_CUDA(cudaMemsetAsync(cmax, 0, sizeof(unsigned), s));
        FGB_LAUNCH(k_q2_geo<__half2><<<grid_for(total, 256), 256, 0, s>>>(total, perm, cell_dofs, dof_xyz,
                                                                         static_cast<__half2*>(out), cmax));
    } else {
        FGB_LAUNCH(k_q2_geo<float2><<<grid_for(total, 256), 256, 0, s>>>(total, perm, cell_dofs, dof_xyz,
                                                                        static_cast<float2*>(out), cmax));
    }
}

void q2_cell_stiffness(int nc, const int32_t* cd, const double* dxyz, double* ke, cudaStream_t s) {
    upload_tables();
    FGB_LAUNCH(k_q2_cell_stiffness<<<grid_for(nc, kQ2Warps), 32 * kQ2Warps, 0, s>>>(nc, cd, dxyz, ke));
}

int q2_sell_columns(int n, int n_slices, const int64_t* sptr, const int32_t* slen, const int32_t* row_len,
                    const int32_t* r2c_ptr, const int32_t* r2c_item, const int32_t* cell_dofs, int max_cells,
                    int32_t* scol, cudaStream_t s) {
    int cap = 32;
    while (cap < 27 * max_cells) cap <<= 1;
    const size_t smem = sizeof(int32_t) * (size_t)cap;
    FGB_REQUIRE(smem <= 227 * 1024, "a Q2 row has too many cells for the shared-memory sort");
    if (smem > 48 * 1024)
        FGB_CUDA(cudaFuncSetAttribute(k_q2_sell_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    DBuf<int> bad(1);
    bad.zero(s);
    FGB_LAUNCH(k_q2_sell_cols<<<32 * n_slices, 32, smem, s>>>(n, sptr, slen, row_len, r2c_ptr, r2c_item, cell_dofs,
                                                              scol, bad.get()));
    FGB_CUDA(cudaGetLastError());
    int h = 0;
    FGB_CUDA(cudaMemcpyAsync(&h, bad.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
    FGB_CUDA(cudaStreamSynchronize(s));
    return h;
}

void q2_assemble_rows(int n, int max_len, const int64_t* sptr, const int32_t* scol, const int32_t* row_len,
                      const int32_t* r2c_ptr, const int32_t* r2c_item, const int32_t* cd, const double* ke, double* kval,
                      cudaStream_t s) {
    const size_t smem = (size_t)kQ2Warps * max_len * (sizeof(double) + sizeof(int32_t));
    static std::once_flag attr;
    std::call_once(attr, [] {
        cudaFuncSetAttribute(k_q2_assemble_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    });
    FGB_REQUIRE(smem <= 200 * 1024, "Q2 rows too long for the shared-memory assembly");
    FGB_LAUNCH(k_q2_assemble_rows<<<grid_for(n, kQ2Warps), 32 * kQ2Warps, smem, s>>>(n, max_len, sptr, scol, row_len,
                                                                                    r2c_ptr, r2c_item, cd, ke, kval));
}

void q2_neumann_rows(int n, const int32_t* r2f_ptr, const int32_t* r2f_item, const int32_t* top, const double* dxyz,
                     double bc, const double* extra, double* rhs, cudaStream_t s) {
    FGB_LAUNCH(k_q2_neumann_rows<<<grid_for(n, 256), 256, 0, s>>>(n, r2f_ptr, r2f_item, top, dxyz, bc, extra, rhs));
}

void sell_dirichlet(int n, const int64_t* sptr, const int32_t* scol, const int32_t* row_len, const double* kval,
                    const int8_t* bc, int anode, double v0, double* s64, float* s32, double* dinv64, float* dinv32,
                    double* rhs, double* x, cudaStream_t s) {
    FGB_LAUNCH(k_sell_dirichlet<<<grid_for(n, 256), 256, 0, s>>>(n, sptr, scol, row_len, kval, bc, anode, v0, s64, s32,
                                                                 dinv64, dinv32, rhs, x));
}

void q2_residual_cells(int n, int nc, const int32_t* r2c_ptr, const int32_t* r2c_item, const int32_t* cd,
                       const double* ke, const int8_t* fixed, const double* dinv, const double* x, const double* b,
                       double* y, double* r, cudaStream_t s) {
    if (nc) FGB_LAUNCH(k_q2_cell_products<<<(nc + kQ2Warps - 1) / kQ2Warps, 32 * kQ2Warps, 0, s>>>(nc, cd, ke, fixed, x, y));
    if (n) FGB_LAUNCH(k_q2_residual_rows<<<grid_for(n, 256), 256, 0, s>>>(n, r2c_ptr, r2c_item, y, fixed, dinv, x, b, r));
}

void q2_dirichlet_zero(int n, const int32_t* r2c_ptr, const int32_t* r2c_item, const double* ke, const int8_t* bc,
                       int anode, double* dinv64, float* dinv32, double* rhs, double* x, cudaStream_t s) {
    FGB_LAUNCH(k_q2_dirichlet_zero<<<grid_for(n, 256), 256, 0, s>>>(n, r2c_ptr, r2c_item, ke, bc, anode, dinv64, dinv32,
                                                                    rhs, x));
}

void q2_embedding(int n, int n1, const int32_t* dof_cell, const int8_t* dof_local, const int32_t* cq1,
                  const int8_t* fixed2, const int8_t* fixed1, DeviceCsr32& P, DeviceCsr32& R, cudaStream_t s) {
    CornerTab tab;
    for (int L = 0; L < 27; ++L) {
        int cr[8];
        const int nk = q2_entity_corners(L, cr);
        tab.n[L] = (int8_t)nk;
        for (int q = 0; q < 8; ++q) tab.c[L][q] = (int8_t)(q < nk ? cr[q] : 0);
    }
    const int nb = 256;
    // P: row counts, their scan, the fill
    P.n_rows = n;
    P.n_cols = n1;
    P.ptr.resize((size_t)n + 1);
    {
        dprim::SBuf<int64_t> cnt((size_t)n + 1, s);
        FGB_CUDA(cudaMemsetAsync(cnt.get() + n, 0, sizeof(int64_t), s));
        if (n) FGB_LAUNCH(k_embed_rows<<<(n + nb - 1) / nb, nb, 0, s>>>(n, dof_cell, dof_local, cq1, fixed2, fixed1, tab,
                                                                       nullptr, cnt.get(), nullptr, nullptr, nullptr));
        P.nnz = dprim::exclusive_scan_total<int64_t>(cnt.get(), P.ptr.get(), (int64_t)n + 1, s);
    }
    FGB_REQUIRE(P.nnz < (int64_t)INT32_MAX, "Q2 embedding: too many entries");
    const int64_t nz = P.nnz;
    P.col.resize(std::max<int64_t>(nz, 1));
    P.val.resize(std::max<int64_t>(nz, 1));
    dprim::SBuf<int32_t> rowof(std::max<int64_t>(nz, 1), s);
    if (n) FGB_LAUNCH(k_embed_rows<<<(n + nb - 1) / nb, nb, 0, s>>>(n, dof_cell, dof_local, cq1, fixed2, fixed1, tab,
                                                                   P.ptr.get(), nullptr, P.col.get(), P.val.get(),
                                                                   rowof.get()));
    // R = P^T: the entries sorted by column with a stable radix sort (so ascending P position,
    // i.e. ascending row, within a column), row pointers from per-column counts
    R.n_rows = n1;
    R.n_cols = n;
    R.nnz = nz;
    R.ptr.resize((size_t)n1 + 1);
    R.col.resize(std::max<int64_t>(nz, 1));
    R.val.resize(std::max<int64_t>(nz, 1));
    {
        dprim::SBuf<int64_t> cnt((size_t)n1 + 1, s);
        cnt.fill_bytes(0);
        const unsigned g = (unsigned)((nz + nb - 1) / nb);
        if (nz) FGB_LAUNCH(k_count_cols<<<g, nb, 0, s>>>(nz, P.col.get(), cnt.get()));
        dprim::exclusive_scan<int64_t>(cnt.get(), R.ptr.get(), (int64_t)n1 + 1, nullptr, s);
        if (nz) {
            dprim::SBuf<uint32_t> keys(nz, s);
            dprim::SBuf<int32_t> idx(nz, s);
            FGB_CUDA(cudaMemcpyAsync(keys.get(), P.col.get(), sizeof(int32_t) * nz, cudaMemcpyDeviceToDevice, s));
            FGB_LAUNCH(k_iota32<<<g, nb, 0, s>>>(nz, idx.get()));
            dprim::radix_sort<uint32_t>(keys, &idx, nz, dprim::bits_for((uint64_t)std::max(1, n1 - 1)), s);
            FGB_LAUNCH(k_transpose_fill<<<g, nb, 0, s>>>(nz, idx.get(), rowof.get(), P.val.get(), R.col.get(), R.val.get()));
        }
    }
    FGB_CUDA(cudaStreamSynchronize(s));
}

}  // namespace fgb
