// Device assembly and CG solvers of the vacuum Poisson system (sm_103a).
//
//   k_cell_stiffness   Q1 element matrices, 2x2x2 Gauss, trilinear map
//                      (PoissonSolver::assemble_local_cell, src/PoissonSolver.cpp:239-263)
//   k_assemble_rows    deterministic row-owned scatter of the element matrices into CSR
//                      (DealSolver::copy_global_cell, src/DealSolver.cpp:65-72)
//   k_neumann_rows     2x2 Gauss face integral of the applied field on the top faces
//                      (DealSolver::assemble_rhs, src/DealSolver.cpp:390-430)
//   k_dirichlet_rows   symmetric elimination of the copper (and anode) values, writes the
//                      SELL-32 FP64/FP32 matrices and the Jacobi diagonal
//                      (MatrixTools::apply_boundary_values via src/DealSolver.cpp:433-440)
//   k_sell_spmv        y = A x, SELL-32, one row per thread, coalesced value/column streams
//   k_cg_*             fused Jacobi-PCG iteration (SpMV+dot, update+dots, direction), all
//                      scalars in device memory, replayed from a CUDA graph
//   mixed precision    FP32 inner PCG inside FP64 iterative refinement; the true residual,
//                      the refinement update and the boundary values stay FP64
//   k_pcg_*, k_cg_spmv_pq_df, k_cb_spmv_df
//                      FP64 CG preconditioned by the FP32 multigrid V-cycle (amg.cu), its
//                      A p FP64-accurate from FP32 pairs: the SELL matrix, or for Q2 the
//                      element matrices over the cell blocks (cell_blocks.h)
//   k_ke_cyclic        Q2 element matrices into the cell blocks' FP32 (hi, lo) layout
#include <algorithm>
#include <mutex>
#include <cstring>
#include <chrono>
#include <omp.h>
#include <cstdlib>
#include <cmath>

#include "amg.h"
#include "compensated.cuh"
#include "fem_device.h"
#include "cell_blocks.h"
#include "fem_q2.h"

namespace fgb {

struct FemDevice::CellBlocksDev {
    int n_blocks = 0, max_cells = 0, max_dofs = 0, n_bnd = 0, n_slots = 0;
    int64_t n_local = 0;
    DBuf<int32_t> perm, cell_start, dof_start, dof_list, slot, bnd_dofs, bnd_ptr;
    DBuf<uint16_t> item_end, loc, items;
    DBuf<float> partial;
};

std::atomic<long long> g_kernel_launches{0};

void d2h_staged(void* dst, const void* src, size_t bytes, cudaStream_t s) {
    constexpr size_t kChunk = size_t(32) << 20;
    static std::mutex mu;
    static unsigned char* stage[2] = {nullptr, nullptr};
    static cudaEvent_t done[2];
    std::lock_guard<std::mutex> lk(mu);
    if (!stage[0])
        for (int k = 0; k < 2; ++k) {
            FGB_CUDA(cudaMallocHost(&stage[k], kChunk));
            FGB_CUDA(cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming));
        }
    const unsigned char* in = static_cast<const unsigned char*>(src);
    unsigned char* out = static_cast<unsigned char*>(dst);
    const size_t n_chunks = (bytes + kChunk - 1) / kChunk;
    auto issue = [&](size_t c) {
        const size_t off = c * kChunk, len = std::min(kChunk, bytes - off);
        FGB_CUDA(cudaMemcpyAsync(stage[c & 1], in + off, len, cudaMemcpyDeviceToHost, s));
        FGB_CUDA(cudaEventRecord(done[c & 1], s));
    };
    if (n_chunks) issue(0);
    for (size_t c = 0; c < n_chunks; ++c) {
        if (c + 1 < n_chunks) issue(c + 1);  // the next chunk travels while this one is copied out
        FGB_CUDA(cudaEventSynchronize(done[c & 1]));
        const size_t off = c * kChunk, len = std::min(kChunk, bytes - off);
        const long long parts = (long long)((len + (size_t(1) << 20) - 1) >> 20);
#pragma omp parallel for schedule(static)
        for (long long q = 0; q < parts; ++q) {
            const size_t a = (size_t)q << 20, b = std::min(len, a + (size_t(1) << 20));
            std::memcpy(out + off + a, stage[c & 1] + a, b - a);
        }
    }
}

void h2d_staged(void* dst, const void* src, size_t bytes, cudaStream_t s) {
    constexpr size_t kChunk = size_t(32) << 20;
    static std::mutex mu;
    static unsigned char* stage[2] = {nullptr, nullptr};
    static cudaEvent_t done[2];
    std::lock_guard<std::mutex> lk(mu);
    if (!stage[0]) {
        for (int k = 0; k < 2; ++k) {
            FGB_CUDA(cudaMallocHost(&stage[k], kChunk));
            FGB_CUDA(cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming));
            FGB_CUDA(cudaEventRecord(done[k], s));
        }
    }
    const unsigned char* in = static_cast<const unsigned char*>(src);
    unsigned char* out = static_cast<unsigned char*>(dst);
    int k = 0;
    for (size_t off = 0; off < bytes; off += kChunk, k ^= 1) {
        const size_t len = std::min(kChunk, bytes - off);
        FGB_CUDA(cudaEventSynchronize(done[k]));  // the DMA that last read this buffer is done
        const long long parts = (long long)((len + (size_t(1) << 20) - 1) >> 20);
#pragma omp parallel for schedule(static)
        for (long long q = 0; q < parts; ++q) {
            const size_t a = (size_t)q << 20, b = std::min(len, a + (size_t(1) << 20));
            std::memcpy(stage[k] + a, in + off + a, b - a);
        }
        FGB_CUDA(cudaMemcpyAsync(out + off, stage[k], len, cudaMemcpyHostToDevice, s));
        FGB_CUDA(cudaEventRecord(done[k], s));
    }
}

namespace {

constexpr int kBlock = 256;
constexpr int kProfiledLaunches = 512;  // timing events created ahead per solve (grow on demand)
__constant__ double c_hx[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
__constant__ double c_hy[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
__constant__ double c_hz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};

// ng = Gauss points per direction: 2 (the reference's QGauss<3>(2)) or 3 (the Q1 operator of
// the Q2 coarse level: the exact Galerkin product P^T A_Q2 P, whose integrals use 3 points)
__global__ void __launch_bounds__(128) k_cell_stiffness(int nc, const int32_t* __restrict__ cd,
                                                        const double* __restrict__ dxyz, double* __restrict__ ke,
                                                        int ng) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    double X[8][3];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int d = cd[8 * (size_t)c + k];
        X[k][0] = dxyz[3 * (size_t)d];
        X[k][1] = dxyz[3 * (size_t)d + 1];
        X[k][2] = dxyz[3 * (size_t)d + 2];
    }
    double K[36];
#pragma unroll
    for (int i = 0; i < 36; ++i) K[i] = 0.0;
    const double g = 0.57735026918962576451;
    const double g3[3] = {-0.77459666924148337704, 0.0, 0.77459666924148337704};
    const double w3[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
    const int nq = ng == 3 ? 27 : 8;
#pragma unroll 1
    for (int q = 0; q < nq; ++q) {
        double xi, eta, zeta, wq = 1.0;
        if (ng == 3) {
            xi = g3[q % 3];
            eta = g3[(q / 3) % 3];
            zeta = g3[q / 9];
            wq = w3[q % 3] * w3[(q / 3) % 3] * w3[q / 9];
        } else {
            xi = (q & 1) ? g : -g;
            eta = (q & 2) ? g : -g;
            zeta = (q & 4) ? g : -g;
        }
        double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        double dN[8][3];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const double ax = c_hx[k], ay = c_hy[k], az = c_hz[k];
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
        // inv = J^-1 (inv[i][j] = (J^-1)_ij); grad_x N = J^-T grad_xi N
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
#pragma unroll
        for (int k = 0; k < 8; ++k)
#pragma unroll
            for (int a = 0; a < 3; ++a)
                G[k][a] = inv[0][a] * dN[k][0] + inv[1][a] * dN[k][1] + inv[2][a] * dN[k][2];
        const double w = wq * fabs(det);
        int t = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = i; j < 8; ++j, ++t)
                K[t] += w * (G[i][0] * G[j][0] + G[i][1] * G[j][1] + G[i][2] * G[j][2]);
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
}

__global__ void k_assemble_rows(int n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                const int32_t* __restrict__ r2c_ptr, const int32_t* __restrict__ r2c_item,
                                const int32_t* __restrict__ cd, const double* __restrict__ ke, double* __restrict__ kval) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int64_t b = rowptr[r], e = rowptr[r + 1];
    for (int64_t k = b; k < e; ++k) kval[k] = 0.0;
    for (int p = r2c_ptr[r]; p < r2c_ptr[r + 1]; ++p) {
        const int item = r2c_item[p];
        const int c = item >> 3, loc = item & 7;
        const double* kr = ke + 64 * (size_t)c + 8 * loc;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int cj = cd[8 * (size_t)c + j];
            int64_t lo = b, hi = e - 1;
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (col[mid] < cj) lo = mid + 1; else hi = mid;
            }
            kval[lo] += kr[j];
        }
    }
}

// Neumann rows; the face value is `bc`, or fvals[face] when per-face values are given
__global__ void k_neumann_rows(int n, const int32_t* __restrict__ r2f_ptr, const int32_t* __restrict__ r2f_item,
                               const int32_t* __restrict__ top, const double* __restrict__ dxyz, double bc,
                               const double* __restrict__ fvals, const double* __restrict__ extra,
                               double* __restrict__ rhs) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double acc = 0.0;
    const double g = 0.57735026918962576451;
    for (int p = r2f_ptr[r]; p < r2f_ptr[r + 1]; ++p) {
        const int f = r2f_item[p] >> 2, q = r2f_item[p] & 3;
        double P[4][3];
        for (int k = 0; k < 4; ++k)
            for (int a = 0; a < 3; ++a) P[k][a] = dxyz[3 * (size_t)top[4 * (size_t)f + k] + a];
        for (int qp = 0; qp < 4; ++qp) {
            const double s = (qp & 1) ? g : -g, t = (qp & 2) ? g : -g;
            const double N[4] = {0.25 * (1 - s) * (1 - t), 0.25 * (1 + s) * (1 - t), 0.25 * (1 + s) * (1 + t),
                                 0.25 * (1 - s) * (1 + t)};
            double ds[3], dt[3];
            for (int a = 0; a < 3; ++a) {
                ds[a] = 0.25 * (-(1 - t) * P[0][a] + (1 - t) * P[1][a] + (1 + t) * P[2][a] - (1 + t) * P[3][a]);
                dt[a] = 0.25 * (-(1 - s) * P[0][a] - (1 + s) * P[1][a] + (1 + s) * P[2][a] + (1 - s) * P[3][a]);
            }
            const double cx = ds[1] * dt[2] - ds[2] * dt[1], cy = ds[2] * dt[0] - ds[0] * dt[2],
                         cz = ds[0] * dt[1] - ds[1] * dt[0];
            acc += N[q] * (fvals ? fvals[f] : bc) * sqrt(cx * cx + cy * cy + cz * cz);
        }
    }
    if (extra) acc += extra[r];
    rhs[r] = acc;
}

__device__ __forceinline__ bool is_fixed(int8_t k, bool anode) { return k == 1 || (k == 2 && anode); }

// symmetric elimination; rows of kind 1 take the value v1, of kind 2 (anode Dirichlet) v0
__global__ void k_dirichlet_rows(int n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                 const double* __restrict__ kval, const int8_t* __restrict__ bc, int anode, double v0,
                                 double v1,
                                 const int64_t* __restrict__ csr2sell, double* __restrict__ s64, float* __restrict__ s32,
                                 double* __restrict__ dinv64, float* __restrict__ dinv32, double* __restrict__ rhs,
                                 double* __restrict__ x) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int64_t b = rowptr[r], e = rowptr[r + 1];
    double diag = 1.0;
    for (int64_t k = b; k < e; ++k)
        if (col[k] == r) diag = kval[k];
    const bool fr = is_fixed(bc[r], anode);
    if (fr) {
        const double gr = bc[r] == 2 ? v0 : v1;
        for (int64_t k = b; k < e; ++k) {
            const double a = col[k] == r ? kval[k] : 0.0;
            s64[csr2sell[k]] = a;
            s32[csr2sell[k]] = (float)a;
        }
        rhs[r] = gr * diag;
        x[r] = gr;
    } else {
        double acc = rhs[r];
        for (int64_t k = b; k < e; ++k) {
            const int c = col[k];
            double a = kval[k];
            if (is_fixed(bc[c], anode)) {
                const double gc = bc[c] == 2 ? v0 : v1;
                acc -= a * gc;
                a = 0.0;
            }
            s64[csr2sell[k]] = a;
            s32[csr2sell[k]] = (float)a;
        }
        rhs[r] = acc;
    }
    dinv64[r] = 1.0 / diag;
    dinv32[r] = (float)(1.0 / diag);
}

// ---------------------------------------------------------------- SpMV / CG
// y_r of a SELL-32 matrix with 4-wide row chunks (see fem_setup.cpp): per chunk one 16-byte
// column load, one 16/32-byte value load and four gathers; two chunks in flight.
template <typename T>
struct Vec4Of;
template <>
struct Vec4Of<float> {
    __device__ __forceinline__ static void load(const float* p, float (&v)[4]) {
        const float4 q = __ldg(reinterpret_cast<const float4*>(p));
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    }
};
template <>
struct Vec4Of<double> {
    __device__ __forceinline__ static void load(const double* p, double (&v)[4]) {
        const double2 a = __ldg(reinterpret_cast<const double2*>(p));
        const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    }
};

template <typename T>
__device__ __forceinline__ T sell_row(int r, const int64_t* __restrict__ sptr, const int32_t* __restrict__ slen,
                                      const int32_t* __restrict__ scol, const T* __restrict__ sval,
                                      const T* __restrict__ x) {
    const int s = r >> 5;
    const int64_t base = sptr[s] + (int64_t)(r & 31) * 4;
    const int nch = slen[s] >> 2;
    T a0 = 0, a1 = 0;
    int c = 0;
    for (; c + 1 < nch; c += 2) {
        const int64_t o0 = base + (int64_t)c * 128, o1 = o0 + 128;
        const int4 i0 = __ldg(reinterpret_cast<const int4*>(scol + o0));
        const int4 i1 = __ldg(reinterpret_cast<const int4*>(scol + o1));
        T v0[4], v1[4];
        Vec4Of<T>::load(sval + o0, v0);
        Vec4Of<T>::load(sval + o1, v1);
        a0 += v0[0] * __ldg(x + i0.x) + v0[1] * __ldg(x + i0.y) + v0[2] * __ldg(x + i0.z) + v0[3] * __ldg(x + i0.w);
        a1 += v1[0] * __ldg(x + i1.x) + v1[1] * __ldg(x + i1.y) + v1[2] * __ldg(x + i1.z) + v1[3] * __ldg(x + i1.w);
    }
    if (c < nch) {
        const int64_t o0 = base + (int64_t)c * 128;
        const int4 i0 = __ldg(reinterpret_cast<const int4*>(scol + o0));
        T v0[4];
        Vec4Of<T>::load(sval + o0, v0);
        a0 += v0[0] * __ldg(x + i0.x) + v0[1] * __ldg(x + i0.y) + v0[2] * __ldg(x + i0.z) + v0[3] * __ldg(x + i0.w);
    }
    return a0 + a1;
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_sell_spmv(int n, const int64_t* __restrict__ sptr, const int32_t* __restrict__ slen,
                                                      const int32_t* __restrict__ scol, const T* __restrict__ sval,
                                                      const T* __restrict__ x, T* __restrict__ y) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    y[r] = sell_row(r, sptr, slen, scol, sval, x);
}

template <int NV>
__device__ __forceinline__ void block_reduce(double (&v)[NV], double* sh) {
    // sh: NV * 32 doubles
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double a = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) sh[k * 32 + wid] = a;
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double a = lane < nw ? sh[k * 32 + lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
            v[k] = a;
        }
    }
}

// Writes the block's NV partial sums; the last block to finish reduces all partials in a
// fixed order (deterministic) and returns true in thread 0 with the totals in v.
template <int NV>
__device__ __forceinline__ bool grid_reduce(double (&v)[NV], double* partial, unsigned int* ticket) {
    __shared__ double sh[NV * 32];
    __shared__ bool last;
    block_reduce<NV>(v, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) partial[(size_t)NV * blockIdx.x + k] = v[k];
        __threadfence();
        const unsigned t = atomicAdd(ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.0;
    // four partials per thread in flight (L2 reads, after the fence), added in ascending order
    const int nb = (int)gridDim.x, bd = (int)blockDim.x;
    for (int b = threadIdx.x; b < nb; b += 4 * bd) {
        double t[4][NV];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int k = 0; k < NV; ++k) t[u][k] = b + u * bd < nb ? __ldcg(partial + (size_t)NV * (b + u * bd) + k) : 0.0;
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int k = 0; k < NV; ++k) acc[k] += t[u][k];
    }
    __syncthreads();
    block_reduce<NV>(acc, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] = acc[k];
        *ticket = 0;
        return true;
    }
    return false;
}

__device__ __forceinline__ void cg_check(CgState* st, double rr) {
    st->rr = rr;
    if (!(rr == rr)) { st->done = 1; st->status = -2; return; }
    if (rr <= st->tol2) { st->done = 1; st->status = 1; return; }
    if (st->iter >= st->max_iter) { st->done = 1; st->status = -1; }
}

// r = b - A x (x may be null: zero guess), z = D^-1 r, p = z; rz, rr
template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_init(int n, const int64_t* __restrict__ sptr, const int32_t* __restrict__ slen,
                                                    const int32_t* __restrict__ scol, const T* __restrict__ sval,
                                                    const T* __restrict__ x, const T* __restrict__ b, const T* __restrict__ dinv,
                                                    T* __restrict__ r, T* __restrict__ z, T* __restrict__ p,
                                                    double* partial, CgState* st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (i < n) {
        T ri = b[i];
        if (x) ri -= sell_row(i, sptr, slen, scol, sval, x);
        const T zi = dinv[i] * ri;
        r[i] = ri;
        z[i] = zi;
        p[i] = zi;
        v[0] = (double)ri * (double)zi;
        v[1] = (double)ri * (double)ri;
    }
    if (grid_reduce<2>(v, partial, &st->ticket)) {
        st->rz = v[0];
        st->rr0 = v[1];
        st->iter = 0;
        st->done = 0;
        st->status = 0;
        cg_check(st, v[1]);
    }
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_spmv_pq(int n, const int64_t* __restrict__ sptr, const int32_t* __restrict__ slen,
                                                       const int32_t* __restrict__ scol, const T* __restrict__ sval,
                                                       const T* __restrict__ p, T* __restrict__ q, double* partial, CgState* st) {
    if (st->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0.0};
    if (i < n) {
        const T qi = sell_row(i, sptr, slen, scol, sval, p);
        q[i] = qi;
        v[0] = (double)p[i] * (double)qi;
    }
    if (grid_reduce<1>(v, partial, &st->ticket)) {
        st->pq = v[0];
        st->alpha = st->rz / v[0];
    }
}

// ---- FP64-accurate SpMV from FP32 pairs ("double-float"): GB300 runs FP64 at 1/64 of the FP32
// rate, so the outer CG's A p reads the matrix as hi + lo FP32 pairs (hi = fl32(a), lo =
// fl32(a - hi)) and p as hi + lo pairs, forms every product with an error-free FMA split and
// sums each row with TwoSum (Dekker/Knuth); the FP64 pipe only sees one conversion per row.
// Accuracy ~2^-48 relative per term (FP64: 2^-53); the bytes per nonzero equal the FP64
// matrix's (4 + 4 value, 4 column).
// the _rn intrinsics are never contracted into FMAs, which the error-free steps rely on
__device__ __forceinline__ void df_add(float& sh, float& sl, float prod, float small) {
    const float s = __fadd_rn(sh, prod);
    const float bb = __fsub_rn(s, sh);
    const float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(prod, bb));  // TwoSum error
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(e, small));
}

__device__ __forceinline__ void df_term(float& sh, float& sl, float ah, float al, float ph, float pl) {
    const float prod = __fmul_rn(ah, ph);
    const float perr = __fmaf_rn(ah, ph, -prod);  // exact rounding error of ah * ph
    const float cross = __fadd_rn(__fmaf_rn(ah, pl, __fmul_rn(al, ph)), perr);
    df_add(sh, sl, prod, cross);
}

__global__ void __launch_bounds__(kBlock) k_cg_spmv_pq_df(int n, const int64_t* __restrict__ sptr,
                                                          const int32_t* __restrict__ slen,
                                                          const int32_t* __restrict__ scol, const float* __restrict__ vhi,
                                                          const float* __restrict__ vlo, const float2* __restrict__ p2,
                                                          const double* __restrict__ p, double* __restrict__ q,
                                                          double* partial, CgState* st) {
    if (st->done) return;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int s = i >> 5;
        const int64_t base = sptr[s] + (int64_t)(i & 31) * 4;
        const int nch = slen[s] >> 2;
        // two chunks in flight, each with its own (hi, lo) accumulator; p as interleaved pairs
        // (one 8-byte gather per nonzero)
        float sh0 = 0.f, sl0 = 0.f, sh1 = 0.f, sl1 = 0.f;
        auto chunk = [&](int64_t o, float& sh, float& sl) {
            const int4 ci = __ldg(reinterpret_cast<const int4*>(scol + o));
            const float4 hi = __ldg(reinterpret_cast<const float4*>(vhi + o));
            const float4 lo = __ldg(reinterpret_cast<const float4*>(vlo + o));
            const float2 px = __ldg(p2 + ci.x), py = __ldg(p2 + ci.y), pz = __ldg(p2 + ci.z), pw = __ldg(p2 + ci.w);
            df_term(sh, sl, hi.x, lo.x, px.x, px.y);
            df_term(sh, sl, hi.y, lo.y, py.x, py.y);
            df_term(sh, sl, hi.z, lo.z, pz.x, pz.y);
            df_term(sh, sl, hi.w, lo.w, pw.x, pw.y);
        };
        int c = 0;
        for (; c + 1 < nch; c += 2) {
            chunk(base + (int64_t)c * 128, sh0, sl0);
            chunk(base + (int64_t)(c + 1) * 128, sh1, sl1);
        }
        if (c < nch) chunk(base + (int64_t)c * 128, sh0, sl0);
        df_add(sh0, sl0, sh1, sl1);
        const double qi = (double)sh0 + (double)sl0;
        q[i] = qi;
        v[0] += p[i] * qi;
    }
    if (grid_reduce<1>(v, partial, &st->ticket)) {
        st->pq = v[0];
        st->alpha = st->rz / v[0];
    }
}

// lo = fl32(a - fl32(a)) for every stored entry
__global__ void k_split_lo(long long n, const double* __restrict__ a, const float* __restrict__ hi, float* __restrict__ lo) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) lo[i] = (float)(a[i] - (double)hi[i]);
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_update(int n, T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
                                                      const T* __restrict__ q, const T* __restrict__ dinv, T* __restrict__ z,
                                                      double* partial, CgState* st) {
    if (st->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const T alpha = (T)st->alpha;
    double v[2] = {0.0, 0.0};
    if (i < n) {
        x[i] += alpha * p[i];
        const T ri = r[i] - alpha * q[i];
        const T zi = dinv[i] * ri;
        r[i] = ri;
        z[i] = zi;
        v[0] = (double)ri * (double)zi;
        v[1] = (double)ri * (double)ri;
    }
    if (grid_reduce<2>(v, partial, &st->ticket)) {
        st->beta = v[0] / st->rz;
        st->rz = v[0];
        st->iter += 1;
        cg_check(st, v[1]);
    }
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_cg_direction(int n, const T* __restrict__ z, T* __restrict__ p, const CgState* st) {
    if (st->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    p[i] = z[i] + (T)st->beta * p[i];
}

// FP64 residual r = b - A x with its squared norm; comp: each row's product compensated
// (Dot2, as accurate as twice the working precision) for tolerances near the FP64 floor.
__global__ void __launch_bounds__(kBlock) k_residual64(int n, const int64_t* __restrict__ sptr, const int32_t* __restrict__ slen,
                                                       const int32_t* __restrict__ scol, const double* __restrict__ sval,
                                                       const double* __restrict__ x, const double* __restrict__ b,
                                                       double* __restrict__ r, double* partial, CgState* st, int comp) {
    double v[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double mag = 0.0;
        const double ri = comp ? sell_residual_dot2(i, sptr, slen, scol, sval, x, b[i], mag)
                               : b[i] - sell_row(i, sptr, slen, scol, sval, x);
        r[i] = ri;
        v[0] += ri * ri;
        v[1] += mag * mag;
    }
    if (grid_reduce<2>(v, partial, &st->ticket)) {
        st->rr = v[0];
        st->ff = v[1];
    }
}

__global__ void k_norm2(int n, const double* __restrict__ a, double* partial, CgState* st) {
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[0] += a[i] * a[i];
    if (grid_reduce<1>(v, partial, &st->ticket)) st->rr = v[0];
}

__global__ void k_scale_to32(int n, const double* __restrict__ r, const CgState* st, float* __restrict__ r32,
                             float* __restrict__ d32) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double s = 1.0 / sqrt(st->rr);
    r32[i] = (float)(r[i] * s);
    d32[i] = 0.0f;
}

__global__ void k_refine(int n, double* __restrict__ x, const float* __restrict__ d, const CgState* st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] += sqrt(st->rr) * (double)d[i];
}

// ---- FP64 CG preconditioned by the FP32 multigrid V-cycle
__global__ void k_to32(int n, const double* __restrict__ a, float* __restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

// p = z (the V-cycle result, FP32), rz = r.z; phi/plo: the FP32 pair of p (may be null)
__global__ void __launch_bounds__(kBlock) k_pcg_start(int n, const float* __restrict__ z32, const double* __restrict__ r,
                                                      double* __restrict__ p, float2* __restrict__ p2, double* partial,
                                                      CgState* st) {
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double zi = (double)z32[i];
        p[i] = zi;
        if (p2) p2[i] = make_float2(z32[i], 0.f);
        v[0] += r[i] * zi;
    }
    if (grid_reduce<1>(v, partial, &st->ticket)) st->rz = v[0];
}

// x += alpha p, r -= alpha q, FP32 copy of r for the V-cycle, rr and the stop test
__global__ void __launch_bounds__(kBlock) k_pcg_update(int n, double* __restrict__ x, double* __restrict__ r,
                                                       const double* __restrict__ p, const double* __restrict__ q,
                                                       float* __restrict__ r32, double* partial, CgState* st) {
    if (st->done) return;
    const double alpha = st->alpha;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        const double ri = r[i] - alpha * q[i];
        r[i] = ri;
        r32[i] = (float)ri;
        v[0] += ri * ri;
    }
    if (grid_reduce<1>(v, partial, &st->ticket)) {
        st->iter += 1;
        cg_check(st, v[0]);
    }
}

// beta = r.z / r.z_old with z the V-cycle result (FP32)
__global__ void __launch_bounds__(kBlock) k_pcg_rz(int n, const float* __restrict__ z32, const double* __restrict__ r,
                                                   double* partial, CgState* st) {
    if (st->done) return;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[0] += r[i] * (double)z32[i];
    if (grid_reduce<1>(v, partial, &st->ticket)) {
        st->beta = v[0] / st->rz;
        st->rz = v[0];
    }
}

// element matrices (378 packed upper-triangle FP64 entries per cell) to FP32 in block order and
// cyclic-half layout, t paired: entry 54 u + 2 i + s of position p is K(i, (i + t) mod 27) of
// cell perm[p] with t = 2 u + s (u = 0..6, s = 0, 1), so lane i reads (t, t+1) as one float2
__global__ void k_ke_cyclic(long long total, const int32_t* __restrict__ perm, const double* __restrict__ ke,
                            float* __restrict__ out, float* __restrict__ out_lo) {
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const long long p = idx / 378;
    const int e = (int)(idx - p * 378), u = e / 54, rem = e - 54 * u, i = rem >> 1, t = 2 * u + (rem & 1);
    int j = i + t;
    if (j >= 27) j -= 27;
    const int lo = i < j ? i : j, hi = i < j ? j : i;
    const double v = ke[378 * (size_t)perm[p] + lo * 27 - (lo * (lo - 1)) / 2 + (hi - lo)];
    const float h = (float)v;
    out[idx] = h;
    if (out_lo) out_lo[idx] = (float)(v - (double)h);
}


__global__ void k_fixed_flags(int n, const int8_t* __restrict__ bc, int anode, int8_t* __restrict__ fixed) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) fixed[i] = (bc[i] == 1 || (anode && bc[i] == 2)) ? 1 : 0;
}

__global__ void k_scale_mul(int n, double* __restrict__ a, const double* __restrict__ b, double s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] *= s * b[i];
}

__global__ void k_scale_copy64(int n, const double* __restrict__ a, double s, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = s * a[i];
}

// p = z + beta p (and its FP32 pair when phi is not null)
__global__ void __launch_bounds__(kBlock) k_pcg_direction(int n, const float* __restrict__ z32, double* __restrict__ p,
                                                          float2* __restrict__ p2, const CgState* st) {
    if (st->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double pi = (double)z32[i] + st->beta * p[i];
    p[i] = pi;
    if (p2) {
        const float h = (float)pi;
        p2[i] = make_float2(h, (float)(pi - (double)h));
    }
}

// ---- FP32 inner CG of the mixed multigrid solve (precision 3): e (the correction), r, p and
// q = -A p in FP32 with the level-0 operator of the V-cycle, sums in FP64, scalars in CgState

// p = z, rz = r.z
__global__ void __launch_bounds__(kBlock) k_mcg_start(int n, const float* __restrict__ z, const float* __restrict__ r,
                                                      float* __restrict__ p, double* partial, CgState* st) {
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float zi = z[i];
        p[i] = zi;
        v[0] += (double)r[i] * zi;
    }
    if (grid_reduce<1>(v, partial, &st->ticket)) st->rz = v[0];
}

// p.q from q = -A p; alpha = rz / p.A p (a non-positive curvature ends the inner solve)
__global__ void __launch_bounds__(kBlock) k_mcg_pq(int n, const float* __restrict__ p, const float* __restrict__ qn,
                                                   double* partial, CgState* st) {
    if (st->done) return;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[0] += (double)p[i] * qn[i];
    if (grid_reduce<1>(v, partial, &st->ticket)) {
        const double pq = -v[0];
        st->pq = pq;
        if (!(pq > 0.0)) {
            st->done = 1;
            st->status = -2;
        } else {
            st->alpha = st->rz / pq;
        }
    }
}

// e += alpha p, r -= alpha A p (= r + alpha q), rr and the stop test
__global__ void __launch_bounds__(kBlock) k_mcg_update(int n, float* __restrict__ e, float* __restrict__ r,
                                                       const float* __restrict__ p, const float* __restrict__ qn,
                                                       double* partial, CgState* st) {
    if (st->done) return;
    const float alpha = (float)st->alpha;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        e[i] = fmaf(alpha, p[i], e[i]);
        const float ri = fmaf(alpha, qn[i], r[i]);
        r[i] = ri;
        v[0] += (double)ri * ri;
    }
    if (grid_reduce<1>(v, partial, &st->ticket)) {
        st->iter += 1;
        cg_check(st, v[0]);
    }
}

// beta = r.z / r.z_old
__global__ void __launch_bounds__(kBlock) k_mcg_rz(int n, const float* __restrict__ z, const float* __restrict__ r,
                                                   double* partial, CgState* st) {
    if (st->done) return;
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[0] += (double)r[i] * z[i];
    if (grid_reduce<1>(v, partial, &st->ticket)) {
        st->beta = v[0] / st->rz;
        st->rz = v[0];
    }
}

// p = z + beta p
__global__ void __launch_bounds__(kBlock) k_mcg_direction(int n, const float* __restrict__ z, float* __restrict__ p,
                                                          const CgState* st) {
    if (st->done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = fmaf((float)st->beta, p[i], z[i]);
}

// x += e (the FP32 correction into the FP64 solution)
__global__ void k_add_correction(int n, double* __restrict__ x, const float* __restrict__ e) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += (double)e[i];
}

// ---- outer SpMV of the Q2 multigrid PCG by cell blocks (the level-0 smoother's blocks,
// cell_blocks.h), FP64-accurate from FP32 pairs: q = A p and p.q. K_e as hi/lo pairs in the
// cyclic-half layout; lane i < 27 of a warp owns row i of a cell, forms K(i, i+t) p_{i+t} with
// an error-free product and hands the pair K(i, i+t) p_i (product, rounding error + cross terms)
// to lane i+t, all sums compensated (TwoSum). Columns and rows of Dirichlet DoFs follow the
// eliminated matrix: p is taken as 0 on them and their q is diag * p.
struct CbSpmvArgs {
    int n_blocks, max_cells, max_dofs, n_bnd;
    const float* khi;
    const float* klo;
    const int32_t* cell_start;
    const int32_t* dof_start;
    const int32_t* dof_list;
    const int32_t* slot;
    const int32_t* bnd_dofs;
    const int32_t* bnd_ptr;
    const uint16_t* item_end;
    const uint16_t* loc;
    const uint16_t* items;
    const int8_t* fixed;
    float2* pair;   // partial (hi, lo) sums of the split DoFs, one per slot
    double* dot;    // p.q partials: one per block, then one per CTA of the finishing kernel
};

constexpr int kCbT = 256;
__host__ __device__ inline size_t cbdf_smem_bytes(int max_cells, int max_dofs) {
    return 56 * (size_t)max_cells + 8 * (size_t)max_dofs + 216 * (size_t)max_cells;
}

// one cell's row i (lane) of K_e p_e, (hi, lo) pair; kh/kl: K(i, i+t), t = 0..13
__device__ __forceinline__ void cb_row_df(const float (&kh)[14], const float (&kl)[14], float ph, float pl, int lane,
                                          float& sh, float& sl) {
    sh = 0.f;
    sl = 0.f;
    df_term(sh, sl, kh[0], kl[0], ph, pl);
#pragma unroll
    for (int t = 1; t < 14; ++t) {
        int up = lane + t;
        if (up >= 27) up -= 27;
        int dn = lane - t;
        if (dn < 0) dn += 27;
        const float uh = __shfl_sync(0xffffffffu, ph, up);
        const float ul = __shfl_sync(0xffffffffu, pl, up);
        const float prod = __fmul_rn(kh[t], ph);
        const float perr = __fmaf_rn(kh[t], ph, -prod);
        const float cross = __fadd_rn(__fmaf_rn(kh[t], pl, __fmul_rn(kl[t], ph)), perr);
        const float rp = __shfl_sync(0xffffffffu, prod, dn);
        const float rc = __shfl_sync(0xffffffffu, cross, dn);
        df_term(sh, sl, kh[t], kl[t], uh, ul);
        df_add(sh, sl, rp, rc);
    }
}

__global__ void __launch_bounds__(kCbT, 2) k_cb_spmv_df(CbSpmvArgs a, const float2* __restrict__ p2,
                                                        const double* __restrict__ p, const double* __restrict__ dinv,
                                                        double* __restrict__ q, const CgState* st) {
    if (st->done) return;
    extern __shared__ __align__(16) unsigned char cbdf_raw[];
    __shared__ double red[32];
    const int blk = blockIdx.x;
    const int p0 = a.cell_start[blk], nb = a.cell_start[blk + 1] - p0;
    const int q0 = a.dof_start[blk], nq = a.dof_start[blk + 1] - q0;
    uint16_t* sit = reinterpret_cast<uint16_t*>(cbdf_raw);
    float2* sp = reinterpret_cast<float2*>(cbdf_raw + 56 * (size_t)a.max_cells);
    float2* sy = sp + a.max_dofs;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int il = lane < 27 ? lane : 26;  // lanes 27..31 shadow lane 26 and store nothing
    {
        const uint2* gi = reinterpret_cast<const uint2*>(a.items + 28 * (size_t)p0);
        uint2* si = reinterpret_cast<uint2*>(sit);
        const int nw = 7 * nb;
        uint2 w8[7];
#pragma unroll
        for (int r = 0; r < 7; ++r) {
            const int w = tid + r * kCbT;
            if (w < nw) w8[r] = __ldg(gi + w);
        }
#pragma unroll
        for (int r0 = 0; r0 < 16; r0 += 8) {
            int gd[8];
            float2 pv[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int k = tid + (r0 + r) * kCbT;
                gd[r] = k < nq ? __ldg(a.dof_list + q0 + k) : 0;
            }
            int fx[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int k = tid + (r0 + r) * kCbT;
                pv[r] = k < nq ? __ldg(p2 + gd[r]) : make_float2(0.f, 0.f);
                fx[r] = k < nq ? a.fixed[gd[r]] : 0;
            }
#pragma unroll
            for (int r = 0; r < 8; ++r)
                if (fx[r]) pv[r] = make_float2(0.f, 0.f);
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int k = tid + (r0 + r) * kCbT;
                if (k < nq) sp[k] = pv[r];
            }
        }
#pragma unroll
        for (int r = 0; r < 7; ++r) {
            const int w = tid + r * kCbT;
            if (w < nw) si[w] = w8[r];
        }
    }
    __syncthreads();
    const uint16_t* loc = a.loc + 27 * (size_t)p0;
    // one warp per cell (w, w + 8, ...); two register sets alternate so that the next cell's
    // hi/lo element matrix is in flight while the current one is applied
    float hA[14], lA[14], hB[14], lB[14];
    int iA = 0, iB = 0;
    auto load_cell = [&](int c, float (&kh)[14], float (&kl)[14], int& li) {
        const float2* hp = reinterpret_cast<const float2*>(a.khi + 378 * (size_t)(p0 + c));
        const float2* lp = reinterpret_cast<const float2*>(a.klo + 378 * (size_t)(p0 + c));
#pragma unroll
        for (int u = 0; u < 7; ++u) {
            const float2 x = __ldg(hp + 27 * u + il), y = __ldg(lp + 27 * u + il);
            kh[2 * u] = x.x;
            kh[2 * u + 1] = x.y;
            kl[2 * u] = y.x;
            kl[2 * u + 1] = y.y;
        }
        li = __ldg(loc + 27 * c + il);
    };
    auto apply_cell = [&](int c, const float (&kh)[14], const float (&kl)[14], int li) {
        const float2 pv = sp[li];
        float h, l;
        cb_row_df(kh, kl, pv.x, pv.y, lane, h, l);
        if (lane < 27) sy[27 * c + lane] = make_float2(h, l);
    };
    constexpr int kW = kCbT / 32;
    if (warp < nb) load_cell(warp, hA, lA, iA);
    for (int c = warp; c < nb; c += 2 * kW) {
        if (c + kW < nb) load_cell(c + kW, hB, lB, iB);
        apply_cell(c, hA, lA, iA);
        if (c + kW >= nb) break;
        if (c + 2 * kW < nb) load_cell(c + 2 * kW, hA, lA, iA);
        apply_cell(c + kW, hB, lB, iB);
    }
    __syncthreads();
    double v[1] = {0.0};
#pragma unroll 1
    for (int r0 = 0; r0 < 16; r0 += 8) {
        if (tid + r0 * kCbT >= nq) break;
        int e0[8], e1[8], sl[8], g[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int k = tid + (r0 + r) * kCbT;
            const bool ok = k < nq;
            e1[r] = ok ? __ldg(a.item_end + q0 + k) : 0;
            e0[r] = ok && k ? __ldg(a.item_end + q0 + k - 1) : 0;
            sl[r] = ok ? __ldg(a.slot + q0 + k) : -2;
            g[r] = ok ? __ldg(a.dof_list + q0 + k) : 0;
        }
        double pf[8], dv[8];
        int fx[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const bool own = sl[r] == -1;
            pf[r] = own ? p[g[r]] : 0.0;
            fx[r] = own ? a.fixed[g[r]] : 0;
            dv[r] = own && fx[r] ? dinv[g[r]] : 1.0;
        }
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            float h = 0.f, l = 0.f;
            for (int e = e0[r]; e < e1[r]; ++e) {
                const float2 y = sy[sit[e]];
                df_add(h, l, y.x, y.y);
            }
            if (sl[r] >= 0) {
                a.pair[sl[r]] = make_float2(h, l);
            } else if (sl[r] == -1) {
                const double qg = fx[r] ? pf[r] / dv[r] : (double)h + (double)l;
                q[g[r]] = qg;
                v[0] += pf[r] * qg;
            }
        }
    }
    block_reduce<1>(v, red);
    if (tid == 0) a.dot[blk] = v[0];
}

// the split DoFs: their slot pairs summed in ascending block order; then p.q over all blocks
// and CTAs (fixed order) and alpha = rz / p.q
__global__ void __launch_bounds__(kBlock) k_cb_spmv_finish(CbSpmvArgs a, const double* __restrict__ p,
                                                           const double* __restrict__ dinv, double* __restrict__ q,
                                                           CgState* st) {
    if (st->done) return;
    __shared__ double red[32];
    __shared__ bool last;
    double v[1] = {0.0};
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < a.n_bnd; j += gridDim.x * blockDim.x) {
        const int g = a.bnd_dofs[j];
        const double pg = p[g];
        double qg;
        if (a.fixed[g]) {
            qg = pg / dinv[g];
        } else {
            float h = 0.f, l = 0.f;
            for (int s = a.bnd_ptr[j]; s < a.bnd_ptr[j + 1]; ++s) {
                const float2 y = a.pair[s];
                df_add(h, l, y.x, y.y);
            }
            qg = (double)h + (double)l;
        }
        q[g] = qg;
        v[0] += pg * qg;
    }
    block_reduce<1>(v, red);
    if (threadIdx.x == 0) {
        a.dot[a.n_blocks + blockIdx.x] = v[0];
        __threadfence();
        last = atomicAdd(&st->ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double acc[1] = {0.0};
    const int total = a.n_blocks + (int)gridDim.x, bd = (int)blockDim.x;
    for (int b = threadIdx.x; b < total; b += 4 * bd) {
        double t[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) t[u] = b + u * bd < total ? __ldcg(a.dot + b + u * bd) : 0.0;
#pragma unroll
        for (int u = 0; u < 4; ++u) acc[0] += t[u];
    }
    __syncthreads();
    block_reduce<1>(acc, red);
    if (threadIdx.x == 0) {
        st->pq = acc[0];
        st->alpha = st->rz / acc[0];
        st->ticket = 0;
    }
}

}  // namespace

// ==================================================================== FemDevice
FemDevice::FemDevice(const PreparedMesh& pm, FemStructure&& fs, cudaStream_t stream)
    : fs_(std::move(fs)), pm_(&pm), stream_(stream), n_(fs_.n_dofs), nc_(fs_.n_cells) {
    cudaStream_t s = stream_;
    if (fs_.order == 2) {
        // the cell blocks (host, ~0.3 s on the 1.7e7-DoF Q2 nanotip) are built while the
        // uploads below run and until the first assembly needs them
        cb_host_cells_ = cb_cells_;
        cb_host_dofs_ = cb_max_dofs_;
        cb_host_ = std::async(std::launch::async, [this] { return build_cell_blocks(fs_, cb_host_cells_, cb_host_dofs_); });
    }
    level0_ebe_ = fs_.order == 2;
    outer_mode_ = fs_.order == 2 ? 2 : 1;
    cell_dofs_.upload(fs_.cell_dofs, s);
    r2c_ptr_.upload(fs_.r2c_ptr, s);
    r2c_item_.upload(fs_.r2c_item, s);
    r2f_ptr_.upload(fs_.r2f_ptr, s);
    r2f_item_.upload(fs_.r2f_item, s);
    if (!fs_.top_faces.empty()) top_faces_.upload(fs_.top_faces, s);
    dof2node_.upload(fs_.dof2node, s);
    if (fs_.order == 1) {
        rowptr_.upload(fs_.rowptr, s);
        col_.upload(fs_.col, s);
        csr2sell_.upload(fs_.csr2sell, s);
    } else {
        row_len_.upload(fs_.row_len, s);
        for (int v : fs_.row_len) max_row_ = std::max(max_row_, v);
    }
    slice_ptr_.upload(fs_.slice_ptr, s);
    slice_len_.upload(fs_.slice_len, s);
    if (fs_.order == 2 && fs_.sell_col.empty()) {
        // Q2 columns built on the device from the cells of each row
        int max_cells = 0;
        for (int d = 0; d < n_; ++d) max_cells = std::max(max_cells, fs_.r2c_ptr[d + 1] - fs_.r2c_ptr[d]);
        sell_col_.resize(fs_.slice_ptr.back());
        const int bad = q2_sell_columns(n_, (int)fs_.slice_len.size(), slice_ptr_.get(), slice_len_.get(),
                                        row_len_.get(), r2c_ptr_.get(), r2c_item_.get(), cell_dofs_.get(), max_cells,
                                        sell_col_.get(), s);
        FGB_REQUIRE(bad == 0, "Q2 structure: device column count differs from the row length");
    } else {
        sell_col_.upload(fs_.sell_col, s);
    }
    bc_.upload(fs_.bc_kind, s);
    if (fs_.order == 1) {
        std::vector<double> dxyz(3 * (size_t)n_);
        for (int d = 0; d < n_; ++d)
            for (int c = 0; c < 3; ++c) dxyz[3 * (size_t)d + c] = pm.hex.xyz[3 * (size_t)fs_.dof2node[d] + c];
        dof_xyz_.upload(dxyz, s);
        ke_.resize(64 * (size_t)nc_);
        kval_.resize(fs_.nnz());
    } else {
        dof_xyz_.upload(fs_.dof_xyz, s);
        ke_.resize(378 * (size_t)nc_);
        kval_.resize(fs_.slice_ptr.back());  // saved matrix in the SELL layout
        kval_.zero(s);
    }
    sell64_.resize(fs_.slice_ptr.back());
    sell32_.resize(fs_.slice_ptr.back());
    sell64_.zero(s);
    sell32_.zero(s);
    dinv64_.resize(n_);
    dinv32_.resize(n_);
    rhs_.resize(n_);
    x_.resize(n_);
    x_.zero(s);
    r64_.resize(n_); p64_.resize(n_); q64_.resize(n_); z64_.resize(n_);
    r32_.resize(n_); p32_.resize(n_); p32b_.resize(n_); q32_.resize(n_); z32_.resize(n_); d32_.resize(n_);
    partial_.resize(std::max<size_t>(2 * (size_t)grid_for(n_, kBlock), 2 * kMixedSumMax * (size_t)mixed_cg_grid(n_)) + 64);
    mixed_.resize(1);
    FGB_CUDA(cudaMallocHost(&h_mixed_, sizeof(MixedResult)));
    state_.resize(2);
    state_.zero(s);
    FGB_CUDA(cudaMallocHost(&h_state_, 2 * sizeof(CgState)));
    FGB_CUDA(cudaEventCreate(&ev0_));
    FGB_CUDA(cudaEventCreate(&ev1_));
    FGB_CUDA(cudaEventCreate(&kev0_));
    FGB_CUDA(cudaEventCreate(&kev1_));
    FGB_CUDA(cudaStreamSynchronize(s));
    // the host copies of the structure that only the device needs are dropped
    fs_.r2c_item.clear(); fs_.r2c_item.shrink_to_fit();
    fs_.csr2sell.clear(); fs_.csr2sell.shrink_to_fit();
    fs_.sell_col.clear(); fs_.sell_col.shrink_to_fit();
    fs_.dof_xyz.clear(); fs_.dof_xyz.shrink_to_fit();
}

FemDevice::~FemDevice() {
    amg_.reset();
    q1_.reset();
    if (h_state_) cudaFreeHost(h_state_);
    if (h_mixed_) cudaFreeHost(h_mixed_);
    cudaEventDestroy(ev0_);
    cudaEventDestroy(ev1_);
    cudaEventDestroy(kev0_);
    cudaEventDestroy(kev1_);
}

void FemDevice::setup(double applied_field, double applied_potential) {
    applied_field_ = applied_field;
    applied_potential_ = applied_potential;
    x_.zero(stream_);  // solution = dirichlet_bc_value (0), src/DealSolver.cpp:384
    x_zero_ = true;
}

double* FemDevice::space_charge_buffer(bool accumulate) {
    if (!has_extra_ || rhs_extra_.size() != (size_t)n_ || !accumulate) {
        rhs_extra_.resize(n_);
        rhs_extra_.zero(stream_);
    }
    has_extra_ = true;
    return rhs_extra_.get();
}

const int32_t* FemDevice::d_node2dof() {
    if (!node2dof_dev_.size()) node2dof_dev_.upload(fs_.node2dof, stream_);
    return node2dof_dev_.get();
}

const int32_t* FemDevice::d_hex2cell() {
    if (!hex2cell_dev_.size()) {
        std::vector<int32_t> h(pm_->hex.n_hexs(), -1);
        for (size_t c = 0; c < pm_->vac.cells.size(); ++c) h[pm_->vac.cells[c]] = (int32_t)c;
        hex2cell_dev_.upload(h, stream_);
    }
    return hex2cell_dev_.get();
}

void FemDevice::set_space_charge(const double* d_extra) {
    if (!d_extra) { has_extra_ = false; return; }
    rhs_extra_.resize(n_);
    FGB_CUDA(cudaMemcpyAsync(rhs_extra_.get(), d_extra, sizeof(double) * n_, cudaMemcpyDeviceToDevice, stream_));
    has_extra_ = true;
}

void FemDevice::assemble(bool full_run, bool anode_dirichlet) {
    anode_dirichlet_ = anode_dirichlet;
    split_valid_ = false;
    const int gb = grid_for(n_, kBlock);
    if (fs_.order == 2) {
        if (full_run) {
            if (ke_tensor_)
                q2_cell_stiffness_tc(nc_, cell_dofs_.get(), dof_xyz_.get(), ke_.get(), tc_scratch_, tc_err_, stream_);
            else
                q2_cell_stiffness(nc_, cell_dofs_.get(), dof_xyz_.get(), ke_.get(), stream_);
            kval_valid_ = false;
            if (!lazy_matrix_) {
                q2_assemble_rows(n_, max_row_, slice_ptr_.get(), sell_col_.get(), row_len_.get(), r2c_ptr_.get(),
                                 r2c_item_.get(), cell_dofs_.get(), ke_.get(), kval_.get(), stream_);
                kval_valid_ = true;
            }
            if (level0_ebe_ || outer_mode_ == 2) refresh_ke32();
        }
        fixed_.resize(n_);
        FGB_LAUNCH(k_fixed_flags<<<gb, kBlock, 0, stream_>>>(n_, bc_.get(), anode_dirichlet ? 1 : 0, fixed_.get()));
        const double bc = anode_dirichlet ? 0.0 : applied_field_;
        q2_neumann_rows(n_, r2f_ptr_.get(), r2f_item_.get(), top_faces_.get(), dof_xyz_.get(), bc,
                        has_extra_ ? rhs_extra_.get() : nullptr, rhs_.get(), stream_);
        if (lazy_matrix_ && (!anode_dirichlet || applied_potential_ == 0.0)) {
            q2_dirichlet_zero(n_, r2c_ptr_.get(), r2c_item_.get(), ke_.get(), bc_.get(), anode_dirichlet ? 1 : 0,
                              dinv64_.get(), dinv32_.get(), rhs_.get(), x_.get(), stream_);
            sell_valid_ = false;
        } else {
            if (!kval_valid_) {
                q2_assemble_rows(n_, max_row_, slice_ptr_.get(), sell_col_.get(), row_len_.get(), r2c_ptr_.get(),
                                 r2c_item_.get(), cell_dofs_.get(), ke_.get(), kval_.get(), stream_);
                kval_valid_ = true;
            }
            sell_dirichlet(n_, slice_ptr_.get(), sell_col_.get(), row_len_.get(), kval_.get(), bc_.get(),
                           anode_dirichlet ? 1 : 0, applied_potential_, sell64_.get(), sell32_.get(), dinv64_.get(),
                           dinv32_.get(), rhs_.get(), x_.get(), stream_);
            sell_valid_ = true;
            if (anode_dirichlet && applied_potential_ != 0.0) x_zero_ = false;  // x holds the anode value
        }
        FGB_CUDA(cudaGetLastError());
        return;
    }
    if (full_run)
        FGB_LAUNCH(k_cell_stiffness<<<grid_for(nc_, 128), 128, 0, stream_>>>(nc_, cell_dofs_.get(), dof_xyz_.get(), ke_.get(),
                                                                           q1_gauss_));
    assemble_q1_rows(full_run, anode_dirichlet);
}

void FemDevice::assemble_from_ke(bool anode_dirichlet) {
    FGB_REQUIRE(fs_.order == 1, "element matrices from the caller: Q1 only");
    anode_dirichlet_ = anode_dirichlet;
    split_valid_ = false;
    assemble_q1_rows(true, anode_dirichlet);
    // a kept multigrid hierarchy stays a symmetric positive definite preconditioner (its
    // coarse levels are those of an earlier matrix of the same pattern); level 0 is the new
    // matrix itself, so its smoothing interval follows the new lambda_max
    if (amg_ && amg_anode_ == (anode_dirichlet ? 1 : 0)) amg_->set_level0_lambda(estimate_lambda(15, kAmgLambdaSeed));
}

void FemDevice::assemble_q1_rows(bool matrix, bool anode_dirichlet) {
    const int gb = grid_for(n_, kBlock);
    if (matrix) {
        FGB_LAUNCH(k_assemble_rows<<<gb, kBlock, 0, stream_>>>(n_, rowptr_.get(), col_.get(), r2c_ptr_.get(), r2c_item_.get(),
                                                    cell_dofs_.get(), ke_.get(), kval_.get()));
        FGB_CUDA(cudaGetLastError());
    }
    // Neumann rhs (or zero when the anode is a Dirichlet boundary)
    const double bc = anode_dirichlet ? 0.0 : applied_field_;
    FGB_LAUNCH(k_neumann_rows<<<gb, kBlock, 0, stream_>>>(n_, r2f_ptr_.get(), r2f_item_.get(), top_faces_.get(), dof_xyz_.get(), bc,
                                               face_vals_, has_extra_ ? rhs_extra_.get() : nullptr, rhs_.get()));
    FGB_LAUNCH(k_dirichlet_rows<<<gb, kBlock, 0, stream_>>>(n_, rowptr_.get(), col_.get(), kval_.get(), bc_.get(), anode_dirichlet ? 1 : 0,
                                                 applied_potential_, dirichlet_value_, csr2sell_.get(), sell64_.get(),
                                                 sell32_.get(), dinv64_.get(), dinv32_.get(), rhs_.get(), x_.get()));
    FGB_CUDA(cudaGetLastError());
    // x holds the boundary values on the Dirichlet rows
    if (dirichlet_value_ != 0.0 || (anode_dirichlet && applied_potential_ != 0.0)) x_zero_ = false;
}

void FemDevice::ensure_sell() {
    if (fs_.order != 2 || sell_valid_) return;
    if (!kval_valid_) {
        q2_assemble_rows(n_, max_row_, slice_ptr_.get(), sell_col_.get(), row_len_.get(), r2c_ptr_.get(),
                         r2c_item_.get(), cell_dofs_.get(), ke_.get(), kval_.get(), stream_);
        kval_valid_ = true;
    }
    // the eliminated values only: D^-1, the right-hand side and x are those of the assembly
    sell_dirichlet(n_, slice_ptr_.get(), sell_col_.get(), row_len_.get(), kval_.get(), bc_.get(),
                   anode_dirichlet_ ? 1 : 0, applied_potential_, sell64_.get(), sell32_.get(), nullptr, nullptr,
                   nullptr, nullptr, stream_);
    sell_valid_ = true;
    split_valid_ = false;
}

double FemDevice::cells_true_residual() {
    FGB_REQUIRE(fs_.order == 2, "residual from element matrices: Q2 fields");
    if (res_state_.size() != 1) res_state_.resize(1);
    CgState* rs = res_state_.get();
    FGB_CUDA(cudaMemsetAsync(rs, 0, sizeof(CgState), stream_));
    cell_y_.resize(27 * (size_t)nc_);
    q2_residual_cells(n_, nc_, r2c_ptr_.get(), r2c_item_.get(), cell_dofs_.get(), ke_.get(), fixed_.get(),
                      dinv64_.get(), x_.get(), rhs_.get(), cell_y_.get(), r64_.get(), stream_);
    FGB_LAUNCH(k_norm2<<<reduce_grid(n_, kBlock), kBlock, 0, stream_>>>(n_, r64_.get(), partial_.get(), rs));
    CgState h{};
    FGB_CUDA(cudaMemcpyAsync(&h, rs, sizeof(CgState), cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    return h.rr;
}

void FemDevice::set_lazy_matrix(bool on) {
    if (!on) ensure_sell();
    lazy_matrix_ = on;
}

void FemDevice::spmv64(const double* x, double* y) {
    ensure_sell();
    FGB_LAUNCH(k_sell_spmv<double><<<grid_for(n_, kBlock), kBlock, 0, stream_>>>(n_, slice_ptr_.get(), slice_len_.get(), sell_col_.get(),
                                                                      sell64_.get(), x, y));
}

double FemDevice::time_spmv(int precision, int reps) {
    ensure_sell();
    if (precision == 2) {
        ensure_amg(nullptr);
        return amg_->time_smoother(reps);
    }
    // times the SpMV+dot kernel of the CG iteration on a scratch state (done = 0, rz = 1)
    const int gb = grid_for(n_, kBlock);
    CgState* ds = state_.get() + 1;
    CgState init{};
    init.rz = 1.0;
    init.max_iter = 1 << 30;
    FGB_CUDA(cudaMemcpyAsync(ds, &init, sizeof(CgState), cudaMemcpyHostToDevice, stream_));
    if (precision) { FGB_CUDA(cudaMemsetAsync(p32_.get(), 0, sizeof(float) * n_, stream_)); }
    else { FGB_CUDA(cudaMemsetAsync(p64_.get(), 0, sizeof(double) * n_, stream_)); }
    auto launch = [&]() {
        if (precision)
            FGB_LAUNCH(k_cg_spmv_pq<float><<<gb, kBlock, 0, stream_>>>(n_, slice_ptr_.get(), slice_len_.get(), sell_col_.get(),
                                                            sell32_.get(), p32_.get(), q32_.get(), partial_.get(), ds));
        else
            FGB_LAUNCH(k_cg_spmv_pq<double><<<gb, kBlock, 0, stream_>>>(n_, slice_ptr_.get(), slice_len_.get(), sell_col_.get(),
                                                             sell64_.get(), p64_.get(), q64_.get(), partial_.get(), ds));
    };
    for (int i = 0; i < 3; ++i) launch();
    FGB_CUDA(cudaEventRecord(ev0_, stream_));
    for (int i = 0; i < reps; ++i) launch();
    FGB_CUDA(cudaEventRecord(ev1_, stream_));
    FGB_CUDA(cudaEventSynchronize(ev1_));
    float ms = 0;
    FGB_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
    return ms / reps;
}

void FemDevice::download_matrix(std::vector<double>& vals, std::vector<double>& rhs) {
    ensure_sell();
    // CSR order values after Dirichlet elimination, gathered back from the SELL layout
    std::vector<double> s = sell64_.to_host(stream_);
    // row r's CSR entries start at off[r] (Q1: the structure's row pointer; Q2: the prefix of
    // the row lengths); entry j of row r sits at its SELL position, rows in parallel
    std::vector<int64_t> q2off;
    if (fs_.order == 2) {
        q2off.assign(n_ + 1, 0);
        for (int r = 0; r < n_; ++r) q2off[r + 1] = q2off[r] + fs_.row_len[r];
    }
    const int64_t* off = fs_.order == 2 ? q2off.data() : fs_.rowptr.data();
    vals.resize(off[n_]);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int r = 0; r < n_; ++r) {
        const int sl = r / 32, lane = r % 32;
        const int64_t b = off[r], len = off[r + 1] - b;
        for (int64_t j = 0; j < len; ++j) vals[b + j] = s[fs_.slice_ptr[sl] + ((j / 4) * 32 + lane) * 4 + j % 4];
    }
    rhs = rhs_.to_host(stream_);
}

void FemDevice::run_cg(bool fp32, CgState* d_state, int max_iter, int chunk) {
    const int gb = grid_for(n_, kBlock);
    CgState* h = h_state_ + (fp32 ? 1 : 0);
    // one chunk = `chunk` iterations, launched back to back; kernels become no-ops once done.
    // The device sets done at max_iter at the latest; the host bound is a second guard.
    const long long max_chunks = (long long)max_iter / chunk + 2;
    for (long long c = 0;; ++c) {
        FGB_REQUIRE(c <= max_chunks, "CG did not report completion within its iteration budget");
        for (int it = 0; it < chunk; ++it) {
            if (fp32) {
                FGB_LAUNCH(k_cg_spmv_pq<float><<<gb, kBlock, 0, stream_>>>(n_, slice_ptr_.get(), slice_len_.get(), sell_col_.get(),
                                                                sell32_.get(), p32_.get(), q32_.get(), partial_.get(), d_state));
                FGB_LAUNCH(k_cg_update<float><<<gb, kBlock, 0, stream_>>>(n_, d32_.get(), r32_.get(), p32_.get(), q32_.get(), dinv32_.get(),
                                                               z32_.get(), partial_.get(), d_state));
                FGB_LAUNCH(k_cg_direction<float><<<gb, kBlock, 0, stream_>>>(n_, z32_.get(), p32_.get(), d_state));
            } else {
                FGB_LAUNCH(k_cg_spmv_pq<double><<<gb, kBlock, 0, stream_>>>(n_, slice_ptr_.get(), slice_len_.get(), sell_col_.get(),
                                                                 sell64_.get(), p64_.get(), q64_.get(), partial_.get(), d_state));
                FGB_LAUNCH(k_cg_update<double><<<gb, kBlock, 0, stream_>>>(n_, x_.get(), r64_.get(), p64_.get(), q64_.get(), dinv64_.get(),
                                                                z64_.get(), partial_.get(), d_state));
                FGB_LAUNCH(k_cg_direction<double><<<gb, kBlock, 0, stream_>>>(n_, z64_.get(), p64_.get(), d_state));
            }
        }
        FGB_CUDA(cudaMemcpyAsync(h, d_state, sizeof(CgState), cudaMemcpyDeviceToHost, stream_));
        FGB_CUDA(cudaStreamSynchronize(stream_));
        if (h->done) break;
    }
    FGB_CUDA(cudaGetLastError());
}

static int compensated_residual(const SolveOptions& opt);

int FemDevice::solve(const SolveOptions& opt, SolveStats* st) {
    SolveStats local;
    if (!st) st = &local;
    *st = SolveStats();
    FGB_CUDA(cudaEventRecord(ev0_, stream_));
    FGB_REQUIRE(opt.precision >= 0 && opt.precision <= 3, "precision 0..3");
    // the multigrid PCG over the cell blocks takes its FP64 true residual from the element
    // matrices when the assembled matrix is not current; everything else reads that matrix
    if (opt.precision != 2 || outer_mode_ != 2 || !level0_ebe_ || compensated_residual(opt)) ensure_sell();
    int rc = opt.precision == 0   ? solve_plain(opt, st)
             : opt.precision == 1 ? solve_mixed(opt, st)
             : opt.precision == 2 ? solve_amg(opt, st)
                                  : solve_amg_mixed(opt, st);
    x_zero_ = false;
    FGB_CUDA(cudaEventRecord(ev1_, stream_));
    FGB_CUDA(cudaEventSynchronize(ev1_));
    float ms = 0;
    FGB_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
    st->ms = ms;
    return rc;
}

static double tol2_of(const SolveOptions& opt, double bnorm) {
    const double t = std::max(opt.rel_tol * bnorm, opt.abs_tol);
    return t * t;
}
// true residuals are evaluated compensated when the relative tolerance approaches the FP64
// rounding floor of b - A x
static int compensated_residual(const SolveOptions& opt) {
    return opt.rel_tol > 0 && opt.rel_tol < kCompensatedResidualBelow ? 1 : 0;
}

int FemDevice::solve_plain(const SolveOptions& opt, SolveStats* st) {
    const int gb = grid_for(n_, kBlock);
    CgState* ds = state_.get();
    // ||b||
    FGB_LAUNCH(k_norm2<<<reduce_grid(n_, kBlock), kBlock, 0, stream_>>>(n_, rhs_.get(), partial_.get(), ds));
    FGB_CUDA(cudaMemcpyAsync(h_state_, ds, sizeof(CgState), cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    const double bnorm = std::sqrt(h_state_->rr);
    st->bnorm = bnorm;
    CgState init{};
    init.tol2 = tol2_of(opt, bnorm);
    init.max_iter = opt.max_iter;
    FGB_CUDA(cudaMemcpyAsync(ds, &init, sizeof(CgState), cudaMemcpyHostToDevice, stream_));
    FGB_LAUNCH(k_cg_init<double><<<gb, kBlock, 0, stream_>>>(n_, slice_ptr_.get(), slice_len_.get(), sell_col_.get(), sell64_.get(),
                                                  x_.get(), rhs_.get(), dinv64_.get(), r64_.get(), z64_.get(), p64_.get(),
                                                  partial_.get(), ds));
    FGB_CUDA(cudaMemcpyAsync(h_state_, ds, sizeof(CgState), cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    if (!h_state_->done) run_cg(false, ds, opt.max_iter, std::max(1, opt.chunk));
    st->iterations = h_state_->iter;
    const int cg_status = h_state_->status;
    // true residual
    FGB_LAUNCH(k_residual64<<<gb, kBlock, 0, stream_>>>(n_, slice_ptr_.get(), slice_len_.get(), sell_col_.get(), sell64_.get(), x_.get(),
                                             rhs_.get(), r64_.get(), partial_.get(), ds, compensated_residual(opt)));
    FGB_CUDA(cudaMemcpyAsync(h_state_, ds, sizeof(CgState), cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    const double rn = std::sqrt(h_state_->rr);
    st->rel_residual = bnorm > 0 ? rn / bnorm : rn;
    st->status = bnorm == 0 ? 1 : cg_status;
    return st->status >= 1 ? st->iterations : -st->iterations;
}

int FemDevice::solve_mixed(const SolveOptions& opt, SolveStats* st) {
    const int gb = grid_for(n_, kBlock);
    CgState* ds = state_.get();
    FGB_LAUNCH(k_norm2<<<reduce_grid(n_, kBlock), kBlock, 0, stream_>>>(n_, rhs_.get(), partial_.get(), ds));
    FGB_CUDA(cudaMemcpyAsync(h_state_, ds, sizeof(CgState), cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    const double bnorm = std::sqrt(h_state_->rr);
    st->bnorm = bnorm;
    MixedArgs a;
    a.n = n_;
    a.sptr = slice_ptr_.get();
    a.slen = slice_len_.get();
    a.scol = sell_col_.get();
    a.s32 = sell32_.get();
    a.s64 = sell64_.get();
    a.dinv32 = dinv32_.get();
    a.b = rhs_.get();
    a.x = x_.get();
    a.d = d32_.get();
    a.r = r32_.get();
    a.z = z32_.get();
    a.pa = p32_.get();
    a.pb = p32b_.get();
    a.q = q32_.get();
    a.partial = partial_.get();
    a.out = mixed_.get();
    a.tol2 = tol2_of(opt, bnorm);
    a.ru2 = opt.inner_tol * opt.inner_tol;
    a.max_iter = opt.max_iter;
    a.comp = compensated_residual(opt);
    FGB_CUDA(cudaEventRecord(kev0_, stream_));
    launch_mixed_cg(a, stream_);
    FGB_CUDA(cudaEventRecord(kev1_, stream_));
    FGB_CUDA(cudaMemcpyAsync(h_mixed_, mixed_.get(), sizeof(MixedResult), cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    float kms = 0;
    FGB_CUDA(cudaEventElapsedTime(&kms, kev0_, kev1_));
    st->kernel_ms = kms;
    st->iterations = h_mixed_->iterations;
    st->outer = h_mixed_->updates;
    st->status = bnorm == 0 ? 1 : h_mixed_->status;
    st->rel_residual = bnorm > 0 ? std::sqrt(h_mixed_->rr) / bnorm : std::sqrt(h_mixed_->rr);
    return st->status >= 1 ? st->iterations : -st->iterations;
}

void FemDevice::ensure_amg(SolveStats* st) {
    const int anode = anode_dirichlet_ ? 1 : 0;
    if (amg_ && amg_anode_ == anode) return;
    if (fs_.order == 2) {
        build_q2_amg(anode, st);
        return;
    }
    std::vector<double> vals, rhs;
    download_matrix(vals, rhs);
    std::vector<int8_t> fixed(n_, 0);
    for (int d = 0; d < n_; ++d) fixed[d] = fs_.bc_kind[d] == 1 || (anode && fs_.bc_kind[d] == 2);
    AmgOptions ao;
    ao.level0_lambda = estimate_lambda(15, kAmgLambdaSeed);  // the host estimate's start vector
    AmgHost h = build_amg(*pm_, fs_, vals, fixed, ao);
    h.levels[0].cheb_degree = smooth_degree_ > 0 ? smooth_degree_ : 4;
    h.levels[0].cheb_lo = smooth_lo_ > 0 ? smooth_lo_ : 0.04;
    amg_.reset(new AmgDevice(h, stream_, slice_ptr_.get(), slice_len_.get(), sell_col_.get(), sell32_.get(),
                             dinv32_.get()));
    amg_->smoother_timer.enabled = profiling_;
    if (profiling_) amg_->smoother_timer.reserve(4 * kProfiledLaunches);
    amg_anode_ = anode;
    if (st) st->setup_ms = h.setup_ms;
}

double FemDevice::estimate_lambda(int iters, uint64_t seed) {
    ensure_sell();
    // power iteration on D^-1 A from a fixed pseudo-random start, FP64 on the device
    std::vector<double> h(n_);
    uint64_t sd = seed;
    double nx = 0.0;
    for (int i = 0; i < n_; ++i) {
        sd = sd * 6364136223846793005ull + 1442695040888963407ull;
        h[i] = (double)((sd >> 11) & 0xfffff) / 1048576.0 - 0.5;
        nx += h[i] * h[i];
    }
    FGB_CUDA(cudaMemcpyAsync(p64_.get(), h.data(), sizeof(double) * n_, cudaMemcpyHostToDevice, stream_));
    nx = std::sqrt(nx);
    const int gb = grid_for(n_, kBlock);
    CgState* ds = state_.get() + 1;
    double lam = 1.0;
    for (int it = 0; it < iters; ++it) {
        FGB_LAUNCH(k_sell_spmv<double><<<gb, kBlock, 0, stream_>>>(n_, slice_ptr_.get(), slice_len_.get(), sell_col_.get(),
                                                                   sell64_.get(), p64_.get(), q64_.get()));
        FGB_LAUNCH(k_scale_mul<<<gb, kBlock, 0, stream_>>>(n_, q64_.get(), dinv64_.get(), 1.0));
        FGB_LAUNCH(k_norm2<<<reduce_grid(n_, kBlock), kBlock, 0, stream_>>>(n_, q64_.get(), partial_.get(), ds));
        FGB_CUDA(cudaMemcpyAsync(h_state_ + 1, ds, sizeof(CgState), cudaMemcpyDeviceToHost, stream_));
        FGB_CUDA(cudaStreamSynchronize(stream_));
        const double ny = std::sqrt(h_state_[1].rr);
        if (!(ny > 0)) break;
        lam = ny / nx;
        FGB_LAUNCH(k_scale_copy64<<<gb, kBlock, 0, stream_>>>(n_, q64_.get(), 1.0 / ny, p64_.get()));
        nx = 1.0;
    }
    return lam;
}

void FemDevice::build_q2_amg(int anode, SolveStats* st) {
    const auto t0 = std::chrono::steady_clock::now();
    SetupPhases phase("q2 multigrid");
    // coarse operator: the Q1 system of the same mesh and boundary conditions (the Q2 space
    // contains the Q1 space, P below is that embedding, so P^T A2 P equals the Q1 matrix up
    // to the quadrature), with the Q1 hierarchy underneath
    if (!q1_) {
        q1_.reset(new FemDevice(*pm_, q1_fs_.valid() ? q1_fs_.get() : build_fem_structure(*pm_), stream_));
        q1_->q1_gauss_ = 3;
    }
    phase("Q1 structure + upload");
    q1_->setup(applied_field_, applied_potential_);
    q1_->assemble(true, anode != 0);
    std::vector<double> v1, r1;
    q1_->download_matrix(v1, r1);
    phase("Q1 assembly + download");
    const FemStructure& f1 = q1_->structure();
    std::vector<int8_t> fixed1(f1.n_dofs, 0);
    for (int d = 0; d < f1.n_dofs; ++d) fixed1[d] = f1.bc_kind[d] == 1 || (anode && f1.bc_kind[d] == 2);
    AmgOptions ao1;
    ao1.level0_lambda = q1_->estimate_lambda(15, kAmgLambdaSeed);
    // (built on a second host thread while the device worked on the embedding, the hierarchy
    // took longer than the device work saved: two OpenMP teams on the same cores)
    AmgHost h1 = build_amg(*pm_, f1, v1, fixed1, ao1);
    phase("Q1 hierarchy (host)");
    // embedding P (a free Q2 DoF takes the mean of the free Q1 values at its entity's corners)
    // and R = P^T, built on the device from the Q1 DoFs of the cell corners
    DeviceCsr32 Pd, Rd;
    {
        std::vector<int32_t> cq1(8 * (size_t)nc_);
#pragma omp parallel for schedule(static)
        for (int c = 0; c < nc_; ++c) {
            const size_t hex = (size_t)pm_->vac.cells[c];
            for (int k = 0; k < 8; ++k) cq1[8 * (size_t)c + k] = f1.node2dof[pm_->hex.hexs[8 * hex + k]];
        }
        DBuf<int32_t> d_cq1, d_cell;
        DBuf<int8_t> d_loc, d_fixed1;
        d_cq1.upload(cq1, stream_);
        d_cell.upload(fs_.dof_cell, stream_);
        d_loc.upload(fs_.dof_local, stream_);
        d_fixed1.upload(fixed1, stream_);
        q2_embedding(n_, f1.n_dofs, d_cell.get(), d_loc.get(), d_cq1.get(), fixed_.get(), d_fixed1.get(), Pd, Rd,
                     stream_);
    }
    phase("embedding P, R = P^T (device)");
    AmgHost h;
    AmgHostLevel l0;
    l0.A.n_rows = l0.A.n_cols = n_;
    l0.A.ptr.assign(1, fs_.nnz());  // structure lives on the device; nnz for reporting
    l0.lambda = estimate_lambda(15);
    // degree 2 on [0.06, 1.1]: more iterations than degree 3-4 but fewer passes over the big Q2
    // matrix per cycle (1.7e7-DoF Q2 nanotip: 95 iterations / 1.11 s vs 84 / 1.23 s at degree 3);
    // the lower end 0.06 against 0.1: 70 -> 68 iterations on a 2.2e6-DoF tip, 96 on the
    // 1.7e7-DoF one either way
    l0.cheb_degree = smooth_degree_ > 0 ? smooth_degree_ : 2;
    l0.cheb_lo = smooth_lo_ > 0 ? smooth_lo_ : 0.06;
    phase("lambda_max (device)");
    // the Q1 level is the coarse solve of the Q2 level: smooth it harder
    h1.levels[0].cheb_degree = 4;
    h1.levels[0].cheb_lo = 0.04;
    // below it one Chebyshev step per side is enough: the 1.7e7-DoF Q2 nanotip keeps its 96 PCG
    // iterations (618 -> 609 ms per solve); degree 2 or 3 there, or 3 or 6 at the Q1 level,
    // cost more
    for (size_t l = 1; l < h1.levels.size(); ++l) h1.levels[l].cheb_degree = 1;
    h1.levels[0].A.col = f1.col;
    h1.levels[0].A.val = std::move(v1);
    // the Q1 level applies the Q1 system's own device SELL matrix (the same FP32 values and
    // layout the hierarchy would pack and upload)
    h1.levels[0].dev_sptr = q1_->slice_ptr_.get();
    h1.levels[0].dev_slen = q1_->slice_len_.get();
    h1.levels[0].dev_scol = q1_->sell_col_.get();
    h1.levels[0].dev_val = q1_->sell32_.get();
    h1.levels[0].dev_dinv = q1_->dinv32_.get();
    l0.P.n_rows = n_;
    l0.P.n_cols = f1.n_dofs;
    l0.R.n_rows = f1.n_dofs;
    l0.R.n_cols = n_;
    l0.transfers_on_device = true;
    h.levels.push_back(std::move(l0));
    for (auto& lv : h1.levels) h.levels.push_back(std::move(lv));
    h.coarse_inv = std::move(h1.coarse_inv);
    h.n_coarse = h1.n_coarse;
    amg_.reset(new AmgDevice(h, stream_, slice_ptr_.get(), slice_len_.get(), sell_col_.get(), sell32_.get(),
                             dinv32_.get()));
    amg_->adopt_transfers(0, std::move(Pd.ptr), std::move(Pd.col), std::move(Pd.val), std::move(Rd.ptr),
                          std::move(Rd.col), std::move(Rd.val), Pd.nnz);
    if (level0_ebe_) {
        if (ke32_.size() != 378 * (size_t)nc_) refresh_ke32();
        CellBlocksDev& c = *cb_;
        EbeOperator op;
        op.n_cells = nc_;
        op.n_blocks = c.n_blocks;
        op.max_cells = c.max_cells;
        op.max_dofs = c.max_dofs;
        op.n_bnd = c.n_bnd;
        op.n_slots = c.n_slots;
        op.n_local = c.n_local;
        op.ke = ke32_.get();
        op.cell_start = c.cell_start.get();
        op.dof_start = c.dof_start.get();
        op.dof_list = c.dof_list.get();
        op.item_end = c.item_end.get();
        op.slot = c.slot.get();
        op.loc = c.loc.get();
        op.items = c.items.get();
        op.bnd_dofs = c.bnd_dofs.get();
        op.bnd_ptr = c.bnd_ptr.get();
        op.partial = c.partial.get();
        op.fixed = fixed_.get();
        op.n_ke = 378LL * nc_;
        amg_->set_level0_ebe(&op);
        amg_->set_level0_stream(level0_stream_);
        amg_->set_level0_prefetch(level0_prefetch_);
        if (level0_geo_) {
            ensure_geo();
            amg_->set_level0_geo(geo_.get(), geo_built_);
        }
    }
    phase("device hierarchy upload");
    amg_->smoother_timer.enabled = profiling_;
    if (profiling_) amg_->smoother_timer.reserve(4 * kProfiledLaunches);
    amg_anode_ = anode;
    if (st) st->setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void FemDevice::download_pattern(std::vector<int64_t>& rowptr, std::vector<int32_t>& col) {
    if (fs_.order == 1) {
        rowptr = fs_.rowptr;
        col = fs_.col;
        return;
    }
    std::vector<int32_t> sc = sell_col_.to_host(stream_);
    rowptr.assign(n_ + 1, 0);
    for (int r = 0; r < n_; ++r) rowptr[r + 1] = rowptr[r] + fs_.row_len[r];
    col.resize(rowptr[n_]);
    for (int r = 0; r < n_; ++r) {
        const int sl = r / 32, lane = r % 32;
        for (int j = 0; j < fs_.row_len[r]; ++j)
            col[rowptr[r] + j] = sc[fs_.slice_ptr[sl] + ((int64_t)(j / 4) * 32 + lane) * 4 + j % 4];
    }
}

std::string FemDevice::amg_levels() const { return amg_ ? amg_->describe() : std::string(); }

void FemDevice::ensure_split() {
    ensure_sell();
    if (split_valid_) return;
    const long long ne = (long long)fs_.slice_ptr.back();
    sell_lo_.resize(ne);
    FGB_LAUNCH(k_split_lo<<<grid_for(ne, kBlock), kBlock, 0, stream_>>>(ne, sell64_.get(), sell32_.get(), sell_lo_.get()));
    split_valid_ = true;
}

void FemDevice::set_outer_spmv(int mode) {
    FGB_REQUIRE(mode >= 0 && mode <= 2, "outer SpMV mode 0 (FP64), 1 (FP32 pairs) or 2 (cell blocks)");
    FGB_REQUIRE(mode != 2 || fs_.order == 2, "the cell-block outer SpMV is for Q2 fields");
    outer_mode_ = mode;
}

void FemDevice::ensure_cell_blocks() {
    if (cb_) return;
    SetupPhases phase("cell blocks");
    CellBlocks h;
    bool have = false;
    if (cb_host_.valid()) {
        CellBlocks b = cb_host_.get();  // the blocks started at construction
        if (cb_host_cells_ == cb_cells_ && cb_host_dofs_ == cb_max_dofs_) {
            h = std::move(b);
            have = true;
        }
    }
    if (!have) h = build_cell_blocks(fs_, cb_cells_, cb_max_dofs_);
    phase("host build (or wait)");
    auto c = std::make_unique<CellBlocksDev>();
    c->n_blocks = h.n_blocks;
    c->max_cells = h.max_cells;
    c->max_dofs = h.max_dofs;
    c->n_bnd = (int)h.bnd_dofs.size();
    c->n_slots = h.n_slots;
    c->n_local = h.local_entries();
    c->perm.upload(h.perm, stream_);
    c->cell_start.upload(h.cell_start, stream_);
    c->dof_start.upload(h.dof_start, stream_);
    c->dof_list.upload(h.dof_list, stream_);
    c->slot.upload(h.slot, stream_);
    c->bnd_dofs.upload(h.bnd_dofs, stream_);
    c->bnd_ptr.upload(h.bnd_ptr, stream_);
    c->item_end.upload(h.item_end, stream_);
    c->loc.upload(h.loc, stream_);
    c->items.upload(h.items, stream_);
    c->partial.resize(std::max(1, h.n_slots));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    phase("upload");
    cb_ = std::move(c);
}

void FemDevice::refresh_ke32() {
    ensure_cell_blocks();
    ke32_.resize(378 * (size_t)nc_);
    if (outer_mode_ == 2) ke32lo_.resize(378 * (size_t)nc_);
    FGB_LAUNCH(k_ke_cyclic<<<grid_for(378LL * nc_, kBlock), kBlock, 0, stream_>>>(
        378LL * nc_, cb_->perm.get(), ke_.get(), ke32_.get(), outer_mode_ == 2 ? ke32lo_.get() : nullptr));
}

double FemDevice::outer_spmv_bytes() const {
    if (outer_mode_ != 2 || !cb_) return (double)fs_.nnz() * 12.0 + 24.0 * n_;
    // per cell: K_e hi + lo (378 x 8), loc (27 x 2) and items (28 x 2); per block-local DoF: its
    // id, item end, slot, the p pair gathered and the Dirichlet flag; per DoF: q written and p
    // read for p.q; per slot: the pair written and read; per split DoF: its id and slot range
    const CellBlocksDev& c = *cb_;
    return nc_ * (3024.0 + 110.0) + (double)c.n_local * 19.0 + 16.0 * n_ + 16.0 * c.n_slots + 8.0 * c.n_bnd;
}

void FemDevice::set_cell_blocks(int cells_per_block, int max_dofs) {
    FGB_REQUIRE(fs_.order == 2, "cell blocks are for Q2 fields");
    FGB_REQUIRE(cells_per_block >= 1 && cells_per_block <= 256 && max_dofs >= 27 && max_dofs <= 4096,
                "cell blocks: 1..256 hexes and 27..4096 DoFs per block");
    cb_cells_ = cells_per_block;
    cb_max_dofs_ = max_dofs;
    cb_.reset();
    geo_built_ = geo_for_ = 0;  // block order changes: rebuilt on the next use
    geo_.release();
    ke32_.release();
    ke32lo_.release();
    amg_.reset();
}

void FemDevice::set_level0_ebe(bool on) {
    FGB_REQUIRE(!on || fs_.order == 2, "the element-by-element level 0 is for Q2 fields");
    level0_ebe_ = on;
    amg_.reset();
}

void FemDevice::set_smoothing(int degree, double lo) {
    FGB_REQUIRE(degree >= 0 && degree <= 15 && lo >= 0 && lo < 1, "smoothing degree 1..15 and interval 0..1");
    smooth_degree_ = degree;
    smooth_lo_ = lo;
    amg_.reset();
}

void FemDevice::set_ke_tensor(bool on) { ke_tensor_ = on; }

void FemDevice::export_element_matrices(double* out) {
    const size_t n = ke_.size();
    FGB_CUDA(cudaMemcpyAsync(out, ke_.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
}

void FemDevice::set_level0_stream(bool on) {
    level0_stream_ = on;
    if (amg_) amg_->set_level0_stream(on);
}

void FemDevice::ensure_geo() {
    if (geo_built_ && geo_for_ == level0_geo_) return;
    ensure_cell_blocks();
    const bool half = level0_geo_ == 2;
    geo_.resize((size_t)nc_ * (half ? 324 : 648));
    if (geo_max_.size() != 1) geo_max_.resize(1);
    q2_geometric_factors(nc_, cb_->perm.get(), cell_dofs_.get(), dof_xyz_.get(), geo_.get(), half, geo_max_.get(),
                         stream_);
    geo_built_ = level0_geo_;
    geo_for_ = level0_geo_;
    if (half) {
        unsigned h = 0;
        FGB_CUDA(cudaMemcpyAsync(&h, geo_max_.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, stream_));
        FGB_CUDA(cudaStreamSynchronize(stream_));
        float mx;
        std::memcpy(&mx, &h, sizeof(mx));
        if (!(mx < 6.0e4f)) {  // beyond FP16 (max 65504): the FP32 factors instead
            geo_.resize((size_t)nc_ * 648);
            q2_geometric_factors(nc_, cb_->perm.get(), cell_dofs_.get(), dof_xyz_.get(), geo_.get(), false, nullptr,
                                 stream_);
            geo_built_ = 1;
        }
    }
}

int FemDevice::set_level0_operator(int kind) {
    FGB_REQUIRE(kind >= 0 && kind <= 2, "level-0 operator: 0 element matrices, 1 FP32 or 2 FP16 geometric factors");
    FGB_REQUIRE(kind == 0 || fs_.order == 2, "geometric factors are for Q2 fields");
    level0_geo_ = kind;
    if (kind == 0) {
        geo_built_ = geo_for_ = 0;
        geo_.release();
    } else {
        ensure_geo();
    }
    if (amg_ && level0_ebe_) amg_->set_level0_geo(kind ? geo_.get() : nullptr, geo_built_);
    return geo_built_;
}

void FemDevice::set_level0_prefetch(int cells) {
    FGB_REQUIRE(cells >= 0 && cells <= 64, "level-0 prefetch depth: 0 (off) to 64 cells per warp");
    level0_prefetch_ = cells;
    if (amg_) amg_->set_level0_prefetch(cells);
}

void FemDevice::set_coarse_cycles(int level, int cycles) {
    FGB_REQUIRE(level >= 0 && level < 16 && cycles >= 1 && cycles <= 8, "coarse cycles: level 0..15, 1..8 cycles");
    if ((int)coarse_cycles_.size() <= level) coarse_cycles_.resize(level + 1, 1);
    coarse_cycles_[level] = cycles;
}

void FemDevice::set_level_smoothing(int level, int degree, double lo) {
    FGB_REQUIRE(level >= 1 && level < 16 && degree >= 0 && degree <= 15 && lo >= 0 && lo < 1,
                "level smoothing: level 1..15, degree 0..15, interval 0..1");
    if ((int)level_smooth_.size() <= level) level_smooth_.resize(level + 1, {0, 0.0});
    level_smooth_[level] = {degree, lo};
}

void FemDevice::set_profiling(bool on) {
    profiling_ = on;
    spmv_timer_.enabled = on;
    if (on) spmv_timer_.reserve(kProfiledLaunches);
    if (amg_) {
        amg_->smoother_timer.enabled = on;
        if (on) amg_->smoother_timer.reserve(4 * kProfiledLaunches);
    }
}

void FemDevice::prepare_amg(SolveStats* st) {
    ensure_amg(st);
    for (int l = 0; l < (int)coarse_cycles_.size(); ++l) amg_->set_coarse_cycles(l, coarse_cycles_[l]);
    // levels the hierarchy has, short of the dense coarsest one
    for (int l = 1; l < (int)level_smooth_.size() && l + 1 < amg_->n_levels(); ++l)
        amg_->set_level_smoothing(l, level_smooth_[l].first, level_smooth_[l].second);
    st->levels = amg_->n_levels();
}

int FemDevice::solve_amg(const SolveOptions& opt, SolveStats* st) {
    prepare_amg(st);
    const int gb = grid_for(n_, kBlock);
    CgState* ds = state_.get();
    FGB_LAUNCH(k_norm2<<<reduce_grid(n_, kBlock), kBlock, 0, stream_>>>(n_, rhs_.get(), partial_.get(), ds));
    FGB_CUDA(cudaMemcpyAsync(h_state_, ds, sizeof(CgState), cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    const double bb = h_state_->rr, bnorm = std::sqrt(bb);
    st->bnorm = bnorm;
    CgState init{};
    init.tol2 = tol2_of(opt, bnorm);
    init.max_iter = opt.max_iter;
    FGB_CUDA(cudaMemcpyAsync(ds, &init, sizeof(CgState), cudaMemcpyHostToDevice, stream_));
    const int mode = outer_mode_;
    const bool df = mode >= 1;
    CbSpmvArgs ca{};
    int cb_grid = 1;
    size_t cb_smem = 0;
    if (df) {
        if (mode == 1) ensure_split();
        p2_.resize(n_);
    }
    if (mode == 2) {
        ensure_cell_blocks();
        if (ke32_.size() != 378 * (size_t)nc_ || ke32lo_.size() != 378 * (size_t)nc_) refresh_ke32();
        CellBlocksDev& c = *cb_;
        cb_grid = reduce_grid(c.n_bnd, kBlock);
        cb_pair_.resize(std::max(1, c.n_slots));
        cb_dot_.resize((size_t)c.n_blocks + cb_grid);
        cb_smem = cbdf_smem_bytes(c.max_cells, c.max_dofs);
        if (!cb_spmv_attr_) {
            // the cap is a property of the kernel, shared by every mesh: always the largest block's
            FGB_REQUIRE(c.max_cells <= 256 && c.max_dofs <= 4096, "cell blocks too large");
            FGB_CUDA(cudaFuncSetAttribute(k_cb_spmv_df, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)cbdf_smem_bytes(256, 4096)));
            cb_spmv_attr_ = true;
        }
        ca = CbSpmvArgs{c.n_blocks, c.max_cells, c.max_dofs, c.n_bnd, ke32_.get(), ke32lo_.get(), c.cell_start.get(),
                        c.dof_start.get(), c.dof_list.get(), c.slot.get(), c.bnd_dofs.get(), c.bnd_ptr.get(),
                        c.item_end.get(), c.loc.get(), c.items.get(), fixed_.get(), cb_pair_.get(), cb_dot_.get()};
    }
    // true FP64 residual b - A x into r64: the assembled matrix when it is current, else (Q2,
    // not compensated: solve() formed the matrix for every other case) the FP64 element
    // matrices row by row
    const bool cell_residual = !sell_valid_;
    FGB_REQUIRE(!cell_residual || (fs_.order == 2 && !compensated_residual(opt)),
                "true residual without the assembled matrix");
    auto true_residual = [&](double* ff) {
        if (cell_residual) {
            *ff = 0.0;
            return cells_true_residual();
        }
        FGB_LAUNCH(k_residual64<<<gb, kBlock, 0, stream_>>>(n_, slice_ptr_.get(), slice_len_.get(), sell_col_.get(),
                                                           sell64_.get(), x_.get(), rhs_.get(), r64_.get(), partial_.get(),
                                                           ds, compensated_residual(opt)));
        FGB_CUDA(cudaMemcpyAsync(h_state_, ds, sizeof(CgState), cudaMemcpyDeviceToHost, stream_));
        FGB_CUDA(cudaStreamSynchronize(stream_));
        *ff = h_state_->ff;
        return h_state_->rr;
    };
    // r = b - A x, stop if already converged; from the zero vector of setup() (every Dirichlet
    // value zero on this path) r is b itself
    double ff_true = 0.0, rr_true = 0.0;
    if (cell_residual && x_zero_) {
        FGB_CUDA(cudaMemcpyAsync(r64_.get(), rhs_.get(), sizeof(double) * n_, cudaMemcpyDeviceToDevice, stream_));
        rr_true = bb;
    } else {
        rr_true = true_residual(&ff_true);
    }
    int status = 0, it = 0, restarts = 0;
    if (rr_true <= init.tol2 || bnorm == 0) status = 1;
    float2* p2 = df ? p2_.get() : nullptr;
    // Convergence is declared on the FP64 true residual b - A x: when the recursion reports
    // convergence, r is recomputed exactly and CG restarts from it if it is still above the
    // tolerance (the FP32-pair SpMV lets the recursive residual drift by ~2^-48 per term)
    while (status == 0) {
        FGB_LAUNCH(k_to32<<<gb, kBlock, 0, stream_>>>(n_, r64_.get(), r32_.get()));
        const float* z = amg_->vcycle(r32_.get());
        FGB_LAUNCH(k_pcg_start<<<reduce_grid(n_, kBlock), kBlock, 0, stream_>>>(n_, z, r64_.get(), p64_.get(), p2, partial_.get(), ds));
        while (true) {
            spmv_timer_.begin(stream_);
            if (mode == 2) {
                FGB_LAUNCH(k_cb_spmv_df<<<ca.n_blocks, kCbT, cb_smem, stream_>>>(ca, p2, p64_.get(), dinv64_.get(),
                                                                                 q64_.get(), ds));
                FGB_LAUNCH(k_cb_spmv_finish<<<cb_grid, kBlock, 0, stream_>>>(ca, p64_.get(), dinv64_.get(), q64_.get(), ds));
            } else if (df)
                FGB_LAUNCH(k_cg_spmv_pq_df<<<gb, kBlock, 0, stream_>>>(n_, slice_ptr_.get(), slice_len_.get(), sell_col_.get(),
                                                                      sell32_.get(), sell_lo_.get(), p2, p64_.get(),
                                                                      q64_.get(), partial_.get(), ds));
            else
                FGB_LAUNCH(k_cg_spmv_pq<double><<<gb, kBlock, 0, stream_>>>(n_, slice_ptr_.get(), slice_len_.get(),
                                                                            sell_col_.get(), sell64_.get(), p64_.get(),
                                                                            q64_.get(), partial_.get(), ds));
            spmv_timer_.end(stream_);
            FGB_LAUNCH(k_pcg_update<<<reduce_grid(n_, kBlock), kBlock, 0, stream_>>>(n_, x_.get(), r64_.get(), p64_.get(), q64_.get(), r32_.get(),
                                                               partial_.get(), ds));
            FGB_CUDA(cudaMemcpyAsync(h_state_, ds, sizeof(CgState), cudaMemcpyDeviceToHost, stream_));
            FGB_CUDA(cudaStreamSynchronize(stream_));
            it = h_state_->iter;
            if (h_state_->done) {
                status = h_state_->status;
                break;
            }
            const float* zi = amg_->vcycle(r32_.get());
            FGB_LAUNCH(k_pcg_rz<<<reduce_grid(n_, kBlock), kBlock, 0, stream_>>>(n_, zi, r64_.get(), partial_.get(), ds));
            FGB_LAUNCH(k_pcg_direction<<<gb, kBlock, 0, stream_>>>(n_, zi, p64_.get(), p2, ds));
        }
        // true FP64 residual of the current x (also the restart residual)
        rr_true = true_residual(&ff_true);
        // with a compensated residual, a solution within twice the FP64 floor is as converged
        // as FP64 can hold it: success (kStatusFloor), no restart on rounding noise
        const bool at_floor = !cell_residual && compensated_residual(opt) && rr_true <= 4.0 * kFloorScale2 * ff_true;
        if (status == 1 && rr_true > init.tol2 && at_floor) {
            status = kStatusFloor;
            break;
        }
        if (status != 1 || rr_true <= init.tol2 || restarts >= 3 || it >= opt.max_iter) {
            if (status == 1 && rr_true > init.tol2) status = -1;  // recursion converged, x did not
            break;
        }
        ++restarts;
        status = 0;
        CgState again = *h_state_;
        again.done = 0;
        again.status = 0;
        again.ticket = 0;
        FGB_CUDA(cudaMemcpyAsync(ds, &again, sizeof(CgState), cudaMemcpyHostToDevice, stream_));
    }
    st->iterations = it;
    st->outer = restarts;
    const double rn = std::sqrt(rr_true);
    st->rel_residual = bnorm > 0 ? rn / bnorm : rn;
    st->status = bnorm == 0 ? 1 : status;
    if (const unsigned e = amg_->level0_errors())
        throw Error("level-0 smoother: a bounded wait of the streamed element matrices ran out (code " +
                    std::to_string(e) + ")");
    st->smoother_ms = amg_->smoother_timer.collect(&st->smoother_launches);
    st->smoother_bytes = amg_->smoother_bytes();
    st->spmv_ms = spmv_timer_.collect(&st->spmv_launches);
    return st->status >= 1 ? it : -it;
}

// Mixed multigrid solve (precision 3): FP64 iterative refinement around an FP32 CG with the
// level-0 operator of the V-cycle (the FP32 SELL matrix, or for Q2 the matrix-free cell-block
// operator) preconditioned by the V-cycle. Each refinement forms the FP64 residual
// r = b - A x of the assembled system (compensated near the FP64 floor), solves A e = r in
// FP32 to a relative reduction inner_tol (or to what the outer tolerance still needs), and
// adds e to x in FP64. The FP32 operator differs from A by its rounding (and the FP16
// factors' 2^-11), which bounds what one refinement can gain: a few refinements reach 1e-9.
int FemDevice::solve_amg_mixed(const SolveOptions& opt, SolveStats* st) {
    prepare_amg(st);
    const int gb = grid_for(n_, kBlock);
    const int rg = reduce_grid(n_, kBlock);
    CgState* ds = state_.get();
    FGB_LAUNCH(k_norm2<<<rg, kBlock, 0, stream_>>>(n_, rhs_.get(), partial_.get(), ds));
    FGB_CUDA(cudaMemcpyAsync(h_state_, ds, sizeof(CgState), cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    const double bnorm = std::sqrt(h_state_->rr);
    st->bnorm = bnorm;
    const double tol2 = tol2_of(opt, bnorm);
    const int comp = compensated_residual(opt);
    float* r = r32_.get();
    float* p = p32_.get();
    float* q = q32_.get();
    float* e = d32_.get();
    float* zero = z32_.get();
    z32_.zero(stream_);
    // true FP64 residual of x into r64 (and rr, ff in the state)
    auto true_residual = [&]() {
        CgState init{};
        init.tol2 = tol2;
        FGB_CUDA(cudaMemcpyAsync(ds, &init, sizeof(CgState), cudaMemcpyHostToDevice, stream_));
        FGB_LAUNCH(k_residual64<<<gb, kBlock, 0, stream_>>>(n_, slice_ptr_.get(), slice_len_.get(), sell_col_.get(),
                                                           sell64_.get(), x_.get(), rhs_.get(), r64_.get(), partial_.get(),
                                                           ds, comp));
        FGB_CUDA(cudaMemcpyAsync(h_state_, ds, sizeof(CgState), cudaMemcpyDeviceToHost, stream_));
        FGB_CUDA(cudaStreamSynchronize(stream_));
        return *h_state_;
    };
    CgState tr = true_residual();
    double rr_true = tr.rr;
    int status = (rr_true <= tol2 || bnorm == 0) ? 1 : 0, it = 0, refinements = 0, stalled = 0;
    const double eta = std::min(std::max(opt.inner_tol, 1e-6), 0.5);
    while (status == 0) {
        FGB_LAUNCH(k_to32<<<gb, kBlock, 0, stream_>>>(n_, r64_.get(), r));
        FGB_CUDA(cudaMemsetAsync(e, 0, sizeof(float) * n_, stream_));
        CgState in{};
        // the inner residual starts at ||r64||: reduce it by eta, or to half the outer target
        in.tol2 = std::max(eta * eta * rr_true, 0.25 * tol2);
        in.max_iter = std::max(1, opt.max_iter - it);
        FGB_CUDA(cudaMemcpyAsync(ds, &in, sizeof(CgState), cudaMemcpyHostToDevice, stream_));
        const float* z = amg_->vcycle(r);
        FGB_LAUNCH(k_mcg_start<<<rg, kBlock, 0, stream_>>>(n_, z, r, p, partial_.get(), ds));
        int inner_status = 0;
        while (true) {
            spmv_timer_.begin(stream_);
            amg_->level0_residual(zero, p, q);
            spmv_timer_.end(stream_);
            FGB_LAUNCH(k_mcg_pq<<<rg, kBlock, 0, stream_>>>(n_, p, q, partial_.get(), ds));
            FGB_LAUNCH(k_mcg_update<<<rg, kBlock, 0, stream_>>>(n_, e, r, p, q, partial_.get(), ds));
            FGB_CUDA(cudaMemcpyAsync(h_state_, ds, sizeof(CgState), cudaMemcpyDeviceToHost, stream_));
            FGB_CUDA(cudaStreamSynchronize(stream_));
            if (h_state_->done) {
                inner_status = h_state_->status;
                it += h_state_->iter;
                break;
            }
            const float* zi = amg_->vcycle(r);
            FGB_LAUNCH(k_mcg_rz<<<rg, kBlock, 0, stream_>>>(n_, zi, r, partial_.get(), ds));
            FGB_LAUNCH(k_mcg_direction<<<gb, kBlock, 0, stream_>>>(n_, zi, p, ds));
        }
        FGB_LAUNCH(k_add_correction<<<gb, kBlock, 0, stream_>>>(n_, x_.get(), e));
        ++refinements;
        const double rr_prev = rr_true;
        tr = true_residual();
        rr_true = tr.rr;
        if (!(rr_true == rr_true)) { status = -2; break; }
        if (rr_true <= tol2) { status = 1; break; }
        // a solution within twice the FP64 floor is as converged as FP64 can hold it
        if (comp && rr_true <= 4.0 * kFloorScale2 * tr.ff) { status = kStatusFloor; break; }
        if (inner_status == -2 && rr_true >= rr_prev) { status = -2; break; }
        if (it >= opt.max_iter) { status = -1; break; }
        // refinements that no longer halve the residual: the FP32 operator's limit
        stalled = rr_true > 0.25 * rr_prev ? stalled + 1 : 0;
        if (stalled >= 2) { status = -3; break; }
    }
    st->iterations = it;
    st->outer = refinements;
    const double rn = std::sqrt(rr_true);
    st->rel_residual = bnorm > 0 ? rn / bnorm : rn;
    st->status = bnorm == 0 ? 1 : status;
    if (const unsigned er = amg_->level0_errors())
        throw Error("level-0 smoother: a bounded wait of the streamed element matrices ran out (code " +
                    std::to_string(er) + ")");
    st->smoother_ms = amg_->smoother_timer.collect(&st->smoother_launches);
    st->smoother_bytes = amg_->smoother_bytes();
    st->spmv_ms = spmv_timer_.collect(&st->spmv_launches);
    return st->status >= 1 ? it : -it;
}

}  // namespace fgb
