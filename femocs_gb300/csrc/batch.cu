// Batched multigrid-preconditioned CG over many resident meshes (sm_103a). Layout and
// scheduling are described in batch.h.
//
//   kb_spmv_pq     q = A v (FP64 SELL-32), v = x for meshes in phase NEW, p otherwise;
//                  per-mesh p.q -> alpha
//   kb_update      NEW: r = b - q; RUNNING: x += alpha p, r -= alpha q; FP32 copy of r;
//                  per-mesh r.r -> stop test
//   kb_cheb_*      degree-4 Chebyshev smoothing on D^-1 A scaled by 1/lambda_max of the mesh
//                  and level, so one coefficient set serves every mesh
//   kb_residual, kb_csr_apply (restriction / prolongation), kb_dense (coarsest level)
//   kb_rz          per-mesh r.z -> beta (0 and phase RUNNING after a NEW pass)
//   kb_direction   p = z + beta p
//   kb_continue    sets the WHILE condition: any admitted mesh unfinished and under the cap
#include <algorithm>
#include <cmath>
#include <numeric>
#include <sstream>

#include "batch.h"

#include <cooperative_groups.h>
namespace cg = cooperative_groups;
#include "fem_device.h"

namespace fgb {

// ------------------------------------------------------------------ RangePool
size_t RangePool::alloc(size_t n) {
    n = (n + align_ - 1) / align_ * align_;
    if (n == 0) n = align_;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
        if (it->second >= n) {
            const size_t off = it->first, len = it->second;
            free_.erase(it);
            if (len > n) free_[off + n] = len - n;
            used_ += n;
            return off;
        }
    }
    // grow: append at the end of the capacity (merging a free tail)
    size_t off = cap_;
    if (!free_.empty()) {
        auto last = std::prev(free_.end());
        if (last->first + last->second == cap_) {
            off = last->first;
            free_.erase(last);
        }
    }
    const size_t need = off + n;
    size_t nc = std::max<size_t>(cap_ * 2, need);
    nc = (nc + align_ - 1) / align_ * align_;
    if (nc > need) free_[need] = nc - need;
    cap_ = nc;
    used_ += n;
    grew_ = true;
    return off;
}

void RangePool::free(size_t off, size_t n) {
    n = (n + align_ - 1) / align_ * align_;
    if (n == 0) n = align_;
    used_ -= n;
    auto it = free_.emplace(off, n).first;
    if (it != free_.begin()) {
        auto prev = std::prev(it);
        if (prev->first + prev->second == it->first) {
            prev->second += it->second;
            free_.erase(it);
            it = prev;
        }
    }
    auto next = std::next(it);
    if (next != free_.end() && it->first + it->second == next->first) {
        it->second += next->second;
        free_.erase(next);
    }
}

// ------------------------------------------------------------------ device layout
struct BatchLevelDev {
    // rows
    DBuf<int64_t> a_begin, p_begin, r_begin;
    DBuf<int32_t> a_len, p_len, r_len, block_mesh;
    DBuf<float> dinv, b, xa, xb, d, rl;
    // entries
    DBuf<int32_t> a_col, p_col, r_col;
    DBuf<float> a_val, p_val, r_val;
    // level 0: SELL slices, FP64 values, CG vectors, per-block partials
    DBuf<int64_t> s_begin;
    DBuf<int32_t> s_len;
    DBuf<double> v64, x, bb, bunit, r, p, q, partial;
    // work lists: S (smoothed rows), D (dense rows), T (restriction targets = S u D)
    DBuf<int32_t> S, D, T;
    int nS = 0, nD = 0, nT = 0;
};

struct BatchSolver::Dev {
    DBuf<BatchMeshState> st;
    DBuf<int32_t> run;        // running slots
    DBuf<int32_t> counts;     // 3 per level
    DBuf<int32_t> loop;       // [0] iterations in this launch, [1] cap, [2] continue flag
    DBuf<float> dense;
    int* h_loop = nullptr;    // pinned mirror of loop
};

struct BatchSolver::Mesh {
    int slot = -1;
    int n_dofs = 0, n_nodes = 0, depth = 0;
    std::vector<int> row0, nrows, nalloc;           // per level
    size_t e0_off = 0, e0_len = 0;
    std::vector<size_t> a_off, a_len, p_off, p_len, r_off, r_len;
    size_t dense_off = 0, dense_len = 0;
    double bunit_norm = 0;
    std::unique_ptr<DeviceMesh> dm;
    cudaStream_t stream = nullptr;
    DBuf<int32_t> dof2node;
    std::vector<int32_t> h_dof2node;
    BatchSolveResult last;
    bool admitted = false;
};

namespace {

constexpr int kB = kBatchRows;

// Chebyshev smoothing of degree kDeg on [0.04, 1.1] for D^-1 A scaled to lambda_max = 1:
// step k: d_k = c1[k] d_{k-1} + c2[k] D^-1 r, rho_0 = 1/sigma, rho_k = 1/(2 sigma - rho_{k-1})
constexpr int kDeg = 4;
struct Cheb {
    float c1[kDeg], c2[kDeg], inv_theta;
};
Cheb cheb_coefficients() {
    const double lmax = 1.1, lmin = 0.04;
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin), sigma = theta / delta;
    Cheb c{};
    double rho = 1.0 / sigma;
    for (int k = 1; k < kDeg; ++k) {
        const double rn = 1.0 / (2.0 * sigma - rho);
        c.c1[k] = (float)(rn * rho);
        c.c2[k] = (float)(2.0 * rn / delta);
        rho = rn;
    }
    c.inv_theta = (float)(1.0 / theta);
    return c;
}

// --- row kernels
template <typename T>
struct Vec4Of;
template <>
struct Vec4Of<float> {
    __device__ static void load(const float* p, float (&v)[4]) {
        const float4 a = __ldg(reinterpret_cast<const float4*>(p));
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    }
};
template <>
struct Vec4Of<double> {
    __device__ static void load(const double* p, double (&v)[4]) {
        const double2 a = __ldg(reinterpret_cast<const double2*>(p));
        const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    }
};

// one row of the level-0 SELL-32 matrix (4-wide row chunks, 32 rows per slice)
template <typename T>
__device__ __forceinline__ T sell_row_b(int row, const int64_t* __restrict__ sb, const int32_t* __restrict__ sl,
                                        const int32_t* __restrict__ col, const T* __restrict__ val,
                                        const T* __restrict__ x) {
    const int s = row >> 5;
    const int64_t base = sb[s] + (int64_t)(row & 31) * 4;
    const int nch = sl[s] >> 2;
    T acc0 = 0, acc1 = 0;
    int c = 0;
    for (; c + 1 < nch; c += 2) {
        const int64_t o0 = base + (int64_t)c * 128, o1 = o0 + 128;
        const int4 i0 = __ldg(reinterpret_cast<const int4*>(col + o0));
        const int4 i1 = __ldg(reinterpret_cast<const int4*>(col + o1));
        T v0[4], v1[4];
        Vec4Of<T>::load(val + o0, v0);
        Vec4Of<T>::load(val + o1, v1);
        acc0 += v0[0] * __ldg(x + i0.x) + v0[1] * __ldg(x + i0.y) + v0[2] * __ldg(x + i0.z) + v0[3] * __ldg(x + i0.w);
        acc1 += v1[0] * __ldg(x + i1.x) + v1[1] * __ldg(x + i1.y) + v1[2] * __ldg(x + i1.z) + v1[3] * __ldg(x + i1.w);
    }
    if (c < nch) {
        const int64_t o0 = base + (int64_t)c * 128;
        const int4 i0 = __ldg(reinterpret_cast<const int4*>(col + o0));
        T v0[4];
        Vec4Of<T>::load(val + o0, v0);
        acc0 += v0[0] * __ldg(x + i0.x) + v0[1] * __ldg(x + i0.y) + v0[2] * __ldg(x + i0.z) + v0[3] * __ldg(x + i0.w);
    }
    return acc0 + acc1;
}

// Level operator: TPR 0 = SELL (beg/len per slice), else CSR rows (beg/len per row) read by
// TPR lanes of a warp.
struct OpB {
    const int64_t* beg;
    const int32_t* len;
    const int32_t* col;
    const float* val;
};

template <int TPR>
__device__ __forceinline__ float op_row_b(const OpB& A, int row, const float* __restrict__ x) {
    if constexpr (TPR == 0) {
        return sell_row_b<float>(row, A.beg, A.len, A.col, A.val, x);
    } else {
        const int sub = threadIdx.x & (TPR - 1);
        const int64_t b0 = A.beg[row];
        const int64_t end = b0 + A.len[row];
        int64_t k = b0 + sub;
        float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
        for (; k + 3 * TPR < end; k += 4 * TPR) {
            a0 += __ldg(A.val + k) * __ldg(x + A.col[k]);
            a1 += __ldg(A.val + k + TPR) * __ldg(x + A.col[k + TPR]);
            a2 += __ldg(A.val + k + 2 * TPR) * __ldg(x + A.col[k + 2 * TPR]);
            a3 += __ldg(A.val + k + 3 * TPR) * __ldg(x + A.col[k + 3 * TPR]);
        }
        for (; k < end; k += TPR) a0 += __ldg(A.val + k) * __ldg(x + A.col[k]);
        float acc = a0 + (a1 + a2) + a3;
#pragma unroll
        for (int o = TPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        return acc;
    }
}

// whether the work item's mesh is finished (read once per CTA)
__device__ __forceinline__ bool item_done(const BatchMeshState* st, int m) {
    __shared__ int sdone;
    __syncthreads();
    if (threadIdx.x == 0) sdone = ((volatile const BatchMeshState*)st)[m].done;
    __syncthreads();
    return sdone != 0;
}

template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sh) {
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
    __syncthreads();
}

// Per-mesh reduction: the block's partial goes to partial[blk]; the mesh's last block sums
// the mesh's partials in block order and returns true (totals in thread 0).
template <int NV>
__device__ __forceinline__ bool mesh_reduce(double (&v)[NV], double* partial, int blk, BatchMeshState* st) {
    __shared__ double sh[NV * 32];
    __shared__ int last;
    block_sum<NV>(v, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) partial[(size_t)NV * blk + k] = v[k];
        __threadfence();
        const unsigned t = atomicAdd(&st->ticket, 1u);
        last = (t == (unsigned)st->nblk0 - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.0;
    const int b0 = st->blk0, nb = st->nblk0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] += ((volatile double*)partial)[(size_t)NV * (b0 + b) + k];
    block_sum<NV>(acc, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] = acc[k];
        st->ticket = 0;
    }
    return true;
}

// ---- outer FP64 CG over level-0 blocks
__device__ __forceinline__ void kbd_spmv_pq(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                                 const int32_t* __restrict__ bm, BatchMeshState* st,
                                                 const int64_t* __restrict__ sb, const int32_t* __restrict__ sl,
                                                 const int32_t* __restrict__ col, const double* __restrict__ v64,
                                                 const double* __restrict__ x, const double* __restrict__ p,
                                                 double* __restrict__ q, double* partial) {
    const int cnt = *count;
    for (int w = blockIdx.x; w < cnt; w += gridDim.x) {
        const int blk = list[w], m = bm[blk];
        if (item_done(st, m)) continue;
        BatchMeshState* s = st + m;
        const bool fresh = s->phase == 0;
        const double* v = fresh ? x : p;
        const int row = blk * kB + threadIdx.x;
        const double qi = sell_row_b<double>(row, sb, sl, col, v64, v);
        q[row] = qi;
        double acc[1] = {fresh ? 0.0 : p[row] * qi};
        if (mesh_reduce<1>(acc, partial, blk, s) && threadIdx.x == 0 && !fresh) {
            s->alpha = s->rz / acc[0];
        }
    }
}
__global__ void __launch_bounds__(kB, 8) kb_spmv_pq(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                                 const int32_t* __restrict__ bm, BatchMeshState* st,
                                                 const int64_t* __restrict__ sb, const int32_t* __restrict__ sl,
                                                 const int32_t* __restrict__ col, const double* __restrict__ v64,
                                                 const double* __restrict__ x, const double* __restrict__ p,
                                                 double* __restrict__ q, double* partial) {
    kbd_spmv_pq(list, count, bm, st, sb, sl, col, v64, x, p, q, partial);
}

__device__ __forceinline__ void batch_check(BatchMeshState* s, double rr) {
    s->rr = rr;
    if (!(rr == rr)) { s->done = 1; s->status = -2; return; }
    if (rr <= s->tol2) { s->done = 1; s->status = 1; return; }
    if (s->iter >= s->max_iter) { s->done = 1; s->status = -1; }
}

__device__ __forceinline__ void kbd_update(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                                const int32_t* __restrict__ bm, BatchMeshState* st,
                                                double* __restrict__ x, const double* __restrict__ b,
                                                double* __restrict__ r, const double* __restrict__ p,
                                                const double* __restrict__ q, float* __restrict__ r32, double* partial) {
    const int cnt = *count;
    for (int w = blockIdx.x; w < cnt; w += gridDim.x) {
        const int blk = list[w], m = bm[blk];
        if (item_done(st, m)) continue;
        BatchMeshState* s = st + m;
        const bool fresh = s->phase == 0;
        const int row = blk * kB + threadIdx.x;
        double ri;
        if (fresh) {
            ri = b[row] - q[row];
        } else {
            const double a = s->alpha;
            x[row] += a * p[row];
            ri = r[row] - a * q[row];
        }
        r[row] = ri;
        r32[row] = (float)ri;
        double acc[1] = {ri * ri};
        if (mesh_reduce<1>(acc, partial, blk, s) && threadIdx.x == 0) {
            if (!fresh) s->iter += 1;
            batch_check(s, acc[0]);
        }
    }
}
__global__ void __launch_bounds__(kB, 8) kb_update(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                                const int32_t* __restrict__ bm, BatchMeshState* st,
                                                double* __restrict__ x, const double* __restrict__ b,
                                                double* __restrict__ r, const double* __restrict__ p,
                                                const double* __restrict__ q, float* __restrict__ r32, double* partial) {
    kbd_update(list, count, bm, st, x, b, r, p, q, r32, partial);
}

__device__ __forceinline__ void kbd_rz(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                            const int32_t* __restrict__ bm, BatchMeshState* st,
                                            const double* __restrict__ r, const float* __restrict__ z, double* partial) {
    const int cnt = *count;
    for (int w = blockIdx.x; w < cnt; w += gridDim.x) {
        const int blk = list[w], m = bm[blk];
        if (item_done(st, m)) continue;
        BatchMeshState* s = st + m;
        const int row = blk * kB + threadIdx.x;
        double acc[1] = {r[row] * (double)z[row]};
        if (mesh_reduce<1>(acc, partial, blk, s) && threadIdx.x == 0) {
            if (s->phase == 0) {
                s->beta = 0.0;
                s->phase = 1;
            } else {
                s->beta = acc[0] / s->rz;
            }
            s->rz = acc[0];
        }
    }
}
__global__ void __launch_bounds__(kB, 8) kb_rz(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                            const int32_t* __restrict__ bm, BatchMeshState* st,
                                            const double* __restrict__ r, const float* __restrict__ z, double* partial) {
    kbd_rz(list, count, bm, st, r, z, partial);
}

__device__ __forceinline__ void kbd_direction(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                                   const int32_t* __restrict__ bm, BatchMeshState* st,
                                                   const float* __restrict__ z, double* __restrict__ p) {
    const int cnt = *count;
    for (int w = blockIdx.x; w < cnt; w += gridDim.x) {
        const int blk = list[w], m = bm[blk];
        if (item_done(st, m)) continue;
        const double beta = st[m].beta;
        const int row = blk * kB + threadIdx.x;
        p[row] = beta == 0.0 ? (double)z[row] : (double)z[row] + beta * p[row];
    }
}
__global__ void __launch_bounds__(kB, 8) kb_direction(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                                   const int32_t* __restrict__ bm, BatchMeshState* st,
                                                   const float* __restrict__ z, double* __restrict__ p) {
    kbd_direction(list, count, bm, st, z, p);
}

// ---- V-cycle kernels (any level)
__device__ __forceinline__ void kbd_cheb_zero(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                                   const int32_t* __restrict__ bm, BatchMeshState* st,
                                                   const float* __restrict__ dinv, const float* __restrict__ b,
                                                   float* __restrict__ x, float* __restrict__ d, float inv_theta) {
    const int cnt = *count;
    for (int w = blockIdx.x; w < cnt; w += gridDim.x) {
        const int blk = list[w];
        if (item_done(st, bm[blk])) continue;
        const int row = blk * kB + threadIdx.x;
        const float di = dinv[row] * b[row] * inv_theta;
        d[row] = di;
        x[row] = di;
    }
}
__global__ void __launch_bounds__(kB, 8) kb_cheb_zero(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                                   const int32_t* __restrict__ bm, BatchMeshState* st,
                                                   const float* __restrict__ dinv, const float* __restrict__ b,
                                                   float* __restrict__ x, float* __restrict__ d, float inv_theta) {
    kbd_cheb_zero(list, count, bm, st, dinv, b, x, d, inv_theta);
}

// c1 < 0: first step from a nonzero guess (d = c2 D^-1 r)
template <int TPR>
__device__ __forceinline__ void kbd_cheb_step(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                                   const int32_t* __restrict__ bm, BatchMeshState* st, OpB A,
                                                   const float* __restrict__ dinv, const float* __restrict__ b,
                                                   const float* __restrict__ xin, float* __restrict__ xout,
                                                   float* __restrict__ d, float c1, float c2) {
    constexpr int T = TPR == 0 ? 1 : TPR, RPP = kB / T;
    const int cnt = *count;
    for (int w = blockIdx.x; w < cnt; w += gridDim.x) {
        const int blk = list[w];
        if (item_done(st, bm[blk])) continue;
        for (int pass = 0; pass < T; ++pass) {
            const int row = blk * kB + pass * RPP + threadIdx.x / T;
            const float ax = op_row_b<TPR>(A, row, xin);
            if (T == 1 || (threadIdx.x & (T - 1)) == 0) {
                const float di = (c1 < 0.f ? 0.f : c1 * d[row]) + c2 * dinv[row] * (b[row] - ax);
                d[row] = di;
                xout[row] = xin[row] + di;
            }
        }
    }
}
template <int TPR>
__global__ void __launch_bounds__(kB, 8) kb_cheb_step(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                                   const int32_t* __restrict__ bm, BatchMeshState* st, OpB A,
                                                   const float* __restrict__ dinv, const float* __restrict__ b,
                                                   const float* __restrict__ xin, float* __restrict__ xout,
                                                   float* __restrict__ d, float c1, float c2) {
    kbd_cheb_step<TPR>(list, count, bm, st, A, dinv, b, xin, xout, d, c1, c2);
}

template <int TPR>
__device__ __forceinline__ void kbd_residual(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                                  const int32_t* __restrict__ bm, BatchMeshState* st, OpB A,
                                                  const float* __restrict__ b, const float* __restrict__ x,
                                                  float* __restrict__ r) {
    constexpr int T = TPR == 0 ? 1 : TPR, RPP = kB / T;
    const int cnt = *count;
    for (int w = blockIdx.x; w < cnt; w += gridDim.x) {
        const int blk = list[w];
        if (item_done(st, bm[blk])) continue;
        for (int pass = 0; pass < T; ++pass) {
            const int row = blk * kB + pass * RPP + threadIdx.x / T;
            const float ax = op_row_b<TPR>(A, row, x);
            if (T == 1 || (threadIdx.x & (T - 1)) == 0) r[row] = b[row] - ax;
        }
    }
}
template <int TPR>
__global__ void __launch_bounds__(kB, 8) kb_residual(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                                  const int32_t* __restrict__ bm, BatchMeshState* st, OpB A,
                                                  const float* __restrict__ b, const float* __restrict__ x,
                                                  float* __restrict__ r) {
    kbd_residual<TPR>(list, count, bm, st, A, b, x, r);
}

// y = M x (accumulate: y += M x) over the rows of the listed blocks
template <int TPR>
__device__ __forceinline__ void kbd_csr_apply(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                                   const int32_t* __restrict__ bm, BatchMeshState* st, OpB M,
                                                   const float* __restrict__ x, float* __restrict__ y, int accumulate) {
    constexpr int T = TPR == 0 ? 1 : TPR, RPP = kB / T;
    const int cnt = *count;
    for (int w = blockIdx.x; w < cnt; w += gridDim.x) {
        const int blk = list[w];
        if (item_done(st, bm[blk])) continue;
        for (int pass = 0; pass < T; ++pass) {
            const int row = blk * kB + pass * RPP + threadIdx.x / T;
            const float v = op_row_b<TPR == 0 ? 1 : TPR>(M, row, x);
            if (T == 1 || (threadIdx.x & (T - 1)) == 0) y[row] = accumulate ? y[row] + v : v;
        }
    }
}
template <int TPR>
__global__ void __launch_bounds__(kB, 8) kb_csr_apply(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                                   const int32_t* __restrict__ bm, BatchMeshState* st, OpB M,
                                                   const float* __restrict__ x, float* __restrict__ y, int accumulate) {
    kbd_csr_apply<TPR>(list, count, bm, st, M, x, y, accumulate);
}

// coarsest level: x = A_c^-1 b per mesh, one warp per row
__device__ __forceinline__ void kbd_dense(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                               const int32_t* __restrict__ bm, BatchMeshState* st,
                                               const float* __restrict__ dense, const float* __restrict__ b,
                                               float* __restrict__ x) {
    const int cnt = *count;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = kB / 32;
    for (int w = blockIdx.x; w < cnt; w += gridDim.x) {
        const int blk = list[w], m = bm[blk];
        if (item_done(st, m)) continue;
        const int n = st[m].dense_n, r0 = st[m].dense_row0;
        const float* inv = dense + st[m].dense_off;
        for (int i = wid; i < kB; i += nw) {
            const int row = blk * kB + i, li = row - r0;
            float acc = 0.f;
            if (li < n)
                for (int j = lane; j < n; j += 32) acc += __ldg(inv + (size_t)li * n + j) * __ldg(b + r0 + j);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) x[row] = acc;
        }
    }
}
__global__ void __launch_bounds__(kB, 8) kb_dense(const int32_t* __restrict__ list, const int32_t* __restrict__ count,
                                               const int32_t* __restrict__ bm, BatchMeshState* st,
                                               const float* __restrict__ dense, const float* __restrict__ b,
                                               float* __restrict__ x) {
    kbd_dense(list, count, bm, st, dense, b, x);
}

// WHILE condition: continue while an admitted mesh is unfinished and the cap |loop[1]| is not
// reached; a negative loop[1] also stops after an iteration in which an admitted mesh
// finished (meshes finished before the launch are no longer admitted)
__global__ void kb_continue(const int32_t* __restrict__ run, const int32_t* __restrict__ nrun, const BatchMeshState* st,
                            int32_t* loop, cudaGraphConditionalHandle handle, int use_handle) {
    __shared__ int any, fin;
    if (threadIdx.x == 0) any = fin = 0;
    __syncthreads();
    const int n = *nrun;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        if (!st[run[i]].done) any = 1;
        else fin = 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int it = loop[0] + 1;
        loop[0] = it;
        const int cap = loop[1] < 0 ? -loop[1] : loop[1];
        const int go = (any && it < cap && !(loop[1] < 0 && fin)) ? 1 : 0;
        loop[2] = go;
        if (use_handle) cudaGraphSetConditional(handle, go);
    }
}

// ---- the whole batched PCG as one persistent cooperative kernel: the iteration body of
// launch_iteration / vcycle (the same phase bodies in the same order) with a grid-wide
// barrier between phases, iterating until every admitted mesh has finished, the cap is
// reached, or (negative cap) an admitted mesh finished in the last iteration. The phase
// bodies reduce per 256-row block and per mesh in block order, so results are those of the
// graph-captured launches bit for bit.
constexpr int kMaxBatchLevels = 12;
struct KbLevel {
    const int32_t* S;      // smoothed-row blocks
    const int32_t* D;      // dense-level blocks
    const int32_t* T;      // restriction targets
    const int32_t* bm;     // block -> mesh
    const int32_t* cnt;    // counts of S, D, T
    OpB A, R, P;           // level operator, restriction into this level, prolongation into it
    const float* dinv;
    float *b, *xa, *xb, *d, *rl;
    int tpr, r_tpr, p_tpr;
};
struct KbParams {
    int n_levels;
    KbLevel lv[kMaxBatchLevels];
    const int64_t* sb;
    const int32_t* sl;
    const int32_t* col;
    const double* v64;
    double *x, *bb, *r, *p, *q, *partial;
    BatchMeshState* st;
    const float* dense;
    const int32_t* run;
    int32_t* loop;  // [0] iterations, [1] cap (negative: stop after a mesh finished), [2] go, [3] running meshes
    Cheb c;
};

#define FGB_KBD_TPR(FN, tpr, ...)                      \
    do {                                               \
        switch (tpr) {                                 \
            case 0: FN<0>(__VA_ARGS__); break;         \
            case 1: FN<1>(__VA_ARGS__); break;         \
            case 4: FN<4>(__VA_ARGS__); break;         \
            case 8: FN<8>(__VA_ARGS__); break;         \
            case 16: FN<16>(__VA_ARGS__); break;       \
            default: FN<32>(__VA_ARGS__); break;       \
        }                                              \
    } while (0)

__device__ __forceinline__ float* kb_result(const KbLevel& L) { return (kDeg % 2 == 1) ? L.xa : L.xb; }

__global__ void __launch_bounds__(kB) kb_persistent(const __grid_constant__ KbParams P) {
    cg::grid_group grid = cg::this_grid();
    BatchMeshState* st = P.st;
    const int cap_raw = P.loop[1];
    const int cap = cap_raw < 0 ? -cap_raw : cap_raw;
    int it = 0;
    while (true) {
        const KbLevel& L0 = P.lv[0];
        kbd_spmv_pq(L0.S, L0.cnt, L0.bm, st, P.sb, P.sl, P.col, P.v64, P.x, P.p, P.q, P.partial);
        grid.sync();
        kbd_update(L0.S, L0.cnt, L0.bm, st, P.x, P.bb, P.r, P.p, P.q, L0.b, P.partial);
        grid.sync();
        // V-cycle, down: pre-smoothing from zero (step k writes pre_buf(k), the last one xb),
        // residual, restriction, the coarsest solve of the meshes whose dense level is next
        for (int l = 0; l + 1 < P.n_levels; ++l) {
            const KbLevel& L = P.lv[l];
            const KbLevel& C = P.lv[l + 1];
            auto pre_buf = [&](int k) { return ((kDeg - 1 - k) % 2 == 0) ? L.xb : L.xa; };
            kbd_cheb_zero(L.S, L.cnt, L.bm, st, L.dinv, L.b, pre_buf(0), L.d, P.c.inv_theta);
            grid.sync();
            for (int k = 1; k < kDeg; ++k) {
                FGB_KBD_TPR(kbd_cheb_step, L.tpr, L.S, L.cnt, L.bm, st, L.A, L.dinv, L.b, pre_buf(k - 1), pre_buf(k),
                            L.d, P.c.c1[k], P.c.c2[k]);
                grid.sync();
            }
            FGB_KBD_TPR(kbd_residual, L.tpr, L.S, L.cnt, L.bm, st, L.A, L.b, L.xb, L.rl);
            grid.sync();
            FGB_KBD_TPR(kbd_csr_apply, C.r_tpr, C.T, C.cnt + 2, C.bm, st, C.R, L.rl, C.b, 0);
            grid.sync();
            kbd_dense(C.D, C.cnt + 1, C.bm, st, P.dense, C.b, kb_result(C));
            grid.sync();
        }
        // up: prolongation of the coarser result, post-smoothing (even steps write xa, odd xb)
        for (int l = P.n_levels - 2; l >= 0; --l) {
            const KbLevel& L = P.lv[l];
            const KbLevel& C = P.lv[l + 1];
            FGB_KBD_TPR(kbd_csr_apply, L.p_tpr, L.S, L.cnt, L.bm, st, L.P, kb_result(C), L.xb, 1);
            grid.sync();
            float* xin = L.xb;
            for (int k = 0; k < kDeg; ++k) {
                float* xout = (k % 2 == 0) ? L.xa : L.xb;
                FGB_KBD_TPR(kbd_cheb_step, L.tpr, L.S, L.cnt, L.bm, st, L.A, L.dinv, L.b, xin, xout, L.d,
                            k == 0 ? -1.f : P.c.c1[k], k == 0 ? P.c.inv_theta : P.c.c2[k]);
                grid.sync();
                xin = xout;
            }
        }
        kbd_rz(L0.S, L0.cnt, L0.bm, st, P.r, kb_result(L0), P.partial);
        grid.sync();
        kbd_direction(L0.S, L0.cnt, L0.bm, st, kb_result(L0), P.p);
        // every block takes the same decision from the states, which no phase before the next
        // grid barrier changes
        ++it;
        __shared__ int any, fin;
        if (threadIdx.x == 0) any = fin = 0;
        __syncthreads();
        const int n = P.loop[3];
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            if (!((volatile BatchMeshState*)st)[P.run[i]].done) any = 1;
            else fin = 1;
        }
        __syncthreads();
        const bool go = any && it < cap && !(cap_raw < 0 && fin);
        grid.sync();
        if (!go) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.loop[0] = it;
        P.loop[2] = 0;
    }
}

// ---- setup / admission helpers
__global__ void kb_offset_cols(int32_t* __restrict__ col, long long n, int add) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) col[i] += add;
}

__global__ void kb_scale_copy(float* __restrict__ dst, const float* __restrict__ src, int n, float s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i] * s;
}

__global__ void kb_set_rhs(double* __restrict__ b, const double* __restrict__ bunit, int n, double s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = s * bunit[i];
}

// ||b - A x||^2 and ||b||^2 over a row range (one mesh); two-stage deterministic reduction
__global__ void __launch_bounds__(kB) kb_true_residual(int row0, int n, const int64_t* __restrict__ sb,
                                                       const int32_t* __restrict__ sl, const int32_t* __restrict__ col,
                                                       const double* __restrict__ v64, const double* __restrict__ x,
                                                       const double* __restrict__ b, double* __restrict__ part) {
    __shared__ double sh[64];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (i < n) {
        const int row = row0 + i;
        const double ri = b[row] - sell_row_b<double>(row, sb, sl, col, v64, x);
        v[0] = ri * ri;
        v[1] = b[row] * b[row];
    }
    block_sum<2>(v, sh);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = v[0];
        part[2 * blockIdx.x + 1] = v[1];
    }
}

// Work-list kernels walk their list with a fixed grid, every CTA taking an equal share, so
// the grid must be resident in one wave: at most the CTAs of 256 threads that the kernel's
// registers let an SM hold, times the SMs, capped by `cap`. The work-list kernels are built
// for 8 CTAs per SM (32 registers; the level-0 SELL step and residual spill 8 and 4 bytes).
int resident_grid(const void* fn, int cap) {
    static std::mutex mu;
    static std::map<const void*, int> per_sm;
    static int sms = 0;
    std::lock_guard<std::mutex> lk(mu);
    if (!sms) {
        int dev = 0;
        FGB_CUDA(cudaGetDevice(&dev));
        FGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    }
    auto it = per_sm.find(fn);
    if (it == per_sm.end()) {
        int n = 0;
        FGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kB, 0));
        it = per_sm.emplace(fn, std::max(1, n)).first;
    }
    return std::max(1, std::min(cap, it->second * sms));
}
#define FGB_RG(KERNEL, cap) resident_grid((const void*)(KERNEL), (cap))

#define FGB_BATCH_TPR(KERNEL, tpr, grid, stream, ...)                                                 \
    do {                                                                                              \
        switch (tpr) {                                                                                \
            case 0: FGB_LAUNCH(KERNEL<0><<<FGB_RG(KERNEL<0>, grid), kB, 0, stream>>>(__VA_ARGS__)); break;               \
            case 1: FGB_LAUNCH(KERNEL<1><<<FGB_RG(KERNEL<1>, grid), kB, 0, stream>>>(__VA_ARGS__)); break;               \
            case 4: FGB_LAUNCH(KERNEL<4><<<FGB_RG(KERNEL<4>, grid), kB, 0, stream>>>(__VA_ARGS__)); break;               \
            case 8: FGB_LAUNCH(KERNEL<8><<<FGB_RG(KERNEL<8>, grid), kB, 0, stream>>>(__VA_ARGS__)); break;               \
            case 16: FGB_LAUNCH(KERNEL<16><<<FGB_RG(KERNEL<16>, grid), kB, 0, stream>>>(__VA_ARGS__)); break;             \
            default: FGB_LAUNCH(KERNEL<32><<<FGB_RG(KERNEL<32>, grid), kB, 0, stream>>>(__VA_ARGS__)); break;             \
        }                                                                                             \
    } while (0)

int tpr_guess(double avg) {
    if (avg <= 3.0) return 1;
    if (avg <= 8.0) return 4;
    if (avg <= 20.0) return 8;
    if (avg <= 48.0) return 16;
    return 32;
}

size_t round_up(size_t n, size_t a) { return (n + a - 1) / a * a; }

}  // namespace

// ------------------------------------------------------------------ BatchSolver
BatchSolver::BatchSolver(const BatchOptions& opt) : opt_(opt), d_(new Dev) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        throw Error("no CUDA device available: the batched field path runs on the GPU only");
    FGB_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    int dev = 0, sms = 0;
    FGB_CUDA(cudaGetDevice(&dev));
    FGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    grid_ = opt_.grid_ctas > 0 ? opt_.grid_ctas : 8 * sms;
    d_->loop.resize(4);
    d_->loop.zero(stream_);
    FGB_CUDA(cudaMallocHost(&d_->h_loop, 4 * sizeof(int)));
    FGB_CUDA(cudaStreamSynchronize(stream_));
}

void BatchSolver::mark(int k) {
    FGB_REQUIRE(k >= 0 && k < 8, "event index out of range");
    if (!marks_[k]) FGB_CUDA(cudaEventCreate(&marks_[k]));
    FGB_CUDA(cudaEventRecord(marks_[k], stream_));
}

float BatchSolver::elapsed_ms(int a, int b) {
    FGB_REQUIRE(a >= 0 && a < 8 && b >= 0 && b < 8 && marks_[a] && marks_[b], "events not recorded");
    FGB_CUDA(cudaEventSynchronize(marks_[b]));
    float ms = 0;
    FGB_CUDA(cudaEventElapsedTime(&ms, marks_[a], marks_[b]));
    return ms;
}

BatchSolver::~BatchSolver() {
    for (cudaEvent_t e : marks_)
        if (e) cudaEventDestroy(e);
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    for (auto& m : meshes_)
        if (m) {
            m->dm.reset();
            if (m->stream) cudaStreamDestroy(m->stream);
        }
    if (d_ && d_->h_loop) cudaFreeHost(d_->h_loop);
    lv_.clear();
    d_.reset();
    if (stream_) cudaStreamDestroy(stream_);
}

size_t BatchSolver::estimate_bytes(long long n_dofs, long long n_hexs) {
    // level 0: ~25 nonzeros per row at 16 B (FP64 + FP32 value, column) plus 72 B of vectors;
    // coarse levels and transfers ~15%; interpolator ~ 400 B per hex; the temporary
    // assembly system ~ 700 B per dof
    return (size_t)(n_dofs * (25 * 16 + 72) * 1.15 + n_hexs * 400.0 + n_dofs * 700.0);
}

int BatchSolver::n_dofs(int slot) const { return meshes_.at(slot)->n_dofs; }
int BatchSolver::n_nodes(int slot) const { return meshes_.at(slot)->n_nodes; }
int BatchSolver::levels(int slot) const { return meshes_.at(slot)->depth + 1; }
DeviceMesh& BatchSolver::interp(int slot) { return *meshes_.at(slot)->dm; }
cudaStream_t BatchSolver::slot_stream(int slot) { return meshes_.at(slot)->stream; }

long long BatchSolver::total_rows() const {
    long long t = 0;
    for (auto& m : meshes_)
        if (m) t += m->n_dofs;
    return t;
}

size_t BatchSolver::device_bytes() const {
    size_t t = 0;
    for (auto& L : lv_) {
        t += L->a_begin.bytes() + L->p_begin.bytes() + L->r_begin.bytes() + L->a_len.bytes() + L->p_len.bytes() +
             L->r_len.bytes() + L->block_mesh.bytes() + L->dinv.bytes() + 5 * L->b.bytes() + L->a_col.bytes() +
             L->p_col.bytes() + L->r_col.bytes() + L->a_val.bytes() + L->p_val.bytes() + L->r_val.bytes() +
             L->s_begin.bytes() + L->s_len.bytes() + L->v64.bytes() + 6 * L->x.bytes() + L->partial.bytes();
    }
    return t + d_->dense.bytes();
}

std::string BatchSolver::tuning() const {
    std::ostringstream o;
    for (size_t l = 0; l < lv_.size(); ++l)
        o << (l ? " " : "") << "L" << l << ":A" << (l == 0 ? std::string("sell") : std::to_string(l < tpr_.size() ? tpr_[l] : -1)) << ",P"
          << (l < p_tpr_.size() ? p_tpr_[l] : -1) << ",R" << (l < r_tpr_.size() ? r_tpr_[l] : -1);
    return o.str();
}

// grow the device arrays of every level to their pools' capacities
void BatchSolver::ensure_capacity() {
    bool grew = rows0_entries_.grew() || dense_pool_.grew();
    for (size_t l = 0; l < lv_.size(); ++l)
        grew = grew || row_pools_[l]->grew() || a_pools_[l]->grew() || p_pools_[l]->grew() || r_pools_[l]->grew();
    if (!grew && !dirty_) return;
    cudaStream_t s = stream_;
    for (size_t l = 0; l < lv_.size(); ++l) {
        BatchLevelDev& L = *lv_[l];
        const size_t R = row_pools_[l]->capacity();
        L.p_begin.grow(R, s); L.p_len.grow(R, s);
        L.r_begin.grow(R, s); L.r_len.grow(R, s);
        L.a_begin.grow(R, s); L.a_len.grow(R, s);
        L.dinv.grow(R, s); L.b.grow(R, s); L.xa.grow(R, s); L.xb.grow(R, s); L.d.grow(R, s); L.rl.grow(R, s);
        L.block_mesh.grow(std::max<size_t>(1, R / kB), s);
        L.S.grow(std::max<size_t>(1, R / kB), s);
        L.D.grow(std::max<size_t>(1, R / kB), s);
        L.T.grow(std::max<size_t>(1, R / kB), s);
        const size_t A = l == 0 ? rows0_entries_.capacity() : a_pools_[l]->capacity();
        L.a_col.grow(std::max<size_t>(4, A), s);
        L.a_val.grow(std::max<size_t>(4, A), s);
        L.p_col.grow(std::max<size_t>(1, p_pools_[l]->capacity()), s);
        L.p_val.grow(std::max<size_t>(1, p_pools_[l]->capacity()), s);
        L.r_col.grow(std::max<size_t>(1, r_pools_[l]->capacity()), s);
        L.r_val.grow(std::max<size_t>(1, r_pools_[l]->capacity()), s);
        if (l == 0) {
            L.s_begin.grow(std::max<size_t>(1, R / 32), s);
            L.s_len.grow(std::max<size_t>(1, R / 32), s);
            L.v64.grow(std::max<size_t>(4, A), s);
            L.x.grow(R, s); L.bb.grow(R, s); L.bunit.grow(R, s); L.r.grow(R, s); L.p.grow(R, s); L.q.grow(R, s);
            L.partial.grow(std::max<size_t>(2, 2 * (R / kB)), s);
        }
        row_pools_[l]->clear_grew(); a_pools_[l]->clear_grew(); p_pools_[l]->clear_grew(); r_pools_[l]->clear_grew();
    }
    rows0_entries_.clear_grew();
    d_->dense.grow(std::max<size_t>(1, dense_pool_.capacity()), s);
    dense_pool_.clear_grew();
    d_->counts.grow(3 * std::max<size_t>(1, lv_.size()), s);
    d_->st.grow(std::max<size_t>(16, meshes_.size()), s);
    d_->run.grow(std::max<size_t>(16, meshes_.size()), s);
    dirty_ = true;
}

void BatchSolver::place(Mesh& m, const FemStructure& fs, FemDevice& fem, const AmgHost& h) {
    const int depth = (int)h.levels.size() - 1;
    FGB_REQUIRE(depth >= 1, "the multigrid hierarchy has no coarse level");
    m.depth = depth;
    while ((int)lv_.size() < depth + 1) {
        lv_.emplace_back(new BatchLevelDev);
        row_pools_.emplace_back(new RangePool(kB));
        a_pools_.emplace_back(new RangePool(4));
        p_pools_.emplace_back(new RangePool(4));
        r_pools_.emplace_back(new RangePool(4));
        tpr_.push_back(1); p_tpr_.push_back(1); r_tpr_.push_back(1);
        dirty_ = true;
    }
    max_levels_ = std::max(max_levels_, depth + 1);
    m.row0.assign(depth + 1, 0); m.nrows.assign(depth + 1, 0); m.nalloc.assign(depth + 1, 0);
    m.a_off.assign(depth + 1, 0); m.a_len.assign(depth + 1, 0);
    m.p_off.assign(depth + 1, 0); m.p_len.assign(depth + 1, 0);
    m.r_off.assign(depth + 1, 0); m.r_len.assign(depth + 1, 0);
    for (int l = 0; l <= depth; ++l) {
        m.nrows[l] = l == 0 ? fs.n_dofs : h.levels[l].A.n_rows;
        m.nalloc[l] = (int)round_up(std::max(1, m.nrows[l]), kB);
        m.row0[l] = (int)row_pools_[l]->alloc(m.nalloc[l]);
        FGB_REQUIRE((long long)m.row0[l] + m.nalloc[l] < (1LL << 31), "batch row space exceeds 2^31 rows");
    }
    m.e0_len = (size_t)fs.slice_ptr.back();
    m.e0_off = rows0_entries_.alloc(m.e0_len);
    for (int l = 1; l < depth; ++l) {
        m.a_len[l] = (size_t)h.levels[l].A.nnz();
        m.a_off[l] = a_pools_[l]->alloc(m.a_len[l]);
    }
    for (int l = 0; l < depth; ++l) {
        m.p_len[l] = (size_t)h.levels[l].P.nnz();
        m.p_off[l] = p_pools_[l]->alloc(m.p_len[l]);
        m.r_len[l + 1] = (size_t)h.levels[l].R.nnz();
        m.r_off[l + 1] = r_pools_[l + 1]->alloc(m.r_len[l + 1]);
    }
    const int nd = h.n_coarse;
    m.dense_len = (size_t)nd * nd;
    m.dense_off = dense_pool_.alloc(m.dense_len);
    ensure_capacity();

    cudaStream_t s = stream_;
    auto up = [&](auto& buf, size_t off, const auto& vec) {
        if (!vec.empty())
            FGB_CUDA(cudaMemcpyAsync(buf.get() + off, vec.data(), vec.size() * sizeof(vec[0]), cudaMemcpyHostToDevice, s));
    };
    // ---- level 0: SELL slices, FP64/FP32 values, columns shifted into the batch row space
    {
        BatchLevelDev& L = *lv_[0];
        const int r0 = m.row0[0], ns = (int)fs.slice_len.size(), nsa = m.nalloc[0] / 32;
        std::vector<int64_t> sb(nsa, (int64_t)m.e0_off);
        std::vector<int32_t> sl(nsa, 0);
        for (int q = 0; q < ns; ++q) {
            sb[q] = (int64_t)m.e0_off + fs.slice_ptr[q];
            sl[q] = fs.slice_len[q];
        }
        up(L.s_begin, r0 / 32, sb);
        up(L.s_len, r0 / 32, sl);
        FGB_CUDA(cudaMemcpyAsync(L.v64.get() + m.e0_off, fem.d_sell64(), m.e0_len * sizeof(double), cudaMemcpyDeviceToDevice, s));
        FGB_CUDA(cudaMemcpyAsync(L.a_val.get() + m.e0_off, fem.d_sell32(), m.e0_len * sizeof(float), cudaMemcpyDeviceToDevice, s));
        FGB_CUDA(cudaMemcpyAsync(L.a_col.get() + m.e0_off, fem.d_sell_col(), m.e0_len * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
        FGB_LAUNCH(kb_offset_cols<<<grid_for((long long)m.e0_len, kB), kB, 0, s>>>(L.a_col.get() + m.e0_off, (long long)m.e0_len, r0));
        const size_t na = m.nalloc[0];
        FGB_CUDA(cudaMemsetAsync(L.bunit.get() + r0, 0, na * sizeof(double), s));
        FGB_CUDA(cudaMemcpyAsync(L.bunit.get() + r0, fem.d_rhs(), fs.n_dofs * sizeof(double), cudaMemcpyDeviceToDevice, s));
        FGB_CUDA(cudaMemsetAsync(L.dinv.get() + r0, 0, na * sizeof(float), s));
        FGB_LAUNCH(kb_scale_copy<<<grid_for(fs.n_dofs, kB), kB, 0, s>>>(L.dinv.get() + r0, fem.d_dinv32(), fs.n_dofs,
                                                                         (float)(1.0 / h.levels[0].lambda)));
        for (DBuf<double>* v : {&L.x, &L.bb, &L.r, &L.p, &L.q})
            FGB_CUDA(cudaMemsetAsync(v->get() + r0, 0, na * sizeof(double), s));
        for (DBuf<float>* v : {&L.b, &L.xa, &L.xb, &L.d, &L.rl})
            FGB_CUDA(cudaMemsetAsync(v->get() + r0, 0, na * sizeof(float), s));
    }
    // ---- per level: operator (CSR, levels 1..depth-1), prolongation rows, restriction rows
    for (int l = 0; l <= depth; ++l) {
        BatchLevelDev& L = *lv_[l];
        const int r0 = m.row0[l], n = m.nrows[l], na = m.nalloc[l];
        std::vector<int32_t> bmv(na / kB, m.slot);
        up(L.block_mesh, r0 / kB, bmv);
        if (l >= 1) {
            for (DBuf<float>* v : {&L.b, &L.xa, &L.xb, &L.d, &L.rl, &L.dinv})
                FGB_CUDA(cudaMemsetAsync(v->get() + r0, 0, na * sizeof(float), s));
        }
        if (l >= 1 && l < depth) {
            const CsrD& A = h.levels[l].A;
            std::vector<int64_t> beg(na, (int64_t)m.a_off[l]);
            std::vector<int32_t> len(na, 0), col(A.nnz());
            std::vector<float> val(A.nnz()), dinv(na, 0.f);
            const double lam = h.levels[l].lambda;
            for (int i = 0; i < n; ++i) {
                beg[i] = (int64_t)m.a_off[l] + A.ptr[i];
                len[i] = (int32_t)(A.ptr[i + 1] - A.ptr[i]);
                for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
                    col[k] = A.col[k] + r0;
                    val[k] = (float)A.val[k];
                    if (A.col[k] == i) dinv[i] = (float)(1.0 / (A.val[k] * lam));
                }
            }
            up(L.a_begin, r0, beg); up(L.a_len, r0, len);
            up(L.a_col, m.a_off[l], col); up(L.a_val, m.a_off[l], val);
            up(L.dinv, r0, dinv);
        }
        if (l < depth) {
            // prolongation rows at this level, columns in level l+1
            const CsrD& P = h.levels[l].P;
            const int c0 = m.row0[l + 1];
            std::vector<int64_t> beg(na, (int64_t)m.p_off[l]);
            std::vector<int32_t> len(na, 0), col(P.nnz());
            std::vector<float> val(P.nnz());
            for (int i = 0; i < n; ++i) {
                beg[i] = (int64_t)m.p_off[l] + P.ptr[i];
                len[i] = (int32_t)(P.ptr[i + 1] - P.ptr[i]);
            }
            for (int64_t k = 0; k < P.nnz(); ++k) { col[k] = P.col[k] + c0; val[k] = (float)P.val[k]; }
            up(L.p_begin, r0, beg); up(L.p_len, r0, len);
            up(L.p_col, m.p_off[l], col); up(L.p_val, m.p_off[l], val);
        }
        if (l >= 1) {
            // restriction rows at this level, columns in level l-1
            const CsrD& R = h.levels[l - 1].R;
            const int c0 = m.row0[l - 1];
            std::vector<int64_t> beg(na, (int64_t)m.r_off[l]);
            std::vector<int32_t> len(na, 0), col(R.nnz());
            std::vector<float> val(R.nnz());
            for (int i = 0; i < n; ++i) {
                beg[i] = (int64_t)m.r_off[l] + R.ptr[i];
                len[i] = (int32_t)(R.ptr[i + 1] - R.ptr[i]);
            }
            for (int64_t k = 0; k < R.nnz(); ++k) { col[k] = R.col[k] + c0; val[k] = (float)R.val[k]; }
            up(L.r_begin, r0, beg); up(L.r_len, r0, len);
            up(L.r_col, m.r_off[l], col); up(L.r_val, m.r_off[l], val);
        }
    }
    {
        std::vector<float> inv(h.coarse_inv.begin(), h.coarse_inv.end());
        up(d_->dense, m.dense_off, inv);
    }
    BatchMeshState st{};
    st.done = 1;
    st.status = 0;
    st.blk0 = m.row0[0] / kB;
    st.nblk0 = m.nalloc[0] / kB;
    st.depth = depth;
    st.dense_n = nd;
    st.dense_off = (long long)m.dense_off;
    st.dense_row0 = m.row0[depth];
    FGB_CUDA(cudaMemcpyAsync(d_->st.get() + m.slot, &st, sizeof(st), cudaMemcpyHostToDevice, s));
    FGB_CUDA(cudaStreamSynchronize(s));
    if ((int)h_state_.size() <= m.slot) h_state_.resize(m.slot + 1);
    h_state_[m.slot] = st;
}

int BatchSolver::add_mesh(std::shared_ptr<const PreparedMesh> pm, size_t hbm_reserve) {
    FemStructure fs0 = build_fem_structure(*pm);
    {
        size_t fr = 0, tot = 0;
        FGB_CUDA(cudaMemGetInfo(&fr, &tot));
        if (fr < estimate_bytes(fs0.n_dofs, pm->hex.n_hexs()) + hbm_reserve) return -1;
    }
    cudaStream_t ms = nullptr;
    FGB_CUDA(cudaStreamCreateWithFlags(&ms, cudaStreamNonBlocking));
    auto mesh = std::make_unique<Mesh>();
    mesh->stream = ms;
    try {
        auto fem = std::make_unique<FemDevice>(*pm, std::move(fs0), ms);
        const FemStructure& fs = fem->structure();
        fem->setup(1.0, 0.0);  // unit Neumann value: b = -E0 * bunit for an applied field E0
        fem->assemble(true, false);
        std::vector<double> vals, rhs;
        fem->download_matrix(vals, rhs);
        std::vector<int8_t> fixed(fs.n_dofs, 0);
        for (int d = 0; d < fs.n_dofs; ++d) fixed[d] = fs.bc_kind[d] == 1;
        AmgHost h = build_amg(*pm, fs, vals, fixed);
        double bn = 0;
        for (double v : rhs) bn += v * v;
        mesh->bunit_norm = std::sqrt(bn);
        mesh->n_dofs = fs.n_dofs;
        mesh->n_nodes = pm->hex.n_nodes();
        mesh->h_dof2node = fs.dof2node;
        mesh->dof2node.upload(fs.dof2node, ms);
        mesh->dm.reset(new DeviceMesh(*pm, ms));
        FGB_CUDA(cudaStreamSynchronize(ms));
        std::lock_guard<std::mutex> lk(mu_);
        int slot = -1;
        for (size_t i = 0; i < meshes_.size(); ++i)
            if (!meshes_[i]) { slot = (int)i; break; }
        if (slot < 0) {
            slot = (int)meshes_.size();
            meshes_.emplace_back();
        }
        mesh->slot = slot;
        if (d_->st.size() < meshes_.size()) dirty_ = true;
        place(*mesh, fs, *fem, h);
        meshes_[slot] = std::move(mesh);
        lists_dirty_ = true;
        return slot;
    } catch (...) {
        mesh->dm.reset();
        cudaStreamDestroy(ms);
        mesh->stream = nullptr;
        throw;
    }
}

void BatchSolver::remove_mesh(int slot) {
    std::lock_guard<std::mutex> lk(mu_);
    FGB_REQUIRE(slot >= 0 && slot < (int)meshes_.size() && meshes_[slot], "no mesh in this batch slot");
    FGB_REQUIRE(std::find(running_.begin(), running_.end(), slot) == running_.end(), "the mesh has a solve in flight");
    Mesh& m = *meshes_[slot];
    FGB_CUDA(cudaStreamSynchronize(m.stream));
    for (int l = 0; l <= m.depth; ++l) {
        // blocks of a freed range must not point at the slot any more
        std::vector<int32_t> bmv(m.nalloc[l] / kB, -1);
        FGB_CUDA(cudaMemcpyAsync(lv_[l]->block_mesh.get() + m.row0[l] / kB, bmv.data(), bmv.size() * sizeof(int32_t),
                                 cudaMemcpyHostToDevice, stream_));
        row_pools_[l]->free(m.row0[l], m.nalloc[l]);
        if (m.a_len[l]) a_pools_[l]->free(m.a_off[l], m.a_len[l]);
        if (l < m.depth) p_pools_[l]->free(m.p_off[l], m.p_len[l]);
        if (l >= 1) r_pools_[l]->free(m.r_off[l], m.r_len[l]);
    }
    rows0_entries_.free(m.e0_off, m.e0_len);
    dense_pool_.free(m.dense_off, m.dense_len);
    FGB_CUDA(cudaStreamSynchronize(stream_));
    m.dm.reset();
    cudaStreamDestroy(m.stream);
    meshes_[slot].reset();
    lists_dirty_ = true;
}

void BatchSolver::admit(int slot, double E0, double rel_tol, int max_iter) {
    std::lock_guard<std::mutex> lk(mu_);
    FGB_REQUIRE(slot >= 0 && slot < (int)meshes_.size() && meshes_[slot], "no mesh in this batch slot");
    FGB_REQUIRE(std::find(running_.begin(), running_.end(), slot) == running_.end(), "the mesh has a solve in flight");
    FGB_REQUIRE(max_iter >= 1, "max_iter must be positive");
    Mesh& m = *meshes_[slot];
    BatchLevelDev& L = *lv_[0];
    FGB_CUDA(cudaStreamSynchronize(m.stream));  // post-processing of the previous solve done
    FGB_LAUNCH(kb_set_rhs<<<grid_for(m.n_dofs, kB), kB, 0, stream_>>>(L.bb.get() + m.row0[0], L.bunit.get() + m.row0[0],
                                                                     m.n_dofs, -E0));
    BatchMeshState st = h_state_[slot];
    const double bnorm = std::fabs(E0) * m.bunit_norm;
    st.bnorm = bnorm;
    st.tol2 = (rel_tol * bnorm) * (rel_tol * bnorm);
    st.iter = 0;
    st.max_iter = max_iter;
    st.done = bnorm == 0.0 ? 1 : 0;
    st.status = bnorm == 0.0 ? 1 : 0;
    st.phase = 0;
    st.ticket = 0;
    st.rz = st.alpha = st.beta = st.rr = 0.0;
    h_state_[slot] = st;
    FGB_CUDA(cudaMemcpyAsync(d_->st.get() + slot, &h_state_[slot], sizeof(st), cudaMemcpyHostToDevice, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    running_.push_back(slot);
    m.admitted = true;
    lists_dirty_ = true;
}

void BatchSolver::rebuild_lists() {
    const int NL = (int)lv_.size();
    std::vector<std::vector<int32_t>> S(NL), D(NL), T(NL);
    for (int slot : running_) {
        const Mesh& m = *meshes_[slot];
        for (int l = 0; l <= m.depth; ++l) {
            const int b0 = m.row0[l] / kB, nb = m.nalloc[l] / kB;
            for (int b = 0; b < nb; ++b) {
                if (l < m.depth) S[l].push_back(b0 + b);
                else D[l].push_back(b0 + b);
                T[l].push_back(b0 + b);
            }
        }
    }
    std::vector<int32_t> counts(3 * std::max(1, NL), 0);
    for (int l = 0; l < NL; ++l) {
        BatchLevelDev& L = *lv_[l];
        std::sort(S[l].begin(), S[l].end());
        std::sort(D[l].begin(), D[l].end());
        std::sort(T[l].begin(), T[l].end());
        auto upl = [&](DBuf<int32_t>& buf, const std::vector<int32_t>& v) {
            if (!v.empty())
                FGB_CUDA(cudaMemcpyAsync(buf.get(), v.data(), v.size() * sizeof(int32_t), cudaMemcpyHostToDevice, stream_));
        };
        upl(L.S, S[l]); upl(L.D, D[l]); upl(L.T, T[l]);
        L.nS = (int)S[l].size(); L.nD = (int)D[l].size(); L.nT = (int)T[l].size();
        counts[3 * l] = L.nS; counts[3 * l + 1] = L.nD; counts[3 * l + 2] = L.nT;
    }
    FGB_CUDA(cudaMemcpyAsync(d_->counts.get(), counts.data(), counts.size() * sizeof(int32_t), cudaMemcpyHostToDevice, stream_));
    std::vector<int32_t> run(running_.begin(), running_.end());
    const int nrun = (int)run.size();
    if (nrun) FGB_CUDA(cudaMemcpyAsync(d_->run.get(), run.data(), nrun * sizeof(int32_t), cudaMemcpyHostToDevice, stream_));
    // the running count lives after the three per-level counts of the last level
    h_nrun_ = nrun;
    FGB_CUDA(cudaMemcpyAsync(d_->loop.get() + 3, &h_nrun_, sizeof(int32_t), cudaMemcpyHostToDevice, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    lists_dirty_ = false;
}

// Result of a level's cycle (smoothed or dense): xa for an odd smoothing degree, else xb, so
// meshes that end at different levels share one buffer per level.
static float* level_result(BatchLevelDev& L) { return (kDeg % 2 == 1) ? L.xa.get() : L.xb.get(); }

void BatchSolver::vcycle(int l) {
    BatchLevelDev& L = *lv_[l];
    BatchMeshState* st = d_->st.get();
    const int32_t* cS = d_->counts.get() + 3 * l;
    const Cheb c = cheb_coefficients();
    const int tpr = l == 0 ? 0 : tpr_[l];
    const OpB A = l == 0 ? OpB{L.s_begin.get(), L.s_len.get(), L.a_col.get(), L.a_val.get()}
                         : OpB{L.a_begin.get(), L.a_len.get(), L.a_col.get(), L.a_val.get()};
    // pre-smoothing from zero; step k writes pre_buf(k), the last one xb
    auto pre_buf = [&](int k) { return ((kDeg - 1 - k) % 2 == 0) ? L.xb.get() : L.xa.get(); };
    FGB_LAUNCH(kb_cheb_zero<<<FGB_RG(kb_cheb_zero, grid_), kB, 0, stream_>>>(L.S.get(), cS, L.block_mesh.get(), st, L.dinv.get(), L.b.get(),
                                                       pre_buf(0), L.d.get(), c.inv_theta));
    for (int k = 1; k < kDeg; ++k)
        FGB_BATCH_TPR(kb_cheb_step, tpr, grid_, stream_, L.S.get(), cS, L.block_mesh.get(), st, A, L.dinv.get(),
                      L.b.get(), pre_buf(k - 1), pre_buf(k), L.d.get(), c.c1[k], c.c2[k]);
    FGB_BATCH_TPR(kb_residual, tpr, grid_, stream_, L.S.get(), cS, L.block_mesh.get(), st, A, L.b.get(), L.xb.get(),
                  L.rl.get());
    BatchLevelDev& C = *lv_[l + 1];
    const int32_t* cC = d_->counts.get() + 3 * (l + 1);
    const OpB R{C.r_begin.get(), C.r_len.get(), C.r_col.get(), C.r_val.get()};
    FGB_BATCH_TPR(kb_csr_apply, r_tpr_[l + 1], grid_, stream_, C.T.get(), cC + 2, C.block_mesh.get(), st, R, L.rl.get(),
                  C.b.get(), 0);
    FGB_LAUNCH(kb_dense<<<FGB_RG(kb_dense, grid_), kB, 0, stream_>>>(C.D.get(), cC + 1, C.block_mesh.get(), st, d_->dense.get(), C.b.get(),
                                                   level_result(C)));
    if (l + 2 < max_levels_) vcycle(l + 1);
    const OpB P{L.p_begin.get(), L.p_len.get(), L.p_col.get(), L.p_val.get()};
    FGB_BATCH_TPR(kb_csr_apply, p_tpr_[l], grid_, stream_, L.S.get(), cS, L.block_mesh.get(), st, P, level_result(C),
                  L.xb.get(), 1);
    // post-smoothing (same polynomial) from the corrected xb: even steps write xa, odd ones xb
    float* xin = L.xb.get();
    for (int k = 0; k < kDeg; ++k) {
        float* xout = (k % 2 == 0) ? L.xa.get() : L.xb.get();
        FGB_BATCH_TPR(kb_cheb_step, tpr, grid_, stream_, L.S.get(), cS, L.block_mesh.get(), st, A, L.dinv.get(),
                      L.b.get(), xin, xout, L.d.get(), k == 0 ? -1.f : c.c1[k], k == 0 ? c.inv_theta : c.c2[k]);
        xin = xout;
    }
}

void BatchSolver::launch_iteration() {
    BatchLevelDev& L = *lv_[0];
    BatchMeshState* st = d_->st.get();
    const int32_t* cS = d_->counts.get();
    FGB_LAUNCH(kb_spmv_pq<<<FGB_RG(kb_spmv_pq, grid_), kB, 0, stream_>>>(L.S.get(), cS, L.block_mesh.get(), st, L.s_begin.get(), L.s_len.get(),
                                                     L.a_col.get(), L.v64.get(), L.x.get(), L.p.get(), L.q.get(),
                                                     L.partial.get()));
    FGB_LAUNCH(kb_update<<<FGB_RG(kb_update, grid_), kB, 0, stream_>>>(L.S.get(), cS, L.block_mesh.get(), st, L.x.get(), L.bb.get(), L.r.get(),
                                                    L.p.get(), L.q.get(), L.b.get(), L.partial.get()));
    vcycle(0);
    FGB_LAUNCH(kb_rz<<<FGB_RG(kb_rz, grid_), kB, 0, stream_>>>(L.S.get(), cS, L.block_mesh.get(), st, L.r.get(), level_result(L),
                                                L.partial.get()));
    FGB_LAUNCH(kb_direction<<<FGB_RG(kb_direction, grid_), kB, 0, stream_>>>(L.S.get(), cS, L.block_mesh.get(), st, level_result(L), L.p.get()));
}

void BatchSolver::launch_persistent() {
    FGB_REQUIRE(max_levels_ >= 2 && max_levels_ <= kMaxBatchLevels, "batch hierarchy depth out of range");
    KbParams prm{};
    prm.n_levels = max_levels_;
    auto tp = [](const std::vector<int>& v, int l) { return l < (int)v.size() ? v[l] : 1; };
    for (int l = 0; l < max_levels_; ++l) {
        BatchLevelDev& L = *lv_[l];
        KbLevel& k = prm.lv[l];
        k.S = L.S.get();
        k.D = L.D.get();
        k.T = L.T.get();
        k.bm = L.block_mesh.get();
        k.cnt = d_->counts.get() + 3 * l;
        k.A = l == 0 ? OpB{L.s_begin.get(), L.s_len.get(), L.a_col.get(), L.a_val.get()}
                     : OpB{L.a_begin.get(), L.a_len.get(), L.a_col.get(), L.a_val.get()};
        k.R = OpB{L.r_begin.get(), L.r_len.get(), L.r_col.get(), L.r_val.get()};
        k.P = OpB{L.p_begin.get(), L.p_len.get(), L.p_col.get(), L.p_val.get()};
        k.dinv = L.dinv.get();
        k.b = L.b.get();
        k.xa = L.xa.get();
        k.xb = L.xb.get();
        k.d = L.d.get();
        k.rl = L.rl.get();
        k.tpr = l == 0 ? 0 : tp(tpr_, l);
        k.r_tpr = tp(r_tpr_, l);
        k.p_tpr = tp(p_tpr_, l);
    }
    BatchLevelDev& L0 = *lv_[0];
    prm.sb = L0.s_begin.get();
    prm.sl = L0.s_len.get();
    prm.col = L0.a_col.get();
    prm.v64 = L0.v64.get();
    prm.x = L0.x.get();
    prm.bb = L0.bb.get();
    prm.r = L0.r.get();
    prm.p = L0.p.get();
    prm.q = L0.q.get();
    prm.partial = L0.partial.get();
    prm.st = d_->st.get();
    prm.dense = d_->dense.get();
    prm.run = d_->run.get();
    prm.loop = d_->loop.get();
    prm.c = cheb_coefficients();
    if (persistent_grid_ == 0) {
        int dev = 0, sms = 0, per_sm = 0, coop = 0;
        FGB_CUDA(cudaGetDevice(&dev));
        FGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        FGB_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        FGB_REQUIRE(coop, "device does not support cooperative launches");
        FGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kb_persistent, kB, 0));
        FGB_REQUIRE(per_sm > 0, "the persistent batch kernel does not fit on an SM");
        persistent_grid_ = std::min(per_sm, 8) * sms;
    }
    void* args[] = {&prm};
    FGB_CUDA(cudaLaunchCooperativeKernel((void*)kb_persistent, dim3(persistent_grid_), dim3(kB), args, 0, stream_));
    g_kernel_launches.fetch_add(1);
}

void BatchSolver::capture() {
    if (exec_) { cudaGraphExecDestroy(exec_); exec_ = nullptr; }
    if (graph_) { cudaGraphDestroy(graph_); graph_ = nullptr; }
    FGB_CUDA(cudaGraphCreate(&graph_, 0));
    cudaGraphConditionalHandle handle;
    FGB_CUDA(cudaGraphConditionalHandleCreate(&handle, graph_, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    FGB_CUDA(cudaGraphAddNode(&node, graph_, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    const long long k0 = g_kernel_launches.load();
    FGB_CUDA(cudaStreamBeginCaptureToGraph(stream_, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    launch_iteration();
    FGB_LAUNCH(kb_continue<<<1, 256, 0, stream_>>>(d_->run.get(), d_->loop.get() + 3, d_->st.get(), d_->loop.get(),
                                                   handle, 1));
    cudaGraph_t captured = nullptr;
    FGB_CUDA(cudaStreamEndCapture(stream_, &captured));
    body_kernels_ = (int)(g_kernel_launches.load() - k0);
    g_kernel_launches.fetch_sub(body_kernels_);  // counted when the graph runs
    FGB_CUDA(cudaGraphInstantiate(&exec_, graph_, 0));
}

void BatchSolver::tune() {
    // For each coarse level and transfer operator, time every threads-per-row variant over
    // the current work lists and keep the fastest; results are cached per size bucket
    // (level, log2 rows, average row length) so equal buckets are measured once.
    cudaEvent_t e0, e1;
    FGB_CUDA(cudaEventCreate(&e0));
    FGB_CUDA(cudaEventCreate(&e1));
    // the timed kernels skip finished meshes: time them against a copy of the states with
    // every mesh marked unfinished (the kernels timed here read the states only)
    std::vector<BatchMeshState> hs(h_state_);
    for (auto& x : hs) x.done = 0;
    DBuf<BatchMeshState> tst;
    tst.upload(hs, stream_);
    BatchMeshState* st = tst.get();
    const int cands[] = {1, 4, 8, 16, 32};
    auto bucket_key = [](int kind, int l, long long rows, long long nnz) {
        const int lr = rows > 0 ? (int)std::log2((double)rows) : 0;
        const int la = rows > 0 ? (int)std::lround(2.0 * std::log2(1.0 + (double)nnz / rows)) : 0;
        return ((long long)kind << 48) | ((long long)l << 40) | ((long long)lr << 8) | la;
    };
    auto time_variant = [&](auto&& launch) {
        launch();
        FGB_CUDA(cudaEventRecord(e0, stream_));
        for (int k = 0; k < 5; ++k) launch();
        FGB_CUDA(cudaEventRecord(e1, stream_));
        FGB_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        FGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        return ms;
    };
    for (int l = 0; l < (int)lv_.size(); ++l) {
        BatchLevelDev& L = *lv_[l];
        const int32_t* cl = d_->counts.get() + 3 * l;
        long long rows = 0, a_nnz = 0, p_nnz = 0, r_nnz = 0;
        for (int slot : running_) {
            const Mesh& m = *meshes_[slot];
            if (l > m.depth) continue;
            rows += m.nrows[l];
            a_nnz += (long long)m.a_len[l];
            p_nnz += (long long)m.p_len[l];
            r_nnz += (long long)m.r_len[l];
        }
        if (rows == 0) continue;
        if (l >= 1 && L.nS > 0) {
            const long long key = bucket_key(0, l, rows, a_nnz);
            auto it = tune_cache_.find(key);
            if (it != tune_cache_.end()) tpr_[l] = it->second;
            else {
                const OpB A{L.a_begin.get(), L.a_len.get(), L.a_col.get(), L.a_val.get()};
                float best = 1e30f;
                for (int t : cands) {
                    const float ms = time_variant([&] {
                        FGB_BATCH_TPR(kb_residual, t, grid_, stream_, L.S.get(), cl, L.block_mesh.get(), st, A, L.b.get(),
                                      L.xb.get(), L.rl.get());
                    });
                    if (ms < best) { best = ms; tpr_[l] = t; }
                }
                tune_cache_[key] = tpr_[l];
            }
        }
        if (l + 1 < (int)lv_.size() && L.nS > 0) {
            BatchLevelDev& C = *lv_[l + 1];
            const int32_t* cc = d_->counts.get() + 3 * (l + 1);
            const long long kp = bucket_key(1, l, rows, p_nnz);
            auto ip = tune_cache_.find(kp);
            if (ip != tune_cache_.end()) p_tpr_[l] = ip->second;
            else {
                const OpB P{L.p_begin.get(), L.p_len.get(), L.p_col.get(), L.p_val.get()};
                float best = 1e30f;
                for (int t : cands) {
                    // prolongation accumulates into xb; the V-cycle rewrites xb before its next use
                    const float ms = time_variant([&] {
                        FGB_BATCH_TPR(kb_csr_apply, t, grid_, stream_, L.S.get(), cl, L.block_mesh.get(), st, P,
                                      C.xb.get(), L.xb.get(), 1);
                    });
                    if (ms < best) { best = ms; p_tpr_[l] = t; }
                }
                tune_cache_[kp] = p_tpr_[l];
            }
            long long crow = 0;
            for (int slot : running_) {
                const Mesh& m = *meshes_[slot];
                if (l + 1 <= m.depth) crow += m.nrows[l + 1];
            }
            const long long kr = bucket_key(2, l + 1, crow, r_nnz);
            auto ir = tune_cache_.find(kr);
            if (ir != tune_cache_.end()) r_tpr_[l + 1] = ir->second;
            else {
                const OpB R{C.r_begin.get(), C.r_len.get(), C.r_col.get(), C.r_val.get()};
                float best = 1e30f;
                for (int t : cands) {
                    const float ms = time_variant([&] {
                        FGB_BATCH_TPR(kb_csr_apply, t, grid_, stream_, C.T.get(), cc + 2, C.block_mesh.get(), st, R,
                                      L.rl.get(), C.b.get(), 0);
                    });
                    if (ms < best) { best = ms; r_tpr_[l + 1] = t; }
                }
                tune_cache_[kr] = r_tpr_[l + 1];
            }
        }
    }
    FGB_CUDA(cudaStreamSynchronize(stream_));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
}

int BatchSolver::step(int max_iters, bool stop_at_first) {
    std::lock_guard<std::mutex> lk(mu_);
    if (running_.empty()) return 0;
    ensure_capacity();
    if (opt_.autotune && dirty_) {
        // the layout changed (meshes placed or levels added): tune the threads-per-row over
        // every resident mesh, so that later admissions reuse the choice and the graph
        const std::vector<int> t0 = tpr_, p0 = p_tpr_, r0 = r_tpr_;
        std::vector<int> active;
        active.swap(running_);
        for (size_t i = 0; i < meshes_.size(); ++i)
            if (meshes_[i]) running_.push_back((int)i);
        rebuild_lists();
        tune();
        running_.swap(active);
        lists_dirty_ = true;
        (void)t0; (void)p0; (void)r0;
    }
    if (lists_dirty_) rebuild_lists();
    int iters = 0;
    if (opt_.persistent) {
        dirty_ = false;
        int loop[3] = {0, std::max(1, max_iters) * (stop_at_first ? -1 : 1), 1};
        FGB_CUDA(cudaMemcpyAsync(d_->loop.get(), loop, 3 * sizeof(int), cudaMemcpyHostToDevice, stream_));
        launch_persistent();
        FGB_CUDA(cudaMemcpyAsync(d_->h_loop, d_->loop.get(), 4 * sizeof(int), cudaMemcpyDeviceToHost, stream_));
        FGB_CUDA(cudaStreamSynchronize(stream_));
        iters = d_->h_loop[0];
    } else if (opt_.use_graph) {
        if (dirty_ || !exec_) {
            capture();
            dirty_ = false;
        }
        int loop[3] = {0, std::max(1, max_iters) * (stop_at_first ? -1 : 1), 1};
        FGB_CUDA(cudaMemcpyAsync(d_->loop.get(), loop, 3 * sizeof(int), cudaMemcpyHostToDevice, stream_));
        FGB_CUDA(cudaGraphLaunch(exec_, stream_));
        FGB_CUDA(cudaMemcpyAsync(d_->h_loop, d_->loop.get(), 4 * sizeof(int), cudaMemcpyDeviceToHost, stream_));
        FGB_CUDA(cudaStreamSynchronize(stream_));
        iters = d_->h_loop[0];
        g_kernel_launches.fetch_add((long long)iters * body_kernels_);
    } else {
        dirty_ = false;
        int loop[3] = {0, std::max(1, max_iters) * (stop_at_first ? -1 : 1), 1};
        FGB_CUDA(cudaMemcpyAsync(d_->loop.get(), loop, 3 * sizeof(int), cudaMemcpyHostToDevice, stream_));
        cudaGraphConditionalHandle none{};
        while (true) {
            const long long k0 = g_kernel_launches.load();
            launch_iteration();
            FGB_LAUNCH(kb_continue<<<1, 256, 0, stream_>>>(d_->run.get(), d_->loop.get() + 3, d_->st.get(),
                                                           d_->loop.get(), none, 0));
            body_kernels_ = (int)(g_kernel_launches.load() - k0);
            FGB_CUDA(cudaMemcpyAsync(d_->h_loop, d_->loop.get(), 4 * sizeof(int), cudaMemcpyDeviceToHost, stream_));
            FGB_CUDA(cudaStreamSynchronize(stream_));
            if (!d_->h_loop[2]) break;
        }
        iters = d_->h_loop[0];
    }
    FGB_CUDA(cudaGetLastError());
    launches_ += 1;
    // refresh the host copy of the per-mesh states
    FGB_CUDA(cudaMemcpyAsync(h_state_.data(), d_->st.get(), h_state_.size() * sizeof(BatchMeshState),
                             cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    int still = 0;
    for (int slot : running_)
        if (!h_state_[slot].done) ++still;
    last_iters_ = iters;
    return still;
}

std::vector<std::pair<int, BatchSolveResult>> BatchSolver::collect_finished() {
    std::lock_guard<std::mutex> lk(mu_);
    std::vector<std::pair<int, BatchSolveResult>> out;
    std::vector<int> keep;
    for (int slot : running_) {
        const BatchMeshState& s = h_state_[slot];
        if (s.done) {
            BatchSolveResult r;
            r.iterations = s.iter;
            r.status = s.status;
            r.bnorm = s.bnorm;
            r.rel_residual = s.bnorm > 0 ? std::sqrt(std::max(0.0, s.rr)) / s.bnorm : 0.0;
            meshes_[slot]->last = r;
            meshes_[slot]->admitted = false;
            out.push_back({slot, r});
            lists_dirty_ = true;
        } else {
            keep.push_back(slot);
        }
    }
    running_.swap(keep);
    return out;
}

void BatchSolver::extract(int slot, bool smoothen) {
    Mesh& m = *meshes_.at(slot);
    m.dm->extract_solution(lv_[0]->x.get() + m.row0[0], m.dof2node.get(), m.n_dofs, smoothen);
}

void BatchSolver::export_phi_nodes(int slot, double* phi) {
    Mesh& m = *meshes_.at(slot);
    std::vector<double> x(m.n_dofs);
    FGB_CUDA(cudaMemcpyAsync(x.data(), lv_[0]->x.get() + m.row0[0], sizeof(double) * m.n_dofs, cudaMemcpyDeviceToHost,
                             m.stream));
    FGB_CUDA(cudaStreamSynchronize(m.stream));
    std::fill(phi, phi + m.n_nodes, 0.0);
    for (int d = 0; d < m.n_dofs; ++d)
        if (m.h_dof2node[d] >= 0) phi[m.h_dof2node[d]] = x[d];
}

void BatchSolver::reset_solution(int slot) {
    std::lock_guard<std::mutex> lk(mu_);
    Mesh& m = *meshes_.at(slot);
    FGB_REQUIRE(!m.admitted, "the mesh has a solve in flight");
    FGB_CUDA(cudaMemsetAsync(lv_[0]->x.get() + m.row0[0], 0, sizeof(double) * m.nalloc[0], stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
}

double BatchSolver::true_residual(int slot) {
    std::lock_guard<std::mutex> lk(mu_);
    Mesh& m = *meshes_.at(slot);
    BatchLevelDev& L = *lv_[0];
    const int g = grid_for(m.n_dofs, kB);
    DBuf<double> part(2 * (size_t)g);
    FGB_LAUNCH(kb_true_residual<<<g, kB, 0, stream_>>>(m.row0[0], m.n_dofs, L.s_begin.get(), L.s_len.get(), L.a_col.get(),
                                                      L.v64.get(), L.x.get(), L.bb.get(), part.get()));
    std::vector<double> h = part.to_host(stream_);
    double rr = 0, bb = 0;
    for (int b = 0; b < g; ++b) {
        rr += h[2 * b];
        bb += h[2 * b + 1];
    }
    return bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
}

}  // namespace fgb
