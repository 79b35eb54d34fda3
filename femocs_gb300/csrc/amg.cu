// FP32 multigrid V-cycle on the device (sm_103a); host hierarchy from amg_setup.cpp.
//
//   k_cheb_zero      first Chebyshev step from a zero guess: d = D^-1 b / theta, x = d
//   k_cheb_step      d = c1 d + c2 D^-1 (b - A x_in), x_out = x_in + d   (x_in gathered, so
//                    x is ping-ponged between two buffers)
//   k_residual       r = b - A x
//   k_csr_apply      b_c = R r  (restriction, R = P^T stored explicitly: gather, no atomics)
//                    and x += P x_c (prolongation)
//   k_dense_solve    x = A_c^-1 b on the coarsest level (one warp per row)
// Chebyshev smoothing of D^-1 A on [0.1, 1.1] x lambda_max, degree 2 before and after the
// coarse correction (the same polynomial, so the cycle is a symmetric preconditioner).
// Level 0 runs on the solver's SELL-32 matrix, one thread per row, or for Q2 element by
// element over cell blocks (k_cb_apply, k_cb_finish: one CTA per block of hexes, products
// summed on chip, cell_blocks.h); coarser levels are CSR with 1..32 threads per row, chosen
// from the average row length (the aggregated levels get denser, up to hundreds of entries
// per row), the transfer operators one thread per row up to 8 entries.
#include <cmath>
#include <sstream>

#include <cuda_fp16.h>

#include "amg.h"

namespace fgb {

struct AmgDevLevel {
    int n = 0, n_coarse = 0;
    double lambda = 1.0, cheb_lo = 0.1, built_lo = 0.1;
    int cheb_degree = 2, built_degree = 2;  // built_*: the hierarchy's own choice
    const int64_t* sptr = nullptr;
    const int32_t* slen = nullptr;
    const int32_t* scol = nullptr;
    const float* val = nullptr;
    const float* dinv = nullptr;
    // levels >= 1: CSR with `tpr` threads per row (level 0 uses the solver's SELL arrays)
    DBuf<int64_t> a_ptr;
    DBuf<int32_t> a_col, own_slen;
    DBuf<float> a_val, own_dinv;
    int tpr = 1, p_tpr = 1, r_tpr = 1;
    DBuf<int64_t> p_ptr, r_ptr;
    DBuf<int32_t> p_col, r_col;
    DBuf<float> p_val, r_val;
    DBuf<float> b, xa, xb, d, r;
    DBuf<float> xacc, rtmp;      // repeated coarse cycles: the summed result, the residual
    const float* bin = nullptr;  // right-hand side of this level (level 0: the caller's vector)
    float* x = nullptr;          // result of the last cycle on this level
};

namespace {

constexpr int kB = 256;

__device__ __forceinline__ float sell4_row(int r, const int64_t* __restrict__ sptr, const int32_t* __restrict__ slen,
                                           const int32_t* __restrict__ scol, const float* __restrict__ val,
                                           const float* __restrict__ x) {
    const int s = r >> 5;
    const int64_t base = sptr[s] + (int64_t)(r & 31) * 4;
    const int nch = slen[s] >> 2;
    float a0 = 0.f, a1 = 0.f;
    int c = 0;
    for (; c + 1 < nch; c += 2) {
        const int64_t o0 = base + (int64_t)c * 128, o1 = o0 + 128;
        const int4 i0 = __ldg(reinterpret_cast<const int4*>(scol + o0));
        const int4 i1 = __ldg(reinterpret_cast<const int4*>(scol + o1));
        const float4 v0 = __ldg(reinterpret_cast<const float4*>(val + o0));
        const float4 v1 = __ldg(reinterpret_cast<const float4*>(val + o1));
        a0 += v0.x * __ldg(x + i0.x) + v0.y * __ldg(x + i0.y) + v0.z * __ldg(x + i0.z) + v0.w * __ldg(x + i0.w);
        a1 += v1.x * __ldg(x + i1.x) + v1.y * __ldg(x + i1.y) + v1.z * __ldg(x + i1.z) + v1.w * __ldg(x + i1.w);
    }
    if (c < nch) {
        const int64_t o0 = base + (int64_t)c * 128;
        const int4 i0 = __ldg(reinterpret_cast<const int4*>(scol + o0));
        const float4 v0 = __ldg(reinterpret_cast<const float4*>(val + o0));
        a0 += v0.x * __ldg(x + i0.x) + v0.y * __ldg(x + i0.y) + v0.z * __ldg(x + i0.z) + v0.w * __ldg(x + i0.w);
    }
    return a0 + a1;
}

// Level operator: SELL (level 0, one thread per row) or CSR with TPR threads per row.
struct Op {
    int n;
    const int64_t* sptr;  // SELL slice offsets, or CSR row pointers
    const int32_t* slen;  // SELL slice lengths (unused for CSR)
    const int32_t* scol;
    const float* val;
    const float* dinv;
};

// Row `row` of A x, summed over the TPR lanes of the row's group (valid in every lane of the
// group). All 32 lanes of the warp must call it: rows beyond n contribute nothing.
template <int TPR>
__device__ __forceinline__ float op_row(const Op& A, int row, const float* __restrict__ x) {
    if constexpr (TPR == 0) {
        return sell4_row(row, A.sptr, A.slen, A.scol, A.val, x);
    } else {
        const int sub = threadIdx.x & (TPR - 1);
        float acc = 0.f;
        if (row < A.n) {
            const int64_t end = A.sptr[row + 1];
            int64_t k = A.sptr[row] + sub;
            // four independent chains keep more gathers in flight on the long coarse rows
            float a1 = 0.f, a2 = 0.f, a3 = 0.f;
            for (; k + 3 * TPR < end; k += 4 * TPR) {
                acc += __ldg(A.val + k) * __ldg(x + A.scol[k]);
                a1 += __ldg(A.val + k + TPR) * __ldg(x + A.scol[k + TPR]);
                a2 += __ldg(A.val + k + 2 * TPR) * __ldg(x + A.scol[k + 2 * TPR]);
                a3 += __ldg(A.val + k + 3 * TPR) * __ldg(x + A.scol[k + 3 * TPR]);
            }
            for (; k < end; k += TPR) acc += __ldg(A.val + k) * __ldg(x + A.scol[k]);
            acc += (a1 + a2) + a3;
        }
#pragma unroll
        for (int o = TPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        return acc;
    }
}

// TPR = 0: SELL, one thread per row; TPR = 1..32: CSR, TPR threads per row
template <int TPR>
__device__ __forceinline__ int row_of() {
    constexpr int t = TPR == 0 ? 1 : TPR;
    return (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) / t);
}
template <int TPR>
__device__ __forceinline__ bool row_leader() {
    return TPR <= 1 || (threadIdx.x & (TPR - 1)) == 0;
}

__global__ void __launch_bounds__(kB) k_cheb_zero(int n, const float* __restrict__ dinv, const float* __restrict__ b,
                                                  float* __restrict__ x, float* __restrict__ d, float inv_theta) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float di = dinv[i] * b[i] * inv_theta;
    d[i] = di;
    x[i] = di;
}

// c1 < 0 marks the first step from a nonzero guess: d = D^-1 r / theta (c2 = 1/theta)
// the row kernels below are built for 8 CTAs of 256 threads per SM (32 registers; the SELL
// variants spill 16 bytes): the 2.8e5-DoF Q1 nanotip's level-0 smoothing ran at 0.43 of the copy bandwidth
// with 6 CTAs per SM (40 registers), 0.50 with 8
template <int TPR>
__global__ void __launch_bounds__(kB, 8) k_cheb_step(Op A, const float* __restrict__ b, const float* __restrict__ xin,
                                                  float* __restrict__ xout, float* __restrict__ d, float c1, float c2) {
    const int i = row_of<TPR>();
    if (TPR <= 1 && i >= A.n) return;
    const float ax = op_row<TPR>(A, i, xin);
    if (i >= A.n || !row_leader<TPR>()) return;
    const float ri = b[i] - ax;
    const float di = (c1 < 0.f ? 0.f : c1 * d[i]) + c2 * A.dinv[i] * ri;
    d[i] = di;
    xout[i] = xin[i] + di;
}

__global__ void k_add_f(int n, const float* __restrict__ y, float* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += y[i];
}

template <int TPR>
__global__ void __launch_bounds__(kB, 8) k_residual(Op A, const float* __restrict__ b, const float* __restrict__ x,
                                                 float* __restrict__ r) {
    const int i = row_of<TPR>();
    if (TPR <= 1 && i >= A.n) return;
    const float ax = op_row<TPR>(A, i, x);
    if (i >= A.n || !row_leader<TPR>()) return;
    r[i] = b[i] - ax;
}

// y = M x (accumulate: y += M x) for a CSR transfer operator
template <int TPR>
__global__ void __launch_bounds__(kB, 8) k_csr_apply(int n, const int64_t* __restrict__ ptr, const int32_t* __restrict__ col,
                                                  const float* __restrict__ val, const float* __restrict__ x,
                                                  float* __restrict__ y, int accumulate) {
    const int i = row_of<TPR>();
    if (TPR <= 1 && i >= n) return;
    const Op M{n, ptr, nullptr, col, val, nullptr};
    const float acc = op_row<TPR>(M, i, x);
    if (i >= n || !row_leader<TPR>()) return;
    y[i] = accumulate ? y[i] + acc : acc;
}

// ---- element-by-element level-0 operator (Q2) by cell blocks: one CTA per block
constexpr int kCb = 256;

// final row update of a level-0 application: Chebyshev step (KIND 0) or residual (KIND 1)
template <int KIND>
__device__ __forceinline__ void l0_finish(int g, float ax, float xg, const float* __restrict__ b,
                                          const float* __restrict__ dinv, float* __restrict__ xout,
                                          float* __restrict__ d, float c1, float c2) {
    const float ri = b[g] - ax;
    if constexpr (KIND == 1) {
        xout[g] = ri;
    } else {
        const float di = (c1 < 0.f ? 0.f : c1 * d[g]) + c2 * dinv[g] * ri;
        d[g] = di;
        xout[g] = xg + di;
    }
}

constexpr int kCbPer = 16;     // block-local DoFs per thread at most (max_dofs <= 4096)
constexpr int kCbMaxCells = 256;

// Streamed variant: a producer warp copies each block's element matrices (contiguous in block
// order, 1512 B per cell) with cp.async.bulk into a ring of kCbRing slots of kCbChunk cells,
// one cell per consumer warp per slot; full/empty mbarriers pace it. A copy starts on the
// 16-byte boundary at or below its first cell (cells alternate between 0 and 8 bytes past
// one) and never reads past the array: the last <= 8 bytes of the array are loaded plainly.
constexpr int kCbRing = 4;
constexpr int kCbChunk = kCb / 32;                  // cells per slot = consumer warps
constexpr int kCbSlot = kCbChunk * 1512 + 16;       // bytes per slot (alignment slack)
constexpr unsigned kCbSpin = 1u << 22;              // try_wait rounds before a wait gives up

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// wait for the phase of the given parity to complete, at most kCbSpin rounds
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    for (unsigned i = 0; i < kCbSpin; ++i) {
        unsigned ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// L2 prefetch of bytes [off, off + len) of an array of `total` bytes: the 16-byte-aligned
// span around them (a cell's element matrix starts 0 or 8 bytes past a boundary), clipped to
// the array's last full 16 bytes
__device__ __forceinline__ void prefetch_l2(const void* base, int64_t total, int64_t off, int64_t len) {
    const int64_t a = off & ~(int64_t)15;
    int64_t e = (off + len + 15) & ~(int64_t)15;
    const int64_t end = total & ~(int64_t)15;
    if (e > end) e = end;
    if (e > a)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(reinterpret_cast<const char*>(base) + a),
                     "r"((unsigned)(e - a))
                     : "memory");
}

// Level-0 operator of three cells at once from their geometric factors, by sum
// factorisation: lane l < 27 of a warp works on cell g = l / 9 of the group and owns the
// 1-D pencil p = l % 9 of its 3 x 3 x 3 lattice, so every contraction is three
// independent 3-term sums in registers with constant coefficients; the pencils are
// transposed between the stages through a per-warp shared-memory scratch (3 x 170 floats;
// every store writes 9 consecutive words per cell, every lane reads 3 consecutive words).
// Stages (lattice node (a, b, c) = a + 3b + 9c, Gauss point (qx, qy, qz)):
//   1  lane (a, b):   T1 = S_z u, T2 = D_z u over c            -> W[qz][a][b]
//   2  lane (a, qz):  A1 = S_y T1, A2 = D_y T1, A3 = S_y T2     -> X[qy][qz][a]
//   3  lane (qy, qz): reference gradient (D_x A1, S_x A2, S_x A3) at qx = 0..2, flux
//                     C_q g, then the transposed x contraction  -> Y[a][qz][qy]
//   4  lane (a, qz):  E1 = S_y^T B1 + D_y^T B2, E2 = S_y^T B3    -> Z[b][a][qz]
//   5  lane (a, b):   v = S_z^T E1 + D_z^T E2 at c = 0..2
// with S[q][a] = l_a(t_q), D[q][a] = l_a'(t_q). K_e = sum_q B_q^T C_q B_q is the Q2
// element matrix, so v equals K_e u up to FP32 rounding.
__device__ __forceinline__ constexpr float sfS(int q, int a) {
    return a == 0 ? 0.5f * ((q - 1) * 0.7745966692414834f) * ((q - 1) * 0.7745966692414834f - 1.f)
                  : (a == 1 ? 1.f - ((q - 1) * 0.7745966692414834f) * ((q - 1) * 0.7745966692414834f)
                            : 0.5f * ((q - 1) * 0.7745966692414834f) * ((q - 1) * 0.7745966692414834f + 1.f));
}
__device__ __forceinline__ constexpr float sfD(int q, int a) {
    return a == 0 ? (q - 1) * 0.7745966692414834f - 0.5f
                  : (a == 1 ? -2.f * ((q - 1) * 0.7745966692414834f) : (q - 1) * 0.7745966692414834f + 0.5f);
}
// floats per cell: two regions of 81 (W then Y, X then Z); 170 = 10 mod 32 banks, so the
// three cells' 9-word rows written by one store fall into disjoint banks
constexpr int kSfScratch = 170;
constexpr int kSfWarpBytes = 3 * kSfScratch * 4;
// barrier over the consumer warps of the streamed kernel (the producer does not take part)
__device__ __forceinline__ void consumers_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kCb) : "memory"); }

// shared memory of one block: its item lists (28 u16 per cell), x of its DoFs, the products
__host__ __device__ inline size_t cb_smem_bytes(int max_cells, int max_dofs) {
    return 56 * (size_t)max_cells + 4 * (size_t)max_dofs + 108 * (size_t)max_cells;
}
// the geometric-factor variants: the same, then (16-byte aligned) the warps' scratch
__host__ __device__ inline size_t cb_geo_smem_bytes(int max_cells, int max_dofs) {
    return ((cb_smem_bytes(max_cells, max_dofs) + 15) & ~(size_t)15) + (kCb / 32) * (size_t)kSfWarpBytes;
}
// the streamed variant: the same, then (128-byte aligned) the ring and its full/empty barriers
__host__ __device__ inline size_t cb_stream_smem_bytes(int max_cells, int max_dofs) {
    return ((cb_smem_bytes(max_cells, max_dofs) + 127) & ~(size_t)127) + kCbRing * (size_t)kCbSlot + 2 * kCbRing * 8;
}

// One block per CTA, three phases separated by barriers:
//  A  the block's item lists and x of its DoFs into shared memory (each thread's loads issued
//     together, so the gathers overlap instead of queueing behind one another);
//  B  K_e x_e of each cell: one warp per cell, lane i < 27 owns row i. It holds K(i, i+t) for
//     t = 0..13 (seven float2 loads), takes x_{i+t} from lane i+t and hands K(i, i+t) x_i to
//     lane i+t (indices mod 27), so every entry of the symmetric K_e is loaded once; the next
//     cell's matrix is loaded while the current one is applied;
//  C  the products of each DoF summed in item order; complete DoFs finished (Chebyshev update
//     or residual), the others leave their partial sum in their slot.
//
// SRC selects where phase B takes each cell's operator from:
//  kSrcKe    the element matrices, loaded by the applying warps (above);
//  kSrcRing  the element matrices through the bulk-copy ring (one more warp, the producer;
//            phases separated by a barrier over the consumer warps only);
//  kSrcGeo / kSrcGeo16  the geometric factors C_q of the 27 Gauss points (FP32 / FP16, 648 /
//            324 bytes per cell instead of 1512), applied by sum factorisation over the
//            cells' 1-D pencils (three cells per warp, see sfS / sfD).
constexpr int kSrcKe = 0, kSrcRing = 1, kSrcGeo = 2, kSrcGeo16 = 3;
template <int KIND, int SRC>
__global__ void __launch_bounds__(SRC == kSrcRing ? kCb + 32 : kCb, SRC == kSrcRing ? 2 : (SRC >= kSrcGeo ? 4 : 3))
    k_cb_apply(EbeOperator op, const float* __restrict__ dinv, const float* __restrict__ b,
               const float* __restrict__ xin, float* __restrict__ xout, float* __restrict__ d, float c1, float c2) {
    constexpr bool STREAM = SRC == kSrcRing;
    constexpr bool GEO = SRC == kSrcGeo || SRC == kSrcGeo16;
    constexpr int kGeoBytes = SRC == kSrcGeo16 ? 324 : 648;  // geometric factors per cell
    extern __shared__ __align__(128) unsigned char cb_raw[];
    const int blk = blockIdx.x;
    const int p0 = op.cell_start[blk], nb = op.cell_start[blk + 1] - p0;
    const int q0 = op.dof_start[blk], nq = op.dof_start[blk + 1] - q0;
    uint16_t* sit = reinterpret_cast<uint16_t*>(cb_raw);
    float* sx = reinterpret_cast<float*>(cb_raw + 56 * (size_t)op.max_cells);
    float* sy = sx + op.max_dofs;
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int il = lane < 27 ? lane : 26;  // lanes 27..31 shadow lane 26 and store nothing
    const uint16_t* loc = op.loc + 27 * (size_t)p0;
    // ring and barriers after the phase buffers (128-byte aligned)
    unsigned char* ring = cb_raw + ((cb_smem_bytes(op.max_cells, op.max_dofs) + 127) & ~(size_t)127);
    uint64_t* full = reinterpret_cast<uint64_t*>(ring + kCbRing * (size_t)kCbSlot);
    uint64_t* empty = full + kCbRing;
    const int n_chunks = (nb + kCbChunk - 1) / kCbChunk;
    if constexpr (STREAM) {
        if (tid == 0) {
            for (int s = 0; s < kCbRing; ++s) {
                mbar_init(&full[s], 1);
                mbar_init(&empty[s], kCbChunk);
            }
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
        if (warp == kCb / 32) {
            // producer: chunk j (cells 8j .. 8j+7 of the block) into slot j % kCbRing
            if (lane == 0) {
                const unsigned char* base = reinterpret_cast<const unsigned char*>(op.ke);
                const int64_t end = 4 * op.n_ke;  // bytes in the array
                for (int j = 0; j < n_chunks; ++j) {
                    const int sl = j % kCbRing;
                    if (j >= kCbRing && !mbar_wait(&empty[sl], ((j / kCbRing) - 1) & 1)) {
                        atomicOr(op.err, 1u);
                        break;
                    }
                    const int cells = min(kCbChunk, nb - j * kCbChunk);
                    const int64_t src = 1512 * (int64_t)(p0 + j * kCbChunk);
                    const int64_t a = src & 15;
                    int64_t n = (1512 * (int64_t)cells + a + 15) & ~(int64_t)15;
                    unsigned char* dst = ring + sl * (size_t)kCbSlot;
                    int64_t tail = 0;  // bytes past the last 16-byte boundary of the array
                    if (src - a + n > end) {
                        tail = end - (src - a + n - 16);
                        n -= 16;
                    }
                    if (tail > 0) {
                        // the array's last bytes (a multiple of 4, at most 8): plain loads and
                        // stores before the arrive, whose release makes them visible to the
                        // consumers that acquire the completed phase
                        for (int64_t k = 0; k < tail; k += 4)
                            *reinterpret_cast<unsigned*>(dst + n + k) =
                                __ldg(reinterpret_cast<const unsigned*>(base + src - a + n + k));
                    }
                    mbar_expect_tx(&full[sl], (unsigned)n);
                    bulk_g2s(dst, base + src - a, (unsigned)n, &full[sl]);
                }
            }
            return;
        }
    }
    // cells of warp w: w, w + 8, w + 16, ...; two register sets (A, B) alternate so that the
    // next cell's element matrix is in flight while the current one is applied. The first
    // cell's is requested before phase A, so that it travels while the gathers run.
    float kA[14], kB[14];
    int lA = 0, lB = 0;
    constexpr int kW = kCb / 32;
    // optional L2 prefetch, op.prefetch cells ahead of each warp's loads: the warp's first
    // cells are requested here, then every load requests the cell op.prefetch steps later,
    // so the DRAM stream runs ahead of the register double buffer (and through phase A)
    const int pf = STREAM ? 0 : op.prefetch;
    auto prefetch_cell = [&](int c) {
        if constexpr (GEO)
            prefetch_l2(op.geo, kGeoBytes * (int64_t)op.n_cells, kGeoBytes * (int64_t)(p0 + c), kGeoBytes);
        else
            prefetch_l2(op.ke, 4 * op.n_ke, 1512 * (int64_t)(p0 + c), 1512);
    };
    if (pf > 0 && lane == 0)
        for (int k = 1; k < pf; ++k)
            if (warp + k * kW < nb) prefetch_cell(warp + k * kW);
    auto load_cell = [&](int c, float (&k)[14], int& l) {
        if (pf > 0 && lane == 0 && c + pf * kW < nb) prefetch_cell(c + pf * kW);
        const float2* K = reinterpret_cast<const float2*>(op.ke + 378 * (size_t)(p0 + c));
#pragma unroll
        for (int u = 0; u < 7; ++u) {
            const float2 v = __ldg(K + 27 * u + il);
            k[2 * u] = v.x;
            k[2 * u + 1] = v.y;
        }
        l = __ldg(loc + 27 * c + il);
    };
    // geometric factors: groups of three consecutive cells per warp (group t of the block =
    // cells 3t .. 3t + 2; warp w takes t = w, w + 8, ...), lane l < 27 on cell 3t + l / 9 and
    // pencil l % 9; cg = (C00, C11, C22, C01, C02, C12) at the lane's three Gauss points
    // qx = 0..2 (pairs stored at [(qx, pair m), pencil] per cell), lc = the block-local entries
    // of the pencil's three lattice nodes
    const bool act = lane < 27;
    const int sg = act ? lane / 9 : 2, pp = act ? lane % 9 : 8;
    const int pa = pp % 3, pb = pp / 3;
    const int n_groups = (nb + 2) / 3;
    float cg[18];
    int lc[3];
    auto load_group = [&](int t) {
        if (pf > 0 && lane == 0 && 3 * (t + pf * kW) < nb)
            prefetch_l2(op.geo, kGeoBytes * (int64_t)op.n_cells, kGeoBytes * (int64_t)(p0 + 3 * (t + pf * kW)),
                        3 * kGeoBytes);
        const int cell = min(3 * t + sg, nb - 1);
        if constexpr (SRC == kSrcGeo16) {
            const __half2* G = reinterpret_cast<const __half2*>(op.geo) + 81 * (size_t)(p0 + cell) + pp;
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const float2 v = __half22float2(__ldg(G + 9 * k));
                cg[2 * k] = v.x;
                cg[2 * k + 1] = v.y;
            }
        } else {
            const float2* G = reinterpret_cast<const float2*>(op.geo) + 81 * (size_t)(p0 + cell) + pp;
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const float2 v = __ldg(G + 9 * k);
                cg[2 * k] = v.x;
                cg[2 * k + 1] = v.y;
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) lc[c] = __ldg(loc + 27 * cell + pp + 9 * c);
    };
    if constexpr (GEO) {
        if (warp < n_groups) load_group(warp);
    } else if (!STREAM && warp < nb) {
        load_cell(warp, kA, lA);
    }
    {
        const uint2* gi = reinterpret_cast<const uint2*>(op.items + 28 * (size_t)p0);
        uint2* si = reinterpret_cast<uint2*>(sit);
        const int nw = 7 * nb;
        uint2 w8[7];
#pragma unroll
        for (int r = 0; r < 7; ++r) {
            const int w = tid + r * kCb;
            if (w < nw) w8[r] = __ldg(gi + w);
        }
#pragma unroll
        for (int r0 = 0; r0 < kCbPer; r0 += 8) {
            int gd[8];
            float xv[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int k = tid + (r0 + r) * kCb;
                gd[r] = k < nq ? __ldg(op.dof_list + q0 + k) : 0;
            }
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int k = tid + (r0 + r) * kCb;
                xv[r] = k < nq ? __ldg(xin + gd[r]) : 0.f;
            }
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int k = tid + (r0 + r) * kCb;
                if (k < nq) sx[k] = xv[r];
            }
        }
#pragma unroll
        for (int r = 0; r < 7; ++r) {
            const int w = tid + r * kCb;
            if (w < nw) si[w] = w8[r];
        }
    }
    if constexpr (STREAM) consumers_sync();
    else __syncthreads();
    // source lanes of the shuffles, (lane +- t) mod 27, the same for every cell
    int up[14], dn[14];
#pragma unroll
    for (int t = 1; t < 14; ++t) {
        up[t] = lane + t >= 27 ? lane + t - 27 : lane + t;
        dn[t] = lane - t < 0 ? lane - t + 27 : lane - t;
    }
    auto apply_cell = [&](int c, const float (&k)[14], int l) {
        const float x = sx[l];
        float y = k[0] * x;
#pragma unroll
        for (int t = 1; t < 14; ++t) {
            const float xu = __shfl_sync(0xffffffffu, x, up[t]);
            const float tr = __shfl_sync(0xffffffffu, k[t] * x, dn[t]);
            y = fmaf(k[t], xu, y) + tr;
        }
        if (lane < 27) sy[27 * c + lane] = y;
    };
    if constexpr (STREAM) {
        bool ok = true;
        for (int j = 0; j < n_chunks; ++j) {
            const int sl = j % kCbRing;
            if (ok && !mbar_wait(&full[sl], (j / kCbRing) & 1)) {
                ok = false;
                if (lane == 0) atomicOr(op.err, 2u);
            }
            const int c = j * kCbChunk + warp;
            if (ok && c < nb) {
                const int64_t src = 1512 * (int64_t)(p0 + j * kCbChunk);
                const float2* K = reinterpret_cast<const float2*>(ring + sl * (size_t)kCbSlot + (src & 15) + 1512 * warp);
#pragma unroll
                for (int u = 0; u < 7; ++u) {
                    const float2 v = K[27 * u + il];
                    kA[2 * u] = v.x;
                    kA[2 * u + 1] = v.y;
                }
                lA = __ldg(loc + 27 * c + il);
                apply_cell(c, kA, lA);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[sl]);
        }
        consumers_sync();
    } else if constexpr (GEO) {
        // the warp's scratch: region 1 holds W then Y, region 2 holds X then Z (each 81 floats)
        float* R1 = reinterpret_cast<float*>(cb_raw + ((cb_smem_bytes(op.max_cells, op.max_dofs) + 15) & ~(size_t)15) +
                                             warp * (size_t)kSfWarpBytes) +
                    sg * kSfScratch;
        float* R2 = R1 + 81;
        for (int t = warp; t < n_groups; t += kW) {
            const int cell = 3 * t + sg;
            // 1  lane (a, b) = (pa, pb): contraction over c
            float u[3], T1[3], T2[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) u[c] = sx[lc[c]];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                T1[q] = fmaf(sfS(q, 0), u[0], fmaf(sfS(q, 1), u[1], sfS(q, 2) * u[2]));
                T2[q] = fmaf(sfD(q, 0), u[0], fmaf(sfD(q, 1), u[1], sfD(q, 2) * u[2]));
            }
            if (act) {
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    R1[9 * q + 3 * pa + pb] = T1[q];
                    R1[27 + 9 * q + 3 * pa + pb] = T2[q];
                }
            }
            __syncwarp();
            // 2  lane (a, qz) = (pa, pb): contraction over b
            float t1[3], t2[3], A1[3], A2[3], A3[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                t1[j] = R1[9 * pb + 3 * pa + j];
                t2[j] = R1[27 + 9 * pb + 3 * pa + j];
            }
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                A1[q] = fmaf(sfS(q, 0), t1[0], fmaf(sfS(q, 1), t1[1], sfS(q, 2) * t1[2]));
                A2[q] = fmaf(sfD(q, 0), t1[0], fmaf(sfD(q, 1), t1[1], sfD(q, 2) * t1[2]));
                A3[q] = fmaf(sfS(q, 0), t2[0], fmaf(sfS(q, 1), t2[1], sfS(q, 2) * t2[2]));
            }
            if (act) {
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    R2[9 * q + 3 * pb + pa] = A1[q];
                    R2[27 + 9 * q + 3 * pb + pa] = A2[q];
                    R2[54 + 9 * q + 3 * pb + pa] = A3[q];
                }
            }
            __syncwarp();
            // 3  lane (qy, qz) = (pa, pb): gradient at qx = 0..2, flux, transposed contraction over qx
            float a1[3], a2[3], a3[3], fx[3], fy[3], fz[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                a1[j] = R2[9 * pa + 3 * pb + j];
                a2[j] = R2[27 + 9 * pa + 3 * pb + j];
                a3[j] = R2[54 + 9 * pa + 3 * pb + j];
            }
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const float gx = fmaf(sfD(q, 0), a1[0], fmaf(sfD(q, 1), a1[1], sfD(q, 2) * a1[2]));
                const float gy = fmaf(sfS(q, 0), a2[0], fmaf(sfS(q, 1), a2[1], sfS(q, 2) * a2[2]));
                const float gz = fmaf(sfS(q, 0), a3[0], fmaf(sfS(q, 1), a3[1], sfS(q, 2) * a3[2]));
                const float* C = cg + 6 * q;
                fx[q] = fmaf(C[0], gx, fmaf(C[3], gy, C[4] * gz));
                fy[q] = fmaf(C[3], gx, fmaf(C[1], gy, C[5] * gz));
                fz[q] = fmaf(C[4], gx, fmaf(C[5], gy, C[2] * gz));
            }
            // the next group's factors and lattice entries travel while this group finishes
            if (t + kW < n_groups) load_group(t + kW);
            if (act) {
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    R1[9 * a + 3 * pb + pa] = fmaf(sfD(0, a), fx[0], fmaf(sfD(1, a), fx[1], sfD(2, a) * fx[2]));
                    R1[27 + 9 * a + 3 * pb + pa] = fmaf(sfS(0, a), fy[0], fmaf(sfS(1, a), fy[1], sfS(2, a) * fy[2]));
                    R1[54 + 9 * a + 3 * pb + pa] = fmaf(sfS(0, a), fz[0], fmaf(sfS(1, a), fz[1], sfS(2, a) * fz[2]));
                }
            }
            __syncwarp();
            // 4  lane (a, qz) = (pa, pb): transposed contraction over qy
            float b1[3], b2[3], b3[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                b1[j] = R1[9 * pa + 3 * pb + j];
                b2[j] = R1[27 + 9 * pa + 3 * pb + j];
                b3[j] = R1[54 + 9 * pa + 3 * pb + j];
            }
            if (act) {
#pragma unroll
                for (int bb = 0; bb < 3; ++bb) {
                    R2[9 * bb + 3 * pa + pb] =
                        fmaf(sfS(0, bb), b1[0], fmaf(sfS(1, bb), b1[1], fmaf(sfS(2, bb), b1[2],
                             fmaf(sfD(0, bb), b2[0], fmaf(sfD(1, bb), b2[1], sfD(2, bb) * b2[2])))));
                    R2[27 + 9 * bb + 3 * pa + pb] = fmaf(sfS(0, bb), b3[0], fmaf(sfS(1, bb), b3[1], sfS(2, bb) * b3[2]));
                }
            }
            __syncwarp();
            // 5  lane (a, b) = (pa, pb): transposed contraction over qz, the products at c = 0..2
            float e1[3], e2[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                e1[j] = R2[9 * pb + 3 * pa + j];
                e2[j] = R2[27 + 9 * pb + 3 * pa + j];
            }
            if (act && cell < nb) {
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    sy[27 * cell + pp + 9 * c] =
                        fmaf(sfS(0, c), e1[0], fmaf(sfS(1, c), e1[1], fmaf(sfS(2, c), e1[2],
                             fmaf(sfD(0, c), e2[0], fmaf(sfD(1, c), e2[1], sfD(2, c) * e2[2])))));
            }
        }
        __syncthreads();
    } else {
        for (int c = warp; c < nb; c += 2 * kW) {
            if (c + kW < nb) load_cell(c + kW, kB, lB);
            apply_cell(c, kA, lA);
            if (c + kW >= nb) break;
            if (c + 2 * kW < nb) load_cell(c + 2 * kW, kA, lA);
            apply_cell(c + kW, kB, lB);
        }
        __syncthreads();
    }
    // phase C takes kCw entries per round: 4 in the geometric-factor variants, whose 64-register
    // budget (4 CTAs per SM) the 8-entry rounds would spill
    constexpr int kCw = GEO ? 4 : 8;
#pragma unroll 1
    for (int r0 = 0; r0 < kCbPer; r0 += kCw) {
        if (tid + r0 * kCb >= nq) break;
        int e0[kCw], e1[kCw], sl[kCw], g[kCw];
#pragma unroll
        for (int r = 0; r < kCw; ++r) {
            const int k = tid + (r0 + r) * kCb;
            const bool v = k < nq;
            e1[r] = v ? __ldg(op.item_end + q0 + k) : 0;
            e0[r] = v && k ? __ldg(op.item_end + q0 + k - 1) : 0;
            sl[r] = v ? __ldg(op.slot + q0 + k) : -2;
            g[r] = v ? __ldg(op.dof_list + q0 + k) : 0;
        }
        float ax[kCw], bv[kCw], dv[kCw], dd[kCw];
        int fx[kCw];
#pragma unroll
        for (int r = 0; r < kCw; ++r) {
            const bool own = sl[r] == -1;
            bv[r] = own ? b[g[r]] : 0.f;
            dv[r] = own ? dinv[g[r]] : 1.f;
            dd[r] = own && KIND == 0 && c1 >= 0.f ? d[g[r]] : 0.f;
            fx[r] = own ? op.fixed[g[r]] : 0;
        }
#pragma unroll
        for (int r = 0; r < kCw; ++r) {
            float a = 0.f;
            for (int e = e0[r]; e < e1[r]; ++e) a += sy[sit[e]];
            ax[r] = a;
        }
#pragma unroll
        for (int r = 0; r < kCw; ++r) {
            if (sl[r] >= 0) {
                op.partial[sl[r]] = ax[r];
            } else if (sl[r] == -1) {
                const float xs = sx[tid + (r0 + r) * kCb];
                const float ri = bv[r] - (fx[r] ? xs / dv[r] : ax[r]);
                if constexpr (KIND == 1) {
                    xout[g[r]] = ri;
                } else {
                    const float di = (c1 < 0.f ? 0.f : c1 * dd[r]) + c2 * dv[r] * ri;
                    d[g[r]] = di;
                    xout[g[r]] = xs + di;
                }
            }
        }
    }
}

// DoFs split over blocks: their partial sums in ascending block order
template <int KIND>
__global__ void __launch_bounds__(kB) k_cb_finish(EbeOperator op, const float* __restrict__ dinv,
                                                  const float* __restrict__ b, const float* __restrict__ xin,
                                                  float* __restrict__ xout, float* __restrict__ d, float c1, float c2) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= op.n_bnd) return;
    const int g = op.bnd_dofs[j];
    const float xg = xin[g];
    float ax = 0.f;
    if (op.fixed[g]) {
        ax = xg / dinv[g];
    } else {
        for (int s = op.bnd_ptr[j]; s < op.bnd_ptr[j + 1]; ++s) ax += op.partial[s];
    }
    l0_finish<KIND>(g, ax, xg, b, dinv, xout, d, c1, c2);
}

// threads per row of a transfer operator: rows of up to ~8 entries (the Q2 -> Q1 embedding
// averages 3.2) are read by one thread each, so a warp keeps 32 rows' gathers in flight
int tpr_for(double avg);
int transfer_tpr(double avg) { return avg <= 8.0 ? 1 : tpr_for(avg); }

// threads per row for a CSR operator of average row length `avg`
int tpr_for(double avg) {
    if (avg <= 3.0) return 1;
    if (avg <= 8.0) return 4;
    if (avg <= 20.0) return 8;
    if (avg <= 48.0) return 16;
    return 32;
}

#define FGB_TPR_DISPATCH(KERNEL, tpr, n, stream, ...)                                                         \
    do {                                                                                                      \
        const int t_ = (tpr);                                                                                 \
        const int g_ = grid_for((long long)(n) * (t_ == 0 ? 1 : t_), kB);                                     \
        switch (t_) {                                                                                         \
            case 0: FGB_LAUNCH(KERNEL<0><<<g_, kB, 0, stream>>>(__VA_ARGS__)); break;                         \
            case 1: FGB_LAUNCH(KERNEL<1><<<g_, kB, 0, stream>>>(__VA_ARGS__)); break;                         \
            case 4: FGB_LAUNCH(KERNEL<4><<<g_, kB, 0, stream>>>(__VA_ARGS__)); break;                         \
            case 8: FGB_LAUNCH(KERNEL<8><<<g_, kB, 0, stream>>>(__VA_ARGS__)); break;                         \
            case 16: FGB_LAUNCH(KERNEL<16><<<g_, kB, 0, stream>>>(__VA_ARGS__)); break;                       \
            default: FGB_LAUNCH(KERNEL<32><<<g_, kB, 0, stream>>>(__VA_ARGS__)); break;                       \
        }                                                                                                     \
    } while (0)

__global__ void k_dense_solve(int n, const float* __restrict__ inv, const float* __restrict__ b, float* __restrict__ x) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n) return;
    const float* row = inv + (size_t)warp * n;
    float acc = 0.f;
    for (int j = lane; j < n; j += 32) acc += row[j] * b[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) x[warp] = acc;
}

// SELL-32 with 4-wide row chunks (the level-0 layout) of a CSR level
void sell4_of(const CsrD& A, std::vector<int64_t>& sptr, std::vector<int32_t>& slen, std::vector<int32_t>& scol,
              std::vector<float>& val) {
    const int n = A.n_rows, ns = (n + 31) / 32;
    sptr.assign(ns + 1, 0);
    slen.assign(ns, 0);
#pragma omp parallel for schedule(static)
    for (int s = 0; s < ns; ++s) {
        int m = 0;
        for (int r = s * 32; r < std::min(n, s * 32 + 32); ++r) m = std::max<int>(m, (int)(A.ptr[r + 1] - A.ptr[r]));
        slen[s] = (m + 3) / 4 * 4;
    }
    for (int s = 0; s < ns; ++s) sptr[s + 1] = sptr[s] + (int64_t)slen[s] * 32;
    scol.resize(sptr[ns]);
    val.resize(sptr[ns]);
#pragma omp parallel for schedule(dynamic, 64)
    for (int s = 0; s < ns; ++s)
        for (int lane = 0; lane < 32; ++lane) {
            const int r = s * 32 + lane;
            const int len = r < n ? (int)(A.ptr[r + 1] - A.ptr[r]) : 0;
            for (int j = 0; j < slen[s]; ++j) {
                const int64_t pos = sptr[s] + ((int64_t)(j / 4) * 32 + lane) * 4 + j % 4;
                if (j < len) {
                    scol[pos] = A.col[A.ptr[r] + j];
                    val[pos] = (float)A.val[A.ptr[r] + j];
                } else {
                    scol[pos] = r < n ? r : 0;
                }
            }
        }
}

void upload_csr32(const CsrD& M, DBuf<int64_t>& ptr, DBuf<int32_t>& col, DBuf<float>& val, cudaStream_t s) {
    ptr.upload(M.ptr, s);
    if (M.nnz() > 0) {
        col.upload(M.col, s);
        std::vector<float> v(M.val.size());
        const long long nv = (long long)v.size();
#pragma omp parallel for schedule(static)
        for (long long k = 0; k < nv; ++k) v[k] = (float)M.val[k];
        val.upload(v, s);
    } else {
        col.resize(1);
        val.resize(1);
    }
}

}  // namespace

AmgDevice::AmgDevice(const AmgHost& h, cudaStream_t stream, const int64_t* l0_sptr, const int32_t* l0_slen,
                     const int32_t* l0_scol, const float* l0_val, const float* l0_dinv)
    : stream_(stream), n_coarse_(h.n_coarse) {
    std::ostringstream ds;
    const int L = (int)h.levels.size();
    for (int l = 0; l < L; ++l) {
        const AmgHostLevel& hl = h.levels[l];
        auto lv = std::make_unique<AmgDevLevel>();
        lv->n = hl.A.n_rows;
        lv->lambda = hl.lambda;
        lv->cheb_degree = lv->built_degree = std::max(1, hl.cheb_degree);
        lv->cheb_lo = lv->built_lo = hl.cheb_lo;
        if (l == 0) {
            lv->sptr = l0_sptr;
            lv->slen = l0_slen;
            lv->scol = l0_scol;
            lv->val = l0_val;
            lv->dinv = l0_dinv;
        } else if (l < L - 1 && hl.dev_val) {
            lv->sptr = hl.dev_sptr;
            lv->slen = hl.dev_slen;
            lv->scol = hl.dev_scol;
            lv->val = hl.dev_val;
            lv->dinv = hl.dev_dinv;
            lv->tpr = 0;
        } else if (l < L - 1) {
            std::vector<float> di(lv->n, 1.f);
#pragma omp parallel for schedule(static)
            for (int i = 0; i < lv->n; ++i)
                for (int64_t k = hl.A.ptr[i]; k < hl.A.ptr[i + 1]; ++k)
                    if (hl.A.col[k] == i) di[i] = (float)(1.0 / hl.A.val[k]);
            lv->own_dinv.upload(di, stream);
            lv->dinv = lv->own_dinv.get();
            const double avg = (double)hl.A.nnz() / std::max(1, lv->n);
            if (lv->n >= 32768 && avg <= 48.0) {
                // large, moderately sparse level: the level-0 SELL layout, one thread per row
                std::vector<int64_t> sp;
                std::vector<int32_t> sl, sc;
                std::vector<float> sv;
                sell4_of(hl.A, sp, sl, sc, sv);
                lv->a_ptr.upload(sp, stream);
                lv->own_slen.upload(sl, stream);
                lv->a_col.upload(sc, stream);
                lv->a_val.upload(sv, stream);
                lv->sptr = lv->a_ptr.get();
                lv->slen = lv->own_slen.get();
                lv->tpr = 0;
            } else {
                upload_csr32(hl.A, lv->a_ptr, lv->a_col, lv->a_val, stream);
                lv->sptr = lv->a_ptr.get();
                lv->slen = nullptr;
                lv->tpr = tpr_for(avg);
            }
            lv->scol = lv->a_col.get();
            lv->val = lv->a_val.get();
        }
        if (l == 0) lv->tpr = 0;
        if (l < L - 1) {
            lv->n_coarse = hl.P.n_cols;
            if (!hl.transfers_on_device) {
                upload_csr32(hl.P, lv->p_ptr, lv->p_col, lv->p_val, stream);
                upload_csr32(hl.R, lv->r_ptr, lv->r_col, lv->r_val, stream);
                lv->p_tpr = transfer_tpr((double)hl.P.nnz() / std::max(1, hl.P.n_rows));
                lv->r_tpr = transfer_tpr((double)hl.R.nnz() / std::max(1, hl.R.n_rows));
            }
        }
        lv->b.resize(lv->n);
        lv->xa.resize(lv->n);
        lv->xb.resize(lv->n);
        lv->d.resize(lv->n);
        lv->r.resize(lv->n);
        lv->bin = lv->b.get();
        if (l == 0) nnz0_ = hl.A.nnz();
        ds << (l ? " " : "") << lv->n << ":" << (l == L - 1 ? (long long)lv->n * lv->n : hl.A.nnz())
           << (l == L - 1 ? ":dense" : "");
        lv_.push_back(std::move(lv));
    }
    std::vector<float> inv(h.coarse_inv.begin(), h.coarse_inv.end());
    coarse_inv_.upload(inv, stream);
    desc_ = ds.str();
    FGB_CUDA(cudaStreamSynchronize(stream));
}

AmgDevice::~AmgDevice() = default;

void AmgDevice::set_coarse_cycles(int level, int cycles) {
    FGB_REQUIRE(level >= 0 && cycles >= 1 && cycles <= 8, "coarse cycles: level >= 0, 1..8 cycles");
    if ((int)coarse_cycles_.size() <= level) coarse_cycles_.resize(level + 1, 1);
    coarse_cycles_[level] = cycles;
}

void AmgDevice::set_level_smoothing(int level, int degree, double lo) {
    FGB_REQUIRE(level >= 0 && level < (int)lv_.size() && degree >= 0 && degree <= 15 && lo >= 0 && lo < 1,
                "level smoothing: an existing level, degree 0..15, interval 0..1");
    AmgDevLevel& L = *lv_[level];
    L.cheb_degree = degree > 0 ? degree : L.built_degree;
    L.cheb_lo = lo > 0 ? lo : L.built_lo;
}

void AmgDevice::adopt_transfers(int level, DBuf<int64_t>&& p_ptr, DBuf<int32_t>&& p_col, DBuf<float>&& p_val,
                                DBuf<int64_t>&& r_ptr, DBuf<int32_t>&& r_col, DBuf<float>&& r_val, int64_t nnz) {
    FGB_REQUIRE(level >= 0 && level + 1 < (int)lv_.size(), "transfers: a level with a coarser one");
    AmgDevLevel& L = *lv_[level];
    FGB_REQUIRE(p_ptr.size() == (size_t)L.n + 1 && r_ptr.size() == (size_t)L.n_coarse + 1,
                "transfers: row pointers of P (fine rows) and R (coarse rows)");
    L.p_ptr = std::move(p_ptr);
    L.p_col = std::move(p_col);
    L.p_val = std::move(p_val);
    L.r_ptr = std::move(r_ptr);
    L.r_col = std::move(r_col);
    L.r_val = std::move(r_val);
    L.p_tpr = transfer_tpr((double)nnz / std::max(1, L.n));
    L.r_tpr = transfer_tpr((double)nnz / std::max(1, L.n_coarse));
}

int AmgDevice::n_levels() const { return (int)lv_.size(); }
void AmgDevice::set_level0_lambda(double lambda) {
    FGB_REQUIRE(lambda > 0 && std::isfinite(lambda), "level-0 lambda_max must be positive");
    lv_[0]->lambda = lambda;
}
std::string AmgDevice::describe() const { return desc_; }

void AmgDevice::cycle(int l) {
    AmgDevLevel& L = *lv_[l];
    const int g = grid_for(L.n, kB);
    if (l == (int)lv_.size() - 1) {
        FGB_LAUNCH(k_dense_solve<<<grid_for((long long)L.n * 32, kB), kB, 0, stream_>>>(L.n, coarse_inv_.get(), L.bin,
                                                                                       L.xb.get()));
        L.x = L.xb.get();
        return;
    }
    // Chebyshev on D^-1 A over [lo, 1.1] x lambda: step k uses d_k = c1_k d_{k-1} + c2_k D^-1 r,
    // rho_0 = 1/sigma, rho_k = 1/(2 sigma - rho_{k-1}), c1_k = rho_k rho_{k-1}, c2_k = 2 rho_k / delta
    const double lmax = 1.1 * L.lambda, lmin = L.cheb_lo * L.lambda;
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin), sigma = theta / delta;
    const int deg = L.cheb_degree;
    float c1[16], c2[16];
    {
        double rho = 1.0 / sigma;
        for (int k = 1; k < deg && k < 16; ++k) {
            const double rn = 1.0 / (2.0 * sigma - rho);
            c1[k] = (float)(rn * rho);
            c2[k] = (float)(2.0 * rn / delta);
            rho = rn;
        }
    }
    const float inv_theta = (float)(1.0 / theta);
    const Op A{L.n, L.sptr, L.slen, L.scol, L.val, L.dinv};
    LaunchTimer* tm = l == 0 ? &smoother_timer : nullptr;
    // pre-smoothing from zero: iterate k writes buffer k; the buffers alternate so that the
    // last one (k = deg-1) is xb
    auto pre_buf = [&](int k) { return ((deg - 1 - k) % 2 == 0) ? L.xb.get() : L.xa.get(); };
    FGB_LAUNCH(k_cheb_zero<<<g, kB, 0, stream_>>>(L.n, L.dinv, L.bin, pre_buf(0), L.d.get(), inv_theta));
    for (int k = 1; k < deg; ++k) {
        if (tm) tm->begin(stream_);
        if (l == 0) level0_apply(0, pre_buf(k - 1), pre_buf(k), c1[k], c2[k]);
        else FGB_TPR_DISPATCH(k_cheb_step, L.tpr, L.n, stream_, A, L.bin, pre_buf(k - 1), pre_buf(k), L.d.get(), c1[k], c2[k]);
        if (tm) tm->end(stream_);
    }
    // coarse-grid correction
    if (l == 0) level0_apply(1, L.xb.get(), L.r.get(), 0.f, 0.f);
    else FGB_TPR_DISPATCH(k_residual, L.tpr, L.n, stream_, A, L.bin, L.xb.get(), L.r.get());
    AmgDevLevel& C = *lv_[l + 1];
    FGB_TPR_DISPATCH(k_csr_apply, L.r_tpr, C.n, stream_, C.n, L.r_ptr.get(), L.r_col.get(), L.r_val.get(), L.r.get(),
                     C.b.get(), 0);
    cycle(l + 1);
    const int ncyc = l < (int)coarse_cycles_.size() ? coarse_cycles_[l] : 1;
    if (ncyc > 1 && l + 1 < (int)lv_.size() - 1) {
        // further cycles of the next level on the residual of the sum so far (the coarsest
        // level is solved exactly, so repeating it adds nothing)
        if (C.xacc.size() != (size_t)C.n) C.xacc.resize(C.n);
        if (C.rtmp.size() != (size_t)C.n) C.rtmp.resize(C.n);
        FGB_CUDA(cudaMemcpyAsync(C.xacc.get(), C.x, sizeof(float) * C.n, cudaMemcpyDeviceToDevice, stream_));
        const Op AC{C.n, C.sptr, C.slen, C.scol, C.val, C.dinv};
        const int gc = grid_for(C.n, kB);
        for (int k = 1; k < ncyc; ++k) {
            FGB_TPR_DISPATCH(k_residual, C.tpr, C.n, stream_, AC, C.b.get(), C.xacc.get(), C.rtmp.get());
            C.bin = C.rtmp.get();
            cycle(l + 1);
            C.bin = C.b.get();
            FGB_LAUNCH(k_add_f<<<gc, kB, 0, stream_>>>(C.n, C.x, C.xacc.get()));
        }
        C.x = C.xacc.get();
    }
    FGB_TPR_DISPATCH(k_csr_apply, L.p_tpr, L.n, stream_, L.n, L.p_ptr.get(), L.p_col.get(), L.p_val.get(), C.x,
                     L.xb.get(), 1);
    // post-smoothing (same polynomial) from the corrected xb; even steps write xa, odd ones xb
    float* xin = L.xb.get();
    for (int k = 0; k < deg; ++k) {
        float* xout = (k % 2 == 0) ? L.xa.get() : L.xb.get();
        if (tm) tm->begin(stream_);
        if (l == 0) level0_apply(0, xin, xout, k == 0 ? -1.f : c1[k], k == 0 ? inv_theta : c2[k]);
        else FGB_TPR_DISPATCH(k_cheb_step, L.tpr, L.n, stream_, A, L.bin, xin, xout, L.d.get(), k == 0 ? -1.f : c1[k],
                              k == 0 ? inv_theta : c2[k]);
        if (tm) tm->end(stream_);
        xin = xout;
    }
    L.x = xin;
}

void AmgDevice::set_level0_ebe(const EbeOperator* op) {
    if (!op) {
        ebe_on_ = false;
        return;
    }
    ebe_ = *op;
    ebe_on_ = true;
    FGB_REQUIRE(op->max_cells <= kCbMaxCells && op->max_dofs <= kCbPer * kCb, "cell blocks too large");
    FGB_REQUIRE(op->n_ke == 378LL * op->n_cells, "element matrices: 378 floats per cell");
    if (ebe_err_.size() != 1) ebe_err_.resize(1);
    FGB_CUDA(cudaMemsetAsync(ebe_err_.get(), 0, sizeof(unsigned), stream_));
    ebe_.err = ebe_err_.get();
    // the cap is a property of the kernel, shared by every mesh: always the largest block's
    const int cap = (int)cb_smem_bytes(kCbMaxCells, kCbPer * kCb);
    FGB_CUDA(cudaFuncSetAttribute(k_cb_apply<0, kSrcKe>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap));
    FGB_CUDA(cudaFuncSetAttribute(k_cb_apply<1, kSrcKe>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap));
    const int cap_g = (int)cb_geo_smem_bytes(kCbMaxCells, kCbPer * kCb);
    FGB_CUDA(cudaFuncSetAttribute(k_cb_apply<0, kSrcGeo>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap_g));
    FGB_CUDA(cudaFuncSetAttribute(k_cb_apply<1, kSrcGeo>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap_g));
    FGB_CUDA(cudaFuncSetAttribute(k_cb_apply<0, kSrcGeo16>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap_g));
    FGB_CUDA(cudaFuncSetAttribute(k_cb_apply<1, kSrcGeo16>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap_g));
    const int cap_s = (int)cb_stream_smem_bytes(kCbMaxCells, kCbPer * kCb);
    FGB_CUDA(cudaFuncSetAttribute(k_cb_apply<0, kSrcRing>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap_s));
    FGB_CUDA(cudaFuncSetAttribute(k_cb_apply<1, kSrcRing>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap_s));
}

unsigned AmgDevice::level0_errors() {
    if (!ebe_on_ || ebe_err_.size() != 1) return 0;
    unsigned h = 0;
    FGB_CUDA(cudaMemcpyAsync(&h, ebe_err_.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    return h;
}

double AmgDevice::smoother_bytes() const {
    const double n = lv_[0]->n;
    if (!ebe_on_) return (double)nnz0_ * 8.0 + 24.0 * n;
    // per cell: K_e (378 x 4), its loc list (27 x 2) and items (28 x 2); per block-local DoF: DoF
    // id, item end, slot and the gathered x; per DoF: b, D^-1, d in and out, x out, the
    // Dirichlet flag; per slot: the partial written and read; per split
    // DoF: its id and slot range
    const double per_cell = ebe_.geo_kind == 2 ? 324.0 : (ebe_.geo_kind == 1 ? 648.0 : 378.0 * 4);
    return ebe_.n_cells * (per_cell + 110.0) + (double)ebe_.n_local * 14.0 + n * 21.0 + ebe_.n_slots * 8.0 +
           ebe_.n_bnd * 8.0;
}

// one level-0 operator application fused with the Chebyshev update (kind 0) or the residual
// (kind 1, c1/c2 unused, result in xout)
void AmgDevice::level0_apply(int kind, const float* xin, float* xout, float c1, float c2) {
    AmgDevLevel& L = *lv_[0];
    const int g = grid_for(L.n, kB);
    if (ebe_on_) {
        const int gb = grid_for(ebe_.n_bnd, kB);
        const int src = ebe_.geo_kind == 2 ? kSrcGeo16 : (ebe_.geo_kind == 1 ? kSrcGeo : (stream_ke_ ? kSrcRing : kSrcKe));
        const size_t smem = src == kSrcRing ? cb_stream_smem_bytes(ebe_.max_cells, ebe_.max_dofs)
                            : (src == kSrcGeo || src == kSrcGeo16) ? cb_geo_smem_bytes(ebe_.max_cells, ebe_.max_dofs)
                                                                   : cb_smem_bytes(ebe_.max_cells, ebe_.max_dofs);
        const int threads = src == kSrcRing ? kCb + 32 : kCb;
        float* dd = kind == 0 ? L.d.get() : nullptr;
        const float cc1 = kind == 0 ? c1 : 0.f, cc2 = kind == 0 ? c2 : 0.f;
#define FGB_CB_APPLY(K, S) \
    FGB_LAUNCH(k_cb_apply<K, S><<<ebe_.n_blocks, threads, smem, stream_>>>(ebe_, L.dinv, L.bin, xin, xout, dd, cc1, cc2))
        switch (src * 2 + kind) {
            case kSrcKe * 2: FGB_CB_APPLY(0, kSrcKe); break;
            case kSrcKe * 2 + 1: FGB_CB_APPLY(1, kSrcKe); break;
            case kSrcRing * 2: FGB_CB_APPLY(0, kSrcRing); break;
            case kSrcRing * 2 + 1: FGB_CB_APPLY(1, kSrcRing); break;
            case kSrcGeo * 2: FGB_CB_APPLY(0, kSrcGeo); break;
            case kSrcGeo * 2 + 1: FGB_CB_APPLY(1, kSrcGeo); break;
            case kSrcGeo16 * 2: FGB_CB_APPLY(0, kSrcGeo16); break;
            default: FGB_CB_APPLY(1, kSrcGeo16); break;
        }
#undef FGB_CB_APPLY
        if (gb) {
            if (kind == 0)
                FGB_LAUNCH(k_cb_finish<0><<<gb, kB, 0, stream_>>>(ebe_, L.dinv, L.bin, xin, xout, L.d.get(), c1, c2));
            else
                FGB_LAUNCH(k_cb_finish<1><<<gb, kB, 0, stream_>>>(ebe_, L.dinv, L.bin, xin, xout, nullptr, 0.f, 0.f));
        }
        return;
    }
    const Op A{L.n, L.sptr, L.slen, L.scol, L.val, L.dinv};
    if (kind == 0)
        FGB_LAUNCH(k_cheb_step<0><<<g, kB, 0, stream_>>>(A, L.bin, xin, xout, L.d.get(), c1, c2));
    else
        FGB_LAUNCH(k_residual<0><<<g, kB, 0, stream_>>>(A, L.bin, xin, xout));
}

double AmgDevice::time_smoother(int reps) {
    AmgDevLevel& L = *lv_[0];
    const int g = grid_for(L.n, kB);
    Op A{L.n, L.sptr, L.slen, L.scol, L.val, L.dinv};
    // right-hand side: the level's own buffer, zeroed, so nothing of the caller is read
    FGB_CUDA(cudaMemsetAsync(L.b.get(), 0, sizeof(float) * L.n, stream_));
    FGB_CUDA(cudaMemsetAsync(L.xa.get(), 0, sizeof(float) * L.n, stream_));
    FGB_CUDA(cudaMemsetAsync(L.d.get(), 0, sizeof(float) * L.n, stream_));
    cudaEvent_t e0, e1;
    FGB_CUDA(cudaEventCreate(&e0));
    FGB_CUDA(cudaEventCreate(&e1));
    const float* bin = L.bin;
    L.bin = L.b.get();
    auto launch = [&](int i) {
        float* xi = (i & 1) ? L.xb.get() : L.xa.get();
        float* xo = (i & 1) ? L.xa.get() : L.xb.get();
        level0_apply(0, xi, xo, 0.5f, 0.5f);
    };
    for (int i = 0; i < 3; ++i) launch(i);
    FGB_CUDA(cudaEventRecord(e0, stream_));
    for (int i = 0; i < reps; ++i) launch(i + 1);
    FGB_CUDA(cudaEventRecord(e1, stream_));
    FGB_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    FGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    L.bin = bin;
    (void)g;
    (void)A;
    return ms / reps;
}

const float* AmgDevice::vcycle(const float* r) {
    AmgDevLevel& L0 = *lv_[0];
    L0.bin = r;
    cycle(0);
    FGB_CUDA(cudaGetLastError());
    return L0.x;
}

void AmgDevice::level0_residual(const float* b, const float* x, float* y) {
    AmgDevLevel& L0 = *lv_[0];
    const float* keep = L0.bin;
    L0.bin = b;
    level0_apply(1, x, y, 0.f, 0.f);
    L0.bin = keep;
}

}  // namespace fgb
