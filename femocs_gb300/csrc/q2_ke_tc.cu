// Q2 element matrices on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// K_e is a product of a per-cell matrix and a constant table. With M_q = J_q^-1 J_q^-T and the
// reference gradients g_i(q) of the 27 shape functions,
//     K_e[i][j] = sum_q w_q |det J_q| g_i^T M_q g_j = sum_(q,kl) C[(q,kl)] T[(q,kl), (i,j)],
// C[(q,kl)] = w_q |det J_q| M_q[k][l] (k <= l: 27 x 6 = 162 values per cell) and
// T[(q,kl), (i,j)] = g_i[k] g_j[l] + g_i[l] g_j[k] (k < l) or g_i[k] g_j[k] (k = l), over the 378
// packed upper-triangle entries (i <= j). A tile of 128 cells is one GEMM, K(128 x 378) =
// C(128 x 162) T(162 x 378).
//
// FP64 accuracy from BF16 tensor cores, by error-free splitting (the Ozaki scheme): each row of
// C and each column of T is scaled by a power of two into [-1, 1] and cut into six slices of
// integers in [-128, 128] (exact in BF16), s_0 2^-7 + s_1 2^-15 + ... + s_5 2^-47 (each slice
// the rounded remainder of the ones before, 47 bits in all). A product of two slices is an
// integer below 2^14 in magnitude, and the slice pairs (a, b) with a + b = l (l = 0..5; 21
// pairs) accumulate over K = 162 into one FP32 accumulator per level l: at most 6 x 162 x 2^14
// < 2^24, so every FP32 sum is exact. The levels are combined in FP64,
// K = 2^(e_cell + e_entry) sum_l acc_l 2^(-14 - 8 l); the pairs dropped (a + b > 5) and the
// slicing leave ~2^-46 of the row/column scale (a numpy emulation of this exact arithmetic
// gives 5e-14 of max |K_e| on the nanotip meshes).
//
// One persistent CTA (256 threads) per SM, tiles of 128 cells:
//   1  the threads compute C (Jacobians of the trilinear map at the 27 Gauss points, in
//      double-float arithmetic on FP32 pairs, ~48 bits: GB300's FP64 pipe runs at 1/64 of
//      FP32), keep it in shared memory as FP64, find each row's exponent and write the six
//      BF16 slices of their rows into this CTA's global scratch, already in the K-major
//      core-matrix layout the MMA reads (8 rows x 16 bytes per core matrix, no swizzle);
//   2  for each of 8 N-tiles of 48 entries, one thread moves the N-tile's six T slices and, one
//      after another, the six C slices into shared memory with cp.async.bulk (mbarrier
//      complete_tx) and issues tcgen05.mma (M = 128, N = 48, K = 16, BF16 in, FP32 in TMEM);
//      tcgen05.commit signals when a C slot may be refilled and when the N-tile is done;
//   3  the eight warps read the six level accumulators with tcgen05.ld (warp w: TMEM lanes
//      32 (w % 4) .., i.e. 32 cells, and half of the N-tile's columns), combine them into an
//      FP32 pair (TwoSum), scale it into FP64 on the integer pipes and store the 378 packed
//      FP64 entries per cell.
// Every mbarrier wait is bounded; a wait that runs out sets an error word (checked by the host
// after the launch) and the kernel finishes without further tensor-core work, freeing its TMEM.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "fem_q2.h"

namespace fgb {

namespace {

constexpr int kTcThreads = 256;
constexpr int kTcM = 128;                   // cells per tile (MMA M)
constexpr int kTcN = 48;                    // packed entries per N-tile (MMA N)
constexpr int kTcNT = 8;                    // N-tiles: 8 x 48 = 384 >= 378
constexpr int kTcK = 176;                   // 162 padded to 11 MMA K-steps of 16
constexpr int kTcKS = kTcK / 16;
constexpr int kTcS = 6;                     // slices per operand
constexpr uint32_t kTcSBO = (kTcK / 8) * 128;  // bytes between 8-row core-matrix groups: 2816
constexpr uint32_t kTcLBO = 128;               // bytes between core matrices along K
constexpr int kTcASlice = kTcM * kTcK * 2;     // 45056 B: one C slice of a tile
constexpr int kTcBSlice = kTcN * kTcK * 2;     // 16896 B: one T slice of an N-tile
constexpr int kTcTmemCols = 512;
constexpr int kTcLevelCols = 64;            // TMEM columns per level accumulator (48 used)
constexpr unsigned kTcSpin = 1u << 22;

// shared memory: T slices of the N-tile, two C slots (phase 1 keeps the tile's FP64 C there),
// the trilinear-map gradient table, row exponents, barriers, the TMEM address
constexpr size_t kTcOffT = 0;
constexpr size_t kTcOffA = kTcOffT + kTcS * (size_t)kTcBSlice;          // 101376
constexpr size_t kTcOffD1 = kTcOffA + 2 * (size_t)kTcASlice;            // 191488 (end of phase-1 data)
constexpr size_t kTcOffExp = kTcOffD1;                                  // 191488
constexpr size_t kTcOffBar = kTcOffExp + kTcM * sizeof(int);            // 197184
constexpr size_t kTcOffTmem = kTcOffBar + 8 * sizeof(uint64_t);         // 197248
constexpr size_t kTcSmem = kTcOffTmem + 16;
// phase 1 keeps C (128 x 162) and the cells' scaled trilinear coefficients (128 x 21 pairs) in the
// T and C regions
static_assert(kTcM * (162 * sizeof(double) + 21 * sizeof(float2) + sizeof(int)) <= kTcOffD1,
              "phase 1 data in the T and C regions");
static_assert(kTcSmem <= 232448, "shared memory per CTA");

__constant__ double c_tc_w[27];
__constant__ float2 c_tc_wdf[27];        // the same weights as FP32 (hi, lo) pairs
__constant__ int c_tc_corner[8];         // lattice index of femocs corner k

// ------------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t su32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    // start address, leading (K) and stride (M/N) byte offsets, all >> 4; bits 46-48 = 0b001;
    // base offset 0, absolute LBO mode, no swizzle
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}
// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, N, M
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_alloc(uint32_t* dst, uint32_t ncols) {  // whole warp
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {  // whole warp
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// 8 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void mb_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mb_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mb_wait(uint64_t* bar, unsigned parity) {
    for (unsigned i = 0; i < kTcSpin; ++i) {
        unsigned ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(su32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     su32(dst)),
                 "l"(src), "r"(bytes), "r"(su32(bar))
                 : "memory");
}

// byte offset of element (row r, k) in a K-major, unswizzled core-matrix tile of kTcK columns
__host__ __device__ __forceinline__ uint32_t tc_off(int r, int k) {
    return (uint32_t)(r >> 3) * kTcSBO + (uint32_t)(k >> 3) * 128u + (uint32_t)(r & 7) * 16u + (uint32_t)(k & 7) * 2u;
}

// six rounded slices of v scaled by 2^-e (|v 2^-e| <= 1): integers in [-128, 128],
// v 2^-e ~ sum_i s_i 2^(-7 - 8 i), as BF16 bit patterns
__host__ __device__ inline void tc_slices(double v, int e, uint16_t (&out)[kTcS]) {
    const double r = ldexp(v, -e);
    long long m = llrint(ldexp(r, 52));  // |m| <= 2^52
    int sh = 45;
    for (int i = 0; i < kTcS; ++i) {
        const long long s = (m + (1LL << (sh - 1))) >> sh;  // round half up, arithmetic shift
        m -= s * (1LL << sh);
        const float f = (float)s;                             // |s| <= 128: exact in BF16
        uint32_t bits;
        memcpy(&bits, &f, 4);
        out[i] = (uint16_t)(bits >> 16);
        sh -= 8;
    }
}

// the same slices from the bit pattern of v with integer operations only (no FP64 pipe): v =
// mant 2^(E - 1075); m = round(v 2^(52 - e)) = round(mant 2^-(e + 1023 - E)), e from the row's
// largest magnitude, so the shift is >= 1; subnormal values count as 0
__device__ __forceinline__ void tc_slices_bits(uint64_t bits, int e, uint16_t (&out)[kTcS]) {
    const int E = (int)((bits >> 52) & 0x7FF);
    long long m = 0;
    if (E != 0) {
        const uint64_t mant = (bits & ((1ull << 52) - 1)) | (1ull << 52);
        const int sft = e + 1023 - E;
        m = sft >= 64 ? 0 : (long long)((mant + (1ull << (sft - 1))) >> sft);
        if (bits >> 63) m = -m;
    }
    int sh = 45;
#pragma unroll
    for (int i = 0; i < kTcS; ++i) {
        const long long sl = (m + (1LL << (sh - 1))) >> sh;
        m -= sl * (1LL << sh);
        out[i] = (uint16_t)(__float_as_uint((float)sl) >> 16);
        sh -= 8;
    }
}

// exponent e with |x| 2^-e <= 1 for every x of magnitude at most mx (0 for mx = 0)
__host__ __device__ inline int tc_exponent(double mx) {
    if (!(mx > 0)) return 0;
    int e;
    frexp(mx, &e);  // mx = f 2^e, f in [0.5, 1)
    return e;
}

// ------------------------------------------------------------------ self test
// One 128 x 48 x 32 product of small integers (two MMAs, the second accumulating) checked on the
// host: validates the descriptors, the instruction descriptor and the TMEM lane/column layout
// with the same helpers the element kernel uses.
__global__ void __launch_bounds__(128) k_tc_selftest(float* __restrict__ out, unsigned* __restrict__ err) {
    __shared__ __align__(1024) unsigned char sA[128 * 32 * 2];
    __shared__ __align__(1024) unsigned char sB[48 * 32 * 2];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr uint32_t SBO = (32 / 8) * 128;  // K = 32: 4 core matrices per 8-row group
    auto off = [&](int r, int k) { return (uint32_t)(r >> 3) * SBO + (uint32_t)(k >> 3) * 128u + (r & 7) * 16u + (k & 7) * 2u; };
    for (int i = tid; i < 128 * 32; i += 128) {
        const int r = i / 32, k = i % 32;
        const __nv_bfloat16 a = __float2bfloat16_rn((float)(((r * 3 + k * 5) % 7) - 3));
        *reinterpret_cast<__nv_bfloat16*>(sA + off(r, k)) = a;
    }
    for (int i = tid; i < 48 * 32; i += 128) {
        const int r = i / 32, k = i % 32;
        const __nv_bfloat16 b = __float2bfloat16_rn((float)(((r * 2 + k * 3) % 5) - 2));
        *reinterpret_cast<__nv_bfloat16*>(sB + off(r, k)) = b;
    }
    if (tid == 0) {
        mb_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (warp == 0) tc_alloc(&tmem, 64);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t t0 = tmem;
    if (tid == 0) {
        const uint32_t id = tc_idesc(128, 48);
        for (int ks = 0; ks < 2; ++ks)
            tc_mma(t0, tc_desc(su32(sA) + ks * 256, 128, SBO), tc_desc(su32(sB) + ks * 256, 128, SBO), id, ks > 0);
        tc_commit(&bar);
    }
    __syncwarp();
    const bool ok = mb_wait(&bar, 0);
    if (!ok && lane == 0) atomicOr(err, 1u);
    tc_fence_after();
    if (ok) {
        for (int c = 0; c < 48; c += 8) {
            float v[8];
            tc_ld8(t0 + ((uint32_t)(32 * warp) << 16) + c, v);
            for (int j = 0; j < 8; ++j) out[(32 * warp + lane) * 48 + c + j] = v[j];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(t0, 64);
}


// ---- double-float arithmetic (an FP32 pair hi + lo, ~48 bits) for the per-point factors:
// error-free sums (Knuth's TwoSum) and products (FMA), renormalised after each operation.
// The intrinsics keep the compiler from contracting the error terms.
struct Df {
    float h, l;
};
__device__ __forceinline__ Df df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ Df df_fast_two_sum(float a, float b) {  // |a| >= |b| or a = 0
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ Df df_add(Df a, Df b) {
    Df s = df_two_sum(a.h, b.h);
    const Df t = df_two_sum(a.l, b.l);
    s = df_fast_two_sum(s.h, __fadd_rn(s.l, t.h));
    return df_fast_two_sum(s.h, __fadd_rn(s.l, t.l));
}
__device__ __forceinline__ Df df_neg(Df a) { return {-a.h, -a.l}; }
__device__ __forceinline__ Df df_mul(Df a, Df b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return df_fast_two_sum(p, e);
}
// a b - c d
__device__ __forceinline__ Df df_mul_sub(Df a, Df b, Df c, Df d) { return df_add(df_mul(a, b), df_neg(df_mul(c, d))); }
// s a for s in {-1, 0, 1} (exact)
__device__ __forceinline__ Df df_sgn(int s, Df a) { return s > 0 ? a : (s < 0 ? df_neg(a) : Df{0.f, 0.f}); }

// f 2^k as an FP64 value on the integer pipes: the float's sign, exponent and mantissa moved
// into the double layout (exact); zeros, subnormals and exponents that would leave the normal
// range take the FP64 conversion and scaling instead. -1022 <= k <= 1023.
__device__ __forceinline__ double tc_scaled_f64(float f, int k) {
    const uint32_t u = __float_as_uint(f);
    const int e = (int)((u >> 23) & 0xffu);
    const int ed = e - 127 + 1023 + k;
    if (e == 0 || e == 255 || ed <= 0 || ed >= 2047)
        return (double)f * __longlong_as_double((long long)(k + 1023) << 52);
    const uint64_t d = ((uint64_t)(u >> 31) << 63) | ((uint64_t)ed << 52) | ((uint64_t)(u & 0x7fffffu) << 29);
    return __longlong_as_double((long long)d);
}

// ------------------------------------------------------------------ element matrices
// the six packed symmetric M entries in K order: (0,0) (1,1) (2,2) (0,1) (0,2) (1,2)
__global__ void __launch_bounds__(kTcThreads, 1)
    k_q2_ke_tc(int nc, const int32_t* __restrict__ cd, const double* __restrict__ dxyz, double* __restrict__ ke,
               const uint16_t* __restrict__ tsl, const int* __restrict__ texp, unsigned char* __restrict__ scratch,
               unsigned* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char* sT = sm + kTcOffT;
    unsigned char* sA = sm + kTcOffA;
    double* sC = reinterpret_cast<double*>(sm);  // phase 1 only: 128 x 162 over the T and C regions
    // phase 1: per cell the trilinear coefficients f1..f7 (x, y, z), scaled by 2^-s with s the
    // exponent of the largest, as FP32 pairs, and s
    float2* sFd = reinterpret_cast<float2*>(sC + kTcM * 162);
    int* sFs = reinterpret_cast<int*>(sFd + kTcM * 21);
    int* sExp = reinterpret_cast<int*>(sm + kTcOffExp);
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + kTcOffBar);  // 0 T, 1-2 C full, 3-4 C free, 5 done
    uint32_t* sTmem = reinterpret_cast<uint32_t*>(sm + kTcOffTmem);
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    unsigned char* scr = scratch + (size_t)blockIdx.x * kTcS * kTcASlice;
    if (tid == 0) {
        s_abort = 0;
        for (int k = 0; k < 6; ++k) mb_init(&bars[k], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc_alloc(sTmem, kTcTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *sTmem;
    const uint32_t idesc = tc_idesc(kTcM, kTcN);
    unsigned n_nt = 0;  // N-tiles this CTA has processed: the phase counter of its barriers
    const int n_tiles = (nc + kTcM - 1) / kTcM;
    for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const int c0 = tile * kTcM;
        // ---- 1a: the trilinear map x = f0 + f1 xi + f2 eta + f3 zeta + f4 xi eta + f5 xi zeta +
        // f6 eta zeta + f7 xi eta zeta of each cell (femocs corner signs) in FP64, scaled and
        // kept as FP32 pairs; then C per (cell, Gauss point)
        if (tid < kTcM) {
            const int c = c0 + tid;
            double F[24];
#pragma unroll
            for (int r = 0; r < 24; ++r) F[r] = 0.0;
            if (c < nc) {
                const int hx[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, hy[8] = {-1, -1, 1, 1, -1, -1, 1, 1},
                          hz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const int d = __ldg(cd + 27 * (size_t)c + c_tc_corner[k]);
                    const int sg[8] = {1, hx[k], hy[k], hz[k], hx[k] * hy[k], hx[k] * hz[k], hy[k] * hz[k],
                                       hx[k] * hy[k] * hz[k]};
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const double x = 0.125 * __ldg(dxyz + 3 * (size_t)d + a);
#pragma unroll
                        for (int r = 0; r < 8; ++r) F[3 * r + a] += sg[r] > 0 ? x : -x;
                    }
                }
            }
            // scale by the largest |f1..f7| (its exponent, by the bit pattern), then FP32 pairs
            unsigned long long mx = 0;
#pragma unroll
            for (int r = 3; r < 24; ++r)
                mx = max(mx, (unsigned long long)__double_as_longlong(F[r]) & 0x7FFFFFFFFFFFFFFFull);
            const int sc = mx == 0 ? 0 : (int)(mx >> 52) - 1023;
            const double down = __longlong_as_double((long long)(1023 - sc) << 52);
#pragma unroll
            for (int r = 3; r < 24; ++r) {
                const double v = F[r] * down;
                const float h = (float)v;
                sFd[21 * tid + r - 3] = make_float2(h, (float)(v - (double)h));
            }
            sFs[tid] = sc;
        }
        __syncthreads();
        for (int it = tid; it < kTcM * 27; it += kTcThreads) {
            const int cl = it / 27, q = it - 27 * (it / 27), c = c0 + cl;
            double* out = sC + cl * 162 + 6 * q;
            if (c >= nc) {
                for (int m = 0; m < 6; ++m) out[m] = 0.0;
                continue;
            }
            // per (cell, Gauss point) in double-float, on the scaled coefficients f' = f 2^-s:
            // J columns d x / d xi = f1 + f4 eta + f5 zeta + f7 eta zeta, ... with the Gauss
            // coordinates sx g, sy g, sz g (g = sqrt(3/5), s in {-1, 0, 1}); then
            // C = w |det J| J^-1 J^-T = (w / |det J|) adj(J) adj(J)^T, which scales as a length:
            // C = C' 2^s
            const int sx = q % 3 - 1, sy = (q / 3) % 3 - 1, sz = q / 9 - 1;
            // sqrt(3/5) and 3/5 as FP32 pairs (hi = the FP32 rounding, lo = the remainder)
            const Df g = {0x1.8c97f0p-1f, -0x1.7811b8p-26f}, g2 = {0x1.333334p-1f, -0x1.99999ap-26f};
            const float2* Fp = sFd + 21 * cl;
            auto f = [&](int r, int a) {  // coefficient f_r, component a
                const float2 v = Fp[3 * (r - 1) + a];
                return Df{v.x, v.y};
            };
            Df J[3][3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                // d/d xi: f1 + g (sy f4 + sz f5) + g^2 sy sz f7, and the same pattern for eta, zeta
                J[a][0] = df_add(df_add(f(1, a), df_mul(g, df_add(df_sgn(sy, f(4, a)), df_sgn(sz, f(5, a))))),
                                 df_mul(g2, df_sgn(sy * sz, f(7, a))));
                J[a][1] = df_add(df_add(f(2, a), df_mul(g, df_add(df_sgn(sx, f(4, a)), df_sgn(sz, f(6, a))))),
                                 df_mul(g2, df_sgn(sx * sz, f(7, a))));
                J[a][2] = df_add(df_add(f(3, a), df_mul(g, df_add(df_sgn(sx, f(5, a)), df_sgn(sy, f(6, a))))),
                                 df_mul(g2, df_sgn(sx * sy, f(7, a))));
            }
            Df adj[3][3];  // J^-1 = adj / det, adj[k][a] for d xi_k / d x_a
            adj[0][0] = df_mul_sub(J[1][1], J[2][2], J[1][2], J[2][1]);
            adj[1][0] = df_mul_sub(J[1][2], J[2][0], J[1][0], J[2][2]);
            adj[2][0] = df_mul_sub(J[1][0], J[2][1], J[1][1], J[2][0]);
            adj[0][1] = df_mul_sub(J[0][2], J[2][1], J[0][1], J[2][2]);
            adj[1][1] = df_mul_sub(J[0][0], J[2][2], J[0][2], J[2][0]);
            adj[2][1] = df_mul_sub(J[0][1], J[2][0], J[0][0], J[2][1]);
            adj[0][2] = df_mul_sub(J[0][1], J[1][2], J[0][2], J[1][1]);
            adj[1][2] = df_mul_sub(J[0][2], J[1][0], J[0][0], J[1][2]);
            adj[2][2] = df_mul_sub(J[0][0], J[1][1], J[0][1], J[1][0]);
            Df det = df_add(df_add(df_mul(J[0][0], adj[0][0]), df_mul(J[0][1], adj[1][0])), df_mul(J[0][2], adj[2][0]));
            if (det.h < 0.f) det = df_neg(det);
            // 1 / |det J|: the FP32 reciprocal, then one Newton-Raphson step in double-float
            // (y + y (1 - d y); the error squares: 2^-23 -> 2^-46)
            const Df y0 = {__frcp_rn(det.h), 0.f};
            const Df e1 = df_add(Df{1.f, 0.f}, df_neg(df_mul(det, y0)));
            const Df y = df_add(y0, df_mul(y0, e1));
            const float2 wq = c_tc_wdf[q];
            const Df sw = df_mul(Df{wq.x, wq.y}, y);
            const int kk[6] = {0, 1, 2, 0, 0, 1}, ll[6] = {0, 1, 2, 1, 2, 2};
            const int sc = sFs[cl];
#pragma unroll
            for (int m = 0; m < 6; ++m) {
                const Df mk = df_add(df_add(df_mul(adj[kk[m]][0], adj[ll[m]][0]), df_mul(adj[kk[m]][1], adj[ll[m]][1])),
                                     df_mul(adj[kk[m]][2], adj[ll[m]][2]));
                const Df v = df_mul(sw, mk);
                out[m] = tc_scaled_f64(v.h, sc) + tc_scaled_f64(v.l, sc);
            }
        }
        __syncthreads();
        // ---- 1b: row exponents and the six slices of every row into the scratch, two threads
        // per row (k-groups of 8: 0..10 and 11..21; K = 162..175 are zero)
        {
            const int r = tid >> 1, half = tid & 1;
            const double* row = sC + r * 162;
            // largest magnitude by its bit pattern (non-negative doubles order like integers)
            unsigned long long mx = 0;
            for (int k = half * 81; k < half * 81 + 81; ++k)
                mx = max(mx, (unsigned long long)__double_as_longlong(row[k]) & 0x7FFFFFFFFFFFFFFFull);
            mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
            const int Em = (int)(mx >> 52);
            const int e = mx == 0 ? 0 : (Em == 0 ? -1021 : Em - 1022);  // frexp exponent of the maximum
            if (half == 0) sExp[r] = e;
            for (int g = half * 11; g < half * 11 + 11; ++g) {
                uint32_t pk[kTcS][4];
#pragma unroll
                for (int j = 0; j < 8; j += 2) {
                    uint16_t o0[kTcS], o1[kTcS];
                    const int k = 8 * g + j;
                    tc_slices_bits(k < 162 ? (uint64_t)__double_as_longlong(row[k]) : 0ull, e, o0);
                    tc_slices_bits(k + 1 < 162 ? (uint64_t)__double_as_longlong(row[k + 1]) : 0ull, e, o1);
#pragma unroll
                    for (int sl = 0; sl < kTcS; ++sl) pk[sl][j / 2] = (uint32_t)o0[sl] | ((uint32_t)o1[sl] << 16);
                }
#pragma unroll
                for (int sl = 0; sl < kTcS; ++sl)
                    *reinterpret_cast<uint4*>(scr + sl * (size_t)kTcASlice + tc_off(r, 8 * g)) =
                        make_uint4(pk[sl][0], pk[sl][1], pk[sl][2], pk[sl][3]);
            }
        }
        // the scratch is read next by bulk copies (the async proxy)
        asm volatile("fence.proxy.async.global;" ::: "memory");
        __syncthreads();
        // ---- 2 and 3 per N-tile of 48 packed entries
        for (int nt = 0; nt < kTcNT; ++nt, ++n_nt) {
            if (tid == 0 && !s_abort) {
                bool ok = true;
                mb_expect_tx(&bars[0], kTcS * kTcBSlice);
                for (int b = 0; b < kTcS; ++b)
                    bulk_copy(sT + b * kTcBSlice, tsl + (size_t)(nt * kTcS + b) * (kTcBSlice / 2), kTcBSlice, &bars[0]);
                for (int a = 0; a < kTcS && ok; ++a) {
                    const int slot = a & 1;
                    const unsigned idx = 3 * n_nt + (a >> 1);  // completion index of the slot's barriers
                    if (a >= 2) ok = mb_wait(&bars[3 + slot], (idx - 1) & 1);  // MMAs of load a - 2 done
                    if (!ok) break;
                    mb_expect_tx(&bars[1 + slot], kTcASlice);
                    bulk_copy(sA + slot * kTcASlice, scr + a * (size_t)kTcASlice, kTcASlice, &bars[1 + slot]);
                    ok = mb_wait(&bars[1 + slot], idx & 1) && (a > 0 || mb_wait(&bars[0], n_nt & 1));
                    if (!ok) break;
                    tc_fence_after();
                    const uint32_t abase = su32(sA + slot * kTcASlice);
                    for (int b = 0; a + b < kTcS; ++b) {
                        const uint32_t d = tmem + (uint32_t)((a + b) * kTcLevelCols);
                        const uint32_t bbase = su32(sT + b * kTcBSlice);
#pragma unroll 1
                        for (int ks = 0; ks < kTcKS; ++ks)
                            tc_mma(d, tc_desc(abase + ks * 256, kTcLBO, kTcSBO), tc_desc(bbase + ks * 256, kTcLBO, kTcSBO),
                                   idesc, (a > 0 || ks > 0) ? 1u : 0u);
                    }
                    tc_commit(&bars[3 + slot]);
                }
                if (ok) {
                    tc_commit(&bars[5]);
                } else {
                    atomicOr(err, 1u);
                    s_abort = 1;
                }
            }
            __syncwarp();
            bool okd = !*(volatile int*)&s_abort;
            if (okd) okd = mb_wait(&bars[5], n_nt & 1);
            okd = __all_sync(0xffffffffu, okd);
            if (!okd && lane == 0) {
                atomicOr(err, 2u);
                s_abort = 1;
            }
            tc_fence_after();
            if (okd) {
                const int quad = warp & 3, half = warp >> 2;
                const int r = 32 * quad + lane, c = c0 + r, e_c = sExp[r];
                for (int ch = 0; ch < 3; ++ch) {
                    const int col = half * 24 + ch * 8;
                    // the levels' exact FP32 sums, scaled by 2^(-14 - 8 l) (exact), added from the
                    // smallest with TwoSum into an FP32 hi/lo pair (~2^-48), then to FP64 exactly
                    float hi[8], lo[8];
#pragma unroll
                    for (int l = kTcS - 1; l >= 0; --l) {
                        float v[8];
                        tc_ld8(tmem + ((uint32_t)(32 * quad) << 16) + (uint32_t)(l * kTcLevelCols + col), v);
                        const float sc = __uint_as_float((uint32_t)(127 - 14 - 8 * l) << 23);
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const float t = __fmul_rn(v[j], sc);
                            if (l == kTcS - 1) {
                                hi[j] = t;
                                lo[j] = 0.f;
                            } else {
                                const float sum = __fadd_rn(t, hi[j]);
                                const float bp = __fsub_rn(sum, t);
                                const float er = __fadd_rn(__fsub_rn(t, __fsub_rn(sum, bp)), __fsub_rn(hi[j], bp));
                                hi[j] = sum;
                                lo[j] = __fadd_rn(lo[j], er);
                            }
                        }
                    }
                    if (c < nc)
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const int e = nt * kTcN + col + j;
                            if (e < 378) {
                                // (hi + lo) 2^k: both parts scaled exactly, one FP64 add (exact:
                                // the pair spans fewer than 53 bits)
                                const int k = e_c + __ldg(texp + e);
                                ke[378 * (size_t)c + e] = tc_scaled_f64(hi[j], k) + tc_scaled_f64(lo[j], k);
                            }
                        }
                }
            }
            tc_fence_before();
            __syncthreads();
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tc_dealloc(tmem, kTcTmemCols);
}

}  // namespace


namespace {
// the constant table T in slices: per N-tile nt and slice b, 48 packed entries x 176 K in the
// K-major core-matrix layout; per entry its power-of-two scale
struct TcTables {
    DBuf<uint16_t> tsl;
    DBuf<int> texp;
};

void build_tc_tables(std::vector<uint16_t>& tsl, std::vector<int>& texp, std::vector<double>& d1, std::vector<double>& w,
                     std::vector<int>& corner) {
    const double g3[3] = {-0.77459666924148337704, 0.0, 0.77459666924148337704};
    const double w3[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
    const int hx[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, hy[8] = {-1, -1, 1, 1, -1, -1, 1, 1},
              hz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
    auto l1 = [](int a, double t) { return a == 0 ? 0.5 * t * (t - 1.0) : (a == 1 ? 1.0 - t * t : 0.5 * t * (t + 1.0)); };
    auto dl = [](int a, double t) { return a == 0 ? t - 0.5 : (a == 1 ? -2.0 * t : t + 0.5); };
    std::vector<double> dn(27 * 27 * 3);
    d1.assign(27 * 8 * 3, 0.0);
    w.assign(27, 0.0);
    for (int q = 0; q < 27; ++q) {
        const int qa = q % 3, qb = (q / 3) % 3, qc = q / 9;
        const double x = g3[qa], y = g3[qb], z = g3[qc];
        w[q] = w3[qa] * w3[qb] * w3[qc];
        for (int L = 0; L < 27; ++L) {
            const int a = L % 3, b = (L / 3) % 3, c = L / 9;
            dn[(q * 27 + L) * 3 + 0] = dl(a, x) * l1(b, y) * l1(c, z);
            dn[(q * 27 + L) * 3 + 1] = l1(a, x) * dl(b, y) * l1(c, z);
            dn[(q * 27 + L) * 3 + 2] = l1(a, x) * l1(b, y) * dl(c, z);
        }
        for (int k = 0; k < 8; ++k) {
            d1[(q * 8 + k) * 3 + 0] = 0.125 * hx[k] * (1 + y * hy[k]) * (1 + z * hz[k]);
            d1[(q * 8 + k) * 3 + 1] = 0.125 * (1 + x * hx[k]) * hy[k] * (1 + z * hz[k]);
            d1[(q * 8 + k) * 3 + 2] = 0.125 * (1 + x * hx[k]) * (1 + y * hy[k]) * hz[k];
        }
    }
    corner.resize(8);
    for (int k = 0; k < 8; ++k) corner[k] = (hx[k] + 1) + 3 * (hy[k] + 1) + 9 * (hz[k] + 1);
    const int kk[6] = {0, 1, 2, 0, 0, 1}, ll[6] = {0, 1, 2, 1, 2, 2};
    std::vector<double> T(162 * 384, 0.0);  // [k][e]
    int e = 0;
    for (int i = 0; i < 27; ++i)
        for (int j = i; j < 27; ++j, ++e)
            for (int q = 0; q < 27; ++q)
                for (int m = 0; m < 6; ++m) {
                    const double* gi = &dn[(q * 27 + i) * 3];
                    const double* gj = &dn[(q * 27 + j) * 3];
                    const int k = kk[m], l = ll[m];
                    T[(6 * q + m) * 384 + e] = k == l ? gi[k] * gj[k] : gi[k] * gj[l] + gi[l] * gj[k];
                }
    texp.assign(384, 0);
    tsl.assign((size_t)kTcNT * kTcS * (kTcBSlice / 2), 0);
    for (int ee = 0; ee < 384; ++ee) {
        double mx = 0.0;
        for (int k = 0; k < 162; ++k) mx = std::max(mx, std::fabs(T[k * 384 + ee]));
        texp[ee] = tc_exponent(mx);
        const int nt = ee / kTcN, row = ee % kTcN;
        for (int k = 0; k < 162; ++k) {
            uint16_t o[kTcS];
            tc_slices(T[k * 384 + ee], texp[ee], o);
            for (int b = 0; b < kTcS; ++b)
                tsl[(size_t)(nt * kTcS + b) * (kTcBSlice / 2) + tc_off(row, k) / 2] = o[b];
        }
    }
}

// per device: the table, the constants, the kernel's shared-memory limit
TcTables& tc_tables() {
    static std::mutex mu;
    static std::vector<std::unique_ptr<TcTables>> per_dev;
    int dev = 0;
    FGB_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if ((int)per_dev.size() <= dev) per_dev.resize(dev + 1);
    if (!per_dev[dev]) {
        std::vector<uint16_t> tsl;
        std::vector<int> texp, corner;
        std::vector<double> d1, w;
        build_tc_tables(tsl, texp, d1, w, corner);
        auto t = std::make_unique<TcTables>();
        t->tsl.upload(tsl);
        t->texp.upload(texp);
        FGB_CUDA(cudaMemcpyToSymbol(c_tc_w, w.data(), sizeof(double) * w.size()));
        std::vector<float2> wdf(w.size());
        for (size_t q = 0; q < w.size(); ++q) {
            const float h = (float)w[q];
            wdf[q] = make_float2(h, (float)(w[q] - (double)h));
        }
        FGB_CUDA(cudaMemcpyToSymbol(c_tc_wdf, wdf.data(), sizeof(float2) * wdf.size()));
        FGB_CUDA(cudaMemcpyToSymbol(c_tc_corner, corner.data(), sizeof(int) * corner.size()));
        FGB_CUDA(cudaFuncSetAttribute(k_q2_ke_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
        FGB_CUDA(cudaDeviceSynchronize());
        per_dev[dev] = std::move(t);
    }
    return *per_dev[dev];
}
}  // namespace

void q2_cell_stiffness_tc(int nc, const int32_t* cd, const double* dxyz, double* ke, DBuf<unsigned char>& scratch,
                          DBuf<unsigned>& err, cudaStream_t s) {
    if (nc <= 0) return;
    TcTables& t = tc_tables();
    int dev = 0, sms = 0;
    FGB_CUDA(cudaGetDevice(&dev));
    FGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int tiles = (nc + kTcM - 1) / kTcM;
    const int grid = std::max(1, std::min(sms, tiles));
    const size_t need = (size_t)grid * kTcS * kTcASlice;
    if (scratch.size() < need) scratch.resize(need);
    if (err.size() != 1) err.resize(1);
    FGB_CUDA(cudaMemsetAsync(err.get(), 0, sizeof(unsigned), s));
    FGB_LAUNCH(k_q2_ke_tc<<<grid, kTcThreads, kTcSmem, s>>>(nc, cd, dxyz, ke, t.tsl.get(), t.texp.get(), scratch.get(),
                                                           err.get()));
    unsigned h = 0;
    FGB_CUDA(cudaMemcpyAsync(&h, err.get(), sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    FGB_CUDA(cudaStreamSynchronize(s));
    FGB_REQUIRE(h == 0, "tensor-core element matrices: a bounded wait ran out (code " + std::to_string(h) + ")");
}

double tc_selftest() {
    DBuf<float> d;
    d.resize(128 * 48);
    DBuf<unsigned> e;
    e.resize(1);
    FGB_CUDA(cudaMemset(d.get(), 0, sizeof(float) * 128 * 48));
    FGB_CUDA(cudaMemset(e.get(), 0, sizeof(unsigned)));
    FGB_LAUNCH(k_tc_selftest<<<1, 128>>>(d.get(), e.get()));
    FGB_CUDA(cudaDeviceSynchronize());
    std::vector<float> h(128 * 48);
    unsigned he = 0;
    FGB_CUDA(cudaMemcpy(h.data(), d.get(), sizeof(float) * h.size(), cudaMemcpyDeviceToHost));
    FGB_CUDA(cudaMemcpy(&he, e.get(), sizeof(unsigned), cudaMemcpyDeviceToHost));
    FGB_REQUIRE(he == 0, "tensor-core self test: the MMA completion wait ran out");
    double err = 0;
    for (int r = 0; r < 128; ++r)
        for (int c = 0; c < 48; ++c) {
            double s = 0;
            for (int k = 0; k < 32; ++k) s += (double)(((r * 3 + k * 5) % 7) - 3) * (double)(((c * 2 + k * 3) % 5) - 2);
            err = std::max(err, std::fabs(s - (double)h[r * 48 + c]));
        }
    return err;
}

}  // namespace fgb
