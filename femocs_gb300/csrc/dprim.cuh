// Device building blocks of the preparation kernels (mesh tables, FEM structure):
//   * SBuf: stream-ordered scratch (cudaMallocAsync / cudaFreeAsync);
//   * exclusive_scan: three-kernel prefix sum (tile sums, one-block scan of the sums, tiles);
//   * radix_sort: stable LSD radix sort of 32- or 64-bit keys with an optional int32 payload,
//     8-bit digits; per pass a per-tile digit histogram, a scan of the digit-major histogram,
//     and a scatter in which every tile ranks its keys in index order (warp match + per-warp
//     digit counts), so equal keys keep their input order.
// All work is on the caller's stream; nothing here synchronises except the *_total helpers
// that return a count to the host.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <utility>

#include "device.h"

namespace fgb {
namespace dprim {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;

template <typename T>
class SBuf {
public:
    SBuf() = default;
    SBuf(size_t n, cudaStream_t s) : s_(s), n_(n) {
        if (n) FGB_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&p_), n * sizeof(T), s));
    }
    ~SBuf() {
        if (p_) cudaFreeAsync(p_, s_);
    }
    SBuf(const SBuf&) = delete;
    SBuf& operator=(const SBuf&) = delete;
    SBuf(SBuf&& o) noexcept : p_(o.p_), s_(o.s_), n_(o.n_) { o.p_ = nullptr; o.n_ = 0; }
    SBuf& operator=(SBuf&& o) noexcept {
        if (this != &o) {
            if (p_) cudaFreeAsync(p_, s_);
            p_ = o.p_; s_ = o.s_; n_ = o.n_;
            o.p_ = nullptr; o.n_ = 0;
        }
        return *this;
    }
    T* get() const { return p_; }
    size_t size() const { return n_; }
    void fill_bytes(int byte) {
        if (n_) FGB_CUDA(cudaMemsetAsync(p_, byte, n_ * sizeof(T), s_));
    }
    void to_host(std::vector<T>& v, size_t n) const {
        v.resize(n);
        if (n) FGB_CUDA(cudaMemcpyAsync(v.data(), p_, n * sizeof(T), cudaMemcpyDeviceToHost, s_));
    }

private:
    T* p_ = nullptr;
    cudaStream_t s_ = 0;
    size_t n_ = 0;
};

// ------------------------------------------------------------------ scan
template <typename T, int NT>
__device__ __forceinline__ T block_exclusive_scan(T x, T& total) {
    __shared__ T wsum[NT / 32];
    __shared__ T tot;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const T w = lane < NT / 32 ? wsum[lane] : T(0);
        T wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        if (lane < NT / 32) wsum[lane] = wi - w;
        if (lane == NT / 32 - 1) tot = wi;
    }
    __syncthreads();
    const T r = wsum[warp] + inc - x;
    total = tot;
    __syncthreads();
    return r;
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_scan_tile_sums(const T* __restrict__ in, int64_t n, T* __restrict__ sums) {
    const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
    T s = 0;
#pragma unroll
    for (int j = 0; j < kItems; ++j)
        if (base + j < n) s += in[base + j];
    T total;
    block_exclusive_scan<T, kThreads>(s, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// one block: exclusive scan of n sums in place, grand total at sums[n]
template <typename T>
__global__ void __launch_bounds__(1024) k_scan_sums(T* sums, int64_t n) {
    const int64_t per = (n + 1023) / 1024;
    const int64_t b = threadIdx.x * per, e = b + per < n ? b + per : n;
    T s = 0;
    for (int64_t i = b; i < e; ++i) s += sums[i];
    T total;
    T run = block_exclusive_scan<T, 1024>(s, total);
    for (int64_t i = b; i < e; ++i) {
        const T v = sums[i];
        sums[i] = run;
        run += v;
    }
    if (threadIdx.x == 0) sums[n] = total;
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_scan_tile(const T* in, T* out, int64_t n, const T* __restrict__ sums) {
    const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
    T v[kItems];
    T s = 0;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        v[j] = base + j < n ? in[base + j] : T(0);
        s += v[j];
    }
    T total;
    T run = block_exclusive_scan<T, kThreads>(s, total) + sums[blockIdx.x];
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        if (base + j < n) out[base + j] = run;
        run += v[j];
    }
}

// out[i] = sum of in[0..i-1] (in == out allowed); the total is written to d_total when given
template <typename T>
void exclusive_scan(const T* in, T* out, int64_t n, T* d_total, cudaStream_t s) {
    const int64_t nblk = n > 0 ? (n + kTile - 1) / kTile : 0;
    SBuf<T> sums(nblk + 1, s);
    if (nblk) FGB_LAUNCH(k_scan_tile_sums<T><<<(unsigned)nblk, kThreads, 0, s>>>(in, n, sums.get()));
    FGB_LAUNCH(k_scan_sums<T><<<1, 1024, 0, s>>>(sums.get(), nblk));
    if (nblk) FGB_LAUNCH(k_scan_tile<T><<<(unsigned)nblk, kThreads, 0, s>>>(in, out, n, sums.get()));
    if (d_total) FGB_CUDA(cudaMemcpyAsync(d_total, sums.get() + nblk, sizeof(T), cudaMemcpyDeviceToDevice, s));
}

// exclusive scan whose total the host needs (synchronises the stream)
template <typename T>
T exclusive_scan_total(const T* in, T* out, int64_t n, cudaStream_t s) {
    SBuf<T> t(1, s);
    exclusive_scan(in, out, n, t.get(), s);
    T h = 0;
    FGB_CUDA(cudaMemcpyAsync(&h, t.get(), sizeof(T), cudaMemcpyDeviceToHost, s));
    FGB_CUDA(cudaStreamSynchronize(s));
    return h;
}

// ------------------------------------------------------------------ radix sort
__device__ __forceinline__ unsigned digit_of(uint32_t k, int shift) { return shift < 32 ? (k >> shift) & 255u : 0u; }
__device__ __forceinline__ unsigned digit_of(uint64_t k, int shift) { return (unsigned)(k >> shift) & 255u; }

template <typename K>
__global__ void __launch_bounds__(kThreads) k_radix_hist(const K* __restrict__ keys, int64_t n, int shift,
                                                         int* __restrict__ hist) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kTile;
#pragma unroll 4
    for (int j = 0; j < kItems; ++j) {
        const int64_t i = base + (int64_t)j * kThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[digit_of(keys[i], shift)], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// offs: exclusive scan of the digit-major histogram (digit d of tile b at d * n_tiles + b)
template <typename K>
__global__ void __launch_bounds__(kThreads) k_radix_scatter(const K* __restrict__ kin, const int32_t* __restrict__ vin,
                                                            K* __restrict__ kout, int32_t* __restrict__ vout, int64_t n,
                                                            int shift, const int* __restrict__ offs) {
    __shared__ int base[256];
    __shared__ int wcnt[kThreads / 32][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    base[tid] = offs[(int64_t)tid * gridDim.x + blockIdx.x];
    const int64_t tile0 = (int64_t)blockIdx.x * kTile;
    for (int j = 0; j < kItems; ++j) {
        const int64_t i = tile0 + (int64_t)j * kThreads + tid;
        const bool valid = i < n;
        K k = 0;
        int32_t v = 0;
        unsigned d = 256u + (unsigned)lane;  // invalid slots: a group of their own, never counted
        if (valid) {
            k = kin[i];
            if (vin) v = vin[i];
            d = digit_of(k, shift);
        }
        __syncthreads();  // the previous round's reads of wcnt are done
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w) wcnt[w][tid] = 0;
        __syncthreads();
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        {
            int run = base[tid];
#pragma unroll
            for (int w = 0; w < kThreads / 32; ++w) {
                const int c = wcnt[w][tid];
                wcnt[w][tid] = run;
                run += c;
            }
            base[tid] = run;
        }
        __syncthreads();
        if (valid) {
            const int pos = wcnt[warp][d] + rank;
            kout[pos] = k;
            if (vin) vout[pos] = v;
        }
    }
}

// Stable sort of keys[0..n) (and vals, if given) by their low `bits` bits. The sorted data
// ends in `keys` / `vals` (buffers are swapped with scratch as needed). n < 2^31.
template <typename K>
void radix_sort(SBuf<K>& keys, SBuf<int32_t>* vals, int64_t n, int bits, cudaStream_t s) {
    if (n <= 1 || bits <= 0) return;
    FGB_REQUIRE(n < (int64_t)INT32_MAX, "radix_sort: too many keys");
    const int64_t nblk = (n + kTile - 1) / kTile;
    SBuf<K> k2(n, s);
    SBuf<int32_t> v2(vals ? n : 0, s);
    SBuf<int> hist(256 * nblk, s);
    for (int shift = 0; shift < bits; shift += 8) {
        FGB_LAUNCH(k_radix_hist<K><<<(unsigned)nblk, kThreads, 0, s>>>(keys.get(), n, shift, hist.get()));
        exclusive_scan<int>(hist.get(), hist.get(), 256 * nblk, nullptr, s);
        FGB_LAUNCH(k_radix_scatter<K><<<(unsigned)nblk, kThreads, 0, s>>>(
            keys.get(), vals ? vals->get() : nullptr, k2.get(), vals ? v2.get() : nullptr, n, shift, hist.get()));
        std::swap(keys, k2);
        if (vals) std::swap(*vals, v2);
    }
}

inline int bits_for(uint64_t max_value) {
    int b = 1;
    while (b < 64 && (max_value >> b) != 0) ++b;
    return b;
}

}  // namespace dprim
}  // namespace fgb
