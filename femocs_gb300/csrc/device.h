// Device memory and error helpers shared by the CUDA translation units.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <vector>

#include "common.h"

namespace fgb {

// Count of kernels this library has launched (reported by the benchmark).
extern std::atomic<long long> g_kernel_launches;
#define FGB_LAUNCH(...)                                                              \
    do {                                                                             \
        __VA_ARGS__;                                                                 \
        ::fgb::g_kernel_launches.fetch_add(1, std::memory_order_relaxed);           \
    } while (0)

#define FGB_CUDA(call)                                                                    \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            throw ::fgb::Error(std::string(__FILE__) + ":" + std::to_string(__LINE__) +  \
                               ": " #call " -> " + cudaGetErrorString(e_));               \
    } while (0)

// Host-to-device copy of pageable memory through pinned staging: chunks of the source are
// copied (by all host threads) into two pinned buffers in turn, each sent by an async DMA on
// `s` while the next is filled. Returns once the source may be reused; copies from several
// host threads take turns. Large copies from pageable memory otherwise run at a few GB/s.
void h2d_staged(void* dst, const void* src, size_t bytes, cudaStream_t s);
constexpr size_t kStagedMinBytes = size_t(8) << 20;
// the reverse: device to pageable host memory through the same double buffering; returns
// once the data are in `dst` (synchronous with the host, like a pageable copy)
void d2h_staged(void* dst, const void* src, size_t bytes, cudaStream_t s);

// Owning device buffer (cudaMalloc'd, freed on destruction).
template <typename T>
class DBuf {
public:
    DBuf() = default;
    explicit DBuf(size_t n) { resize(n); }
    ~DBuf() { release(); }
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr; o.n_ = 0; }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) { release(); p_ = o.p_; n_ = o.n_; o.p_ = nullptr; o.n_ = 0; }
        return *this;
    }
    void resize(size_t n) {
        if (n == n_) return;
        release();
        if (n) FGB_CUDA(cudaMalloc(&p_, n * sizeof(T)));
        n_ = n;
    }
    // enlarge to n elements keeping the first size() elements (new tail zeroed); stream-ordered
    void grow(size_t n, cudaStream_t s = 0) {
        if (n <= n_) return;
        T* q = nullptr;
        FGB_CUDA(cudaMalloc(&q, n * sizeof(T)));
        if (n_) FGB_CUDA(cudaMemcpyAsync(q, p_, n_ * sizeof(T), cudaMemcpyDeviceToDevice, s));
        FGB_CUDA(cudaMemsetAsync(q + n_, 0, (n - n_) * sizeof(T), s));
        FGB_CUDA(cudaStreamSynchronize(s));
        release();
        p_ = q;
        n_ = n;
    }
    void release() {
        if (p_) cudaFree(p_);
        p_ = nullptr;
        n_ = 0;
    }
    void upload(const T* h, size_t n, cudaStream_t s = 0) {
        resize(n);
        if (n * sizeof(T) >= kStagedMinBytes) h2d_staged(p_, h, n * sizeof(T), s);
        else if (n) FGB_CUDA(cudaMemcpyAsync(p_, h, n * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void upload(const std::vector<T>& v, cudaStream_t s = 0) { upload(v.data(), v.size(), s); }
    void download(T* h, size_t n, cudaStream_t s = 0) const {
        if (n * sizeof(T) >= kStagedMinBytes) d2h_staged(h, p_, n * sizeof(T), s);
        else if (n) FGB_CUDA(cudaMemcpyAsync(h, p_, n * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    std::vector<T> to_host(cudaStream_t s = 0) const {
        std::vector<T> v(n_);
        download(v.data(), n_, s);
        FGB_CUDA(cudaStreamSynchronize(s));
        return v;
    }
    void zero(cudaStream_t s = 0) {
        if (n_) FGB_CUDA(cudaMemsetAsync(p_, 0, n_ * sizeof(T), s));
    }
    T* get() { return p_; }
    const T* get() const { return p_; }
    size_t size() const { return n_; }
    size_t bytes() const { return n_ * sizeof(T); }

private:
    T* p_ = nullptr;
    size_t n_ = 0;
};

inline int grid_for(long long n, int block) { return (int)((n + block - 1) / block); }
// grid of a grid-stride kernel that ends in a grid-wide reduction: at most 2048 threads per SM,
// so that the last CTA's sum over the per-CTA partials stays a few steps long
inline int reduce_grid(long long n, int block) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms <= 0)
        sms = 152;
    const int cap = sms * (2048 / block);
    const int g = grid_for(n, block);
    return g < cap ? (g > 0 ? g : 1) : cap;
}

// Device time of one kernel inside a sequence of launches on one stream: an event pair is
// recorded around each timed launch while enabled; collect() sums the pairs after the
// stream has been synchronised. Events are pooled and reused across solves.
class LaunchTimer {
public:
    LaunchTimer() = default;
    LaunchTimer(const LaunchTimer&) = delete;
    LaunchTimer& operator=(const LaunchTimer&) = delete;
    ~LaunchTimer() {
        for (cudaEvent_t e : ev_) cudaEventDestroy(e);
    }
    bool enabled = false;
    // create the events of n launches ahead (event creation is a host call that would otherwise
    // fall inside the timed region)
    void reserve(int n) {
        while ((int)ev_.size() < 2 * n) {
            cudaEvent_t e;
            FGB_CUDA(cudaEventCreate(&e));
            ev_.push_back(e);
        }
    }
    void begin(cudaStream_t s) {
        if (enabled) FGB_CUDA(cudaEventRecord(next(), s));
    }
    void end(cudaStream_t s) {
        if (enabled) FGB_CUDA(cudaEventRecord(next(), s));
    }
    // sum of the recorded pairs [ms] and their count; resets the pool
    double collect(int* count) {
        double ms = 0;
        for (int k = 0; k + 1 < used_; k += 2) {
            float t = 0;
            FGB_CUDA(cudaEventElapsedTime(&t, ev_[k], ev_[k + 1]));
            ms += t;
        }
        if (count) *count = used_ / 2;
        used_ = 0;
        return ms;
    }

private:
    cudaEvent_t next() {
        if (used_ == (int)ev_.size()) {
            cudaEvent_t e;
            FGB_CUDA(cudaEventCreate(&e));
            ev_.push_back(e);
        }
        return ev_[used_++];
    }
    std::vector<cudaEvent_t> ev_;
    int used_ = 0;
};

}  // namespace fgb
