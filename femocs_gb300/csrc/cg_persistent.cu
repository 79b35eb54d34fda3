// Mixed-precision Jacobi-PCG as one persistent cooperative kernel (sm_103a).
//
// The whole solve is a single launch: every CTA stays resident, phases are separated by
// grid-wide barriers, and the scalars of the recurrence are reduced redundantly (and
// identically) by every CTA from per-CTA partial sums, so no host round trip and no kernel
// launch happens per iteration.
//
// Precision scheme (FP32 inner iterations inside FP64 refinement): the CG recurrence runs
// in FP32 on the FP32 copy of the matrix and accumulates the correction d in FP32; every
// time the recursive residual has dropped by `ru_factor` since the last refinement (and when
// it claims convergence), the correction is folded into the FP64 solution x and the
// residual is replaced by the true FP64 residual b - A x computed with the FP64 matrix
// ("reliable updates"). The search direction is kept across refinements, so the Krylov
// convergence of the FP64 iteration is preserved. Convergence is declared on the FP64 true
// residual only.
//
// One iteration = 2 grid barriers:
//   phase A: p = z + beta p_old (row owner, double-buffered), q = A p (gathering z and
//            p_old of the neighbours), partial p.q
//   phase B: d += alpha p, r -= alpha q, z = D^-1 r, partials r.z and r.r
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>

#include "compensated.cuh"
#include "fem_device.h"

namespace cg = cooperative_groups;

namespace fgb {


namespace {

constexpr int kThreads = 256;

// SELL-32 with 4-wide row chunks (layout in fem_setup.cpp). Matrix values and columns are
// read-only for the whole kernel (non-coherent loads); vectors written by other CTAs during
// the kernel are read with plain loads after the grid barrier.
__device__ __forceinline__ double sell_dot64(int i, const MixedArgs& a, const double* x) {
    const int s = i >> 5;
    const int64_t base = a.sptr[s] + (int64_t)(i & 31) * 4;
    const int nch = a.slen[s] >> 2;
    double acc0 = 0, acc1 = 0;
    for (int c = 0; c < nch; ++c) {
        const int64_t o = base + (int64_t)c * 128;
        const int4 ci = __ldg(reinterpret_cast<const int4*>(a.scol + o));
        const double2 v01 = __ldg(reinterpret_cast<const double2*>(a.s64 + o));
        const double2 v23 = __ldg(reinterpret_cast<const double2*>(a.s64 + o) + 1);
        acc0 += v01.x * x[ci.x] + v01.y * x[ci.y];
        acc1 += v23.x * x[ci.z] + v23.y * x[ci.w];
    }
    return acc0 + acc1;
}

// b_i - (A x)_i with the FP64 matrix, compensated when the tolerance nears the FP64 floor
// (mag: |b_i| + sum |a_ij x_j| of the compensated evaluation, 0 otherwise)
__device__ __forceinline__ double true_residual(int i, const MixedArgs& a, double& mag) {
    mag = 0.0;
    return a.comp ? sell_residual_dot2(i, a.sptr, a.slen, a.scol, a.s64, a.x, a.b[i], mag)
                  : a.b[i] - sell_dot64(i, a, a.x);
}

// q_i = sum_j a_ij (z_j + beta * pold_j): the new direction is formed on the fly
__device__ __forceinline__ float sell_dir_dot(int i, const MixedArgs& a, const float* z, const float* pold,
                                              float beta) {
    const int s = i >> 5;
    const int64_t base = a.sptr[s] + (int64_t)(i & 31) * 4;
    const int nch = a.slen[s] >> 2;
    float acc0 = 0.f, acc1 = 0.f;
    int c = 0;
    for (; c + 1 < nch; c += 2) {
        const int64_t o0 = base + (int64_t)c * 128, o1 = o0 + 128;
        const int4 i0 = __ldg(reinterpret_cast<const int4*>(a.scol + o0));
        const int4 i1 = __ldg(reinterpret_cast<const int4*>(a.scol + o1));
        const float4 v0 = __ldg(reinterpret_cast<const float4*>(a.s32 + o0));
        const float4 v1 = __ldg(reinterpret_cast<const float4*>(a.s32 + o1));
        acc0 += v0.x * (z[i0.x] + beta * pold[i0.x]) + v0.y * (z[i0.y] + beta * pold[i0.y]) +
                v0.z * (z[i0.z] + beta * pold[i0.z]) + v0.w * (z[i0.w] + beta * pold[i0.w]);
        acc1 += v1.x * (z[i1.x] + beta * pold[i1.x]) + v1.y * (z[i1.y] + beta * pold[i1.y]) +
                v1.z * (z[i1.z] + beta * pold[i1.z]) + v1.w * (z[i1.w] + beta * pold[i1.w]);
    }
    if (c < nch) {
        const int64_t o0 = base + (int64_t)c * 128;
        const int4 i0 = __ldg(reinterpret_cast<const int4*>(a.scol + o0));
        const float4 v0 = __ldg(reinterpret_cast<const float4*>(a.s32 + o0));
        acc0 += v0.x * (z[i0.x] + beta * pold[i0.x]) + v0.y * (z[i0.y] + beta * pold[i0.y]) +
                v0.z * (z[i0.z] + beta * pold[i0.z]) + v0.w * (z[i0.w] + beta * pold[i0.w]);
    }
    return acc0 + acc1;
}

// Grid-wide sum of NV values: per-CTA partials into buffer `buf`, barrier, then every CTA
// sums all partials in the same order (identical result in every CTA, deterministic).
template <int NV>
__device__ __forceinline__ void grid_sum(cg::grid_group& grid, double (&v)[NV], double* partial, int buf) {
    __shared__ double sh[NV][kThreads / 32];
    __shared__ double tot[NV];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double t = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) sh[k][wid] = t;
    }
    __syncthreads();
    static_assert(NV <= kMixedSumMax, "grid_sum buffers hold kMixedSumMax values per CTA");
    double* P = partial + (size_t)buf * kMixedSumMax * gridDim.x;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = 0.0;
            for (int w = 0; w < kThreads / 32; ++w) t += sh[k][w];
            P[(size_t)NV * blockIdx.x + k] = t;
        }
    }
    grid.sync();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = 0.0;
            for (int b = lane; b < (int)gridDim.x; b += 32) t += __ldcg(P + (size_t)NV * b + k);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            if (lane == 0) tot[k] = t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = tot[k];
    __syncthreads();
}

__global__ void __launch_bounds__(kThreads) k_mixed_cg(MixedArgs a) {
    cg::grid_group grid = cg::this_grid();
    const int G = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    int buf = 0;

    // ---- true residual of the initial guess, z = D^-1 r, d = 0, p_old = 0
    double v2[3] = {0.0, 0.0, 0.0};
    for (int i = t0; i < a.n; i += G) {
        double mag;
        const double ri = true_residual(i, a, mag);
        const float r32 = (float)ri;
        const float z32 = a.dinv32[i] * r32;
        a.r[i] = r32;
        a.z[i] = z32;
        a.d[i] = 0.f;
        a.pa[i] = 0.f;
        v2[0] += (double)r32 * (double)z32;
        v2[1] += ri * ri;
        v2[2] += mag * mag;
    }
    grid_sum<3>(grid, v2, a.partial, buf);
    buf ^= 1;
    double gamma = v2[0], rr = v2[1];
    double rr_ref = rr;  // residual at the last refinement
    int it = 0, updates = 0, status = 0, stalls = 0;
    float beta = 0.f;
    float* pold = a.pa;
    float* pnew = a.pb;
    if (rr <= a.tol2) status = 1;

    while (status == 0) {
        // ---- phase A
        double v1[1] = {0.0};
        for (int i = t0; i < a.n; i += G) {
            const float qi = sell_dir_dot(i, a, a.z, pold, beta);
            const float pi = a.z[i] + beta * pold[i];
            pnew[i] = pi;
            a.q[i] = qi;
            v1[0] += (double)pi * (double)qi;
        }
        grid_sum<1>(grid, v1, a.partial, buf);
        buf ^= 1;
        const float alpha = (float)(gamma / v1[0]);
        // ---- phase B
        double w2[2] = {0.0, 0.0};
        for (int i = t0; i < a.n; i += G) {
            a.d[i] += alpha * pnew[i];
            const float ri = a.r[i] - alpha * a.q[i];
            const float zi = a.dinv32[i] * ri;
            a.r[i] = ri;
            a.z[i] = zi;
            w2[0] += (double)ri * (double)zi;
            w2[1] += (double)ri * (double)ri;
        }
        grid_sum<2>(grid, w2, a.partial, buf);
        buf ^= 1;
        ++it;
        float* tmp = pold;
        pold = pnew;
        pnew = tmp;
        double gamma_new = w2[0];
        rr = w2[1];
        if (!(rr == rr) || !(gamma_new == gamma_new)) { status = -2; break; }
        if (rr <= a.tol2 || rr <= a.ru2 * rr_ref || it >= a.max_iter) {
            // ---- refinement: fold d into x (FP64), true residual with the FP64 matrix
            for (int i = t0; i < a.n; i += G) {
                a.x[i] += (double)a.d[i];
                a.d[i] = 0.f;
            }
            grid.sync();
            double u2[3] = {0.0, 0.0, 0.0};
            for (int i = t0; i < a.n; i += G) {
                double mag;
                const double ri = true_residual(i, a, mag);
                const float r32 = (float)ri;
                const float z32 = a.dinv32[i] * r32;
                a.r[i] = r32;
                a.z[i] = z32;
                u2[0] += (double)r32 * (double)z32;
                u2[1] += ri * ri;
                u2[2] += mag * mag;
            }
            grid_sum<3>(grid, u2, a.partial, buf);
            buf ^= 1;
            ++updates;
            gamma_new = u2[0];
            rr = u2[1];
            // a refinement that does not halve the true residual norm makes no progress;
            // four in a row end the solve (rounding floor reached) instead of running to max_iter
            stalls = rr > 0.25 * rr_ref ? stalls + 1 : 0;
            rr_ref = rr;
            if (rr <= a.tol2) { status = 1; break; }
            // compensated: within twice the FP64 floor is as converged as FP64 can hold x
            if (a.comp && rr <= 4.0 * kFloorScale2 * u2[2]) { status = kStatusFloor; break; }
            if (it >= a.max_iter) { status = -1; break; }
            if (!(rr == rr)) { status = -2; break; }
            if (stalls >= 4) { status = -3; break; }
        }
        beta = (float)(gamma_new / gamma);
        gamma = gamma_new;
    }
    if (t0 == 0) {
        a.out->iterations = it;
        a.out->updates = updates;
        a.out->status = status;
        a.out->rr = rr;
    }
}

}  // namespace

int mixed_cg_grid(int n) {
    static int cached = 0;
    if (!cached) {
        int dev = 0, sms = 0, per_sm = 0, coop = 0;
        FGB_CUDA(cudaGetDevice(&dev));
        FGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        FGB_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        FGB_REQUIRE(coop, "device does not support cooperative launches");
        FGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mixed_cg, kThreads, 0));
        FGB_REQUIRE(per_sm > 0, "persistent CG kernel cannot be resident");
        cached = sms * std::min(per_sm, 8);
    }
    // at least four rows per thread: fewer CTAs make the two grid barriers and the partial
    // sums of an iteration cheaper when the system is small
    const int want = (n + 4 * kThreads - 1) / (4 * kThreads);
    return std::max(1, std::min(cached, want));
}

void launch_mixed_cg(const MixedArgs& args, cudaStream_t stream) {
    const int grid = mixed_cg_grid(args.n);
    MixedArgs a = args;
    void* params[] = {&a};
    FGB_LAUNCH(FGB_CUDA(cudaLaunchCooperativeKernel((void*)k_mixed_cg, dim3(grid), dim3(kThreads), params, 0, stream)));
}

}  // namespace fgb
