// Compensated FP64 residual b - A x of a SELL-32 row (4-wide chunks): the dot product in
// twice the working precision by the Dot2 algorithm of Ogita, Rump and Oishi ("Accurate sum
// and dot product", SIAM J. Sci. Comput. 26, 2005): every product split exactly with an FMA
// (TwoProduct), every addition exactly with Knuth's TwoSum, the errors summed separately and
// added once at the end. The result is as accurate as if computed in ~106-bit arithmetic and
// then rounded, so the FP64 rounding floor of b - A x (about 2^-53 |A||x|, which on the
// nanotip Laplacians is ~1e-12 of |b|) drops far below any tolerance a solver is asked for.
// All operations are explicit _rn intrinsics so the compiler cannot contract them.
#pragma once

#include <cstdint>

namespace fgb {

__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
    s = __dadd_rn(a, b);
    const double z = __dsub_rn(s, a);
    e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, z)), __dsub_rn(b, z));
}

// accumulate -a*x into (p, s) and |a*x| into mag
__device__ __forceinline__ void dot2_sub(double a, double x, double& p, double& s, double& mag) {
    const double h = __dmul_rn(-a, x);
    const double e = __fma_rn(-a, x, -h);
    double q;
    two_sum(p, h, p, q);
    s = __dadd_rn(s, __dadd_rn(q, e));
    mag = __dadd_rn(mag, fabs(h));
}

// b - (row r of A) x, A in SELL-32 with 4-wide chunks (columns and values of a row's chunk c
// at sptr[r/32] + (r%32)*4 + c*128), compensated; mag = |b| + sum |a x|, whose norm times
// 2^-53 is the rounding floor of a plain FP64 residual (and, since rounding the exact solution
// to FP64 leaves a residual of that size, the smallest residual an FP64 x can be held to)
__device__ __forceinline__ double sell_residual_dot2(int r, const int64_t* __restrict__ sptr,
                                                     const int32_t* __restrict__ slen, const int32_t* __restrict__ scol,
                                                     const double* __restrict__ sval, const double* __restrict__ x,
                                                     double b, double& mag) {
    const int s = r >> 5;
    const int64_t base = sptr[s] + (int64_t)(r & 31) * 4;
    const int nch = slen[s] >> 2;
    double p = b, err = 0.0;
    mag = fabs(b);
    for (int c = 0; c < nch; ++c) {
        const int64_t o = base + (int64_t)c * 128;
        const int4 ci = __ldg(reinterpret_cast<const int4*>(scol + o));
        const double2 v01 = __ldg(reinterpret_cast<const double2*>(sval + o));
        const double2 v23 = __ldg(reinterpret_cast<const double2*>(sval + o) + 1);
        dot2_sub(v01.x, __ldg(x + ci.x), p, err, mag);
        dot2_sub(v01.y, __ldg(x + ci.y), p, err, mag);
        dot2_sub(v23.x, __ldg(x + ci.z), p, err, mag);
        dot2_sub(v23.y, __ldg(x + ci.w), p, err, mag);
    }
    return __dadd_rn(p, err);
}

// squared rounding floor from the sum of squared row magnitudes: (2^-53)^2 * sum mag^2
constexpr double kFloorScale2 = 1.0 / 81129638414606681695789005144064.0;  // 2^-106

// a solve whose compensated true residual is within twice the floor has reached what FP64
// can hold: status kStatusFloor (a success) instead of iterating on rounding noise
constexpr int kStatusFloor = 2;

// the relative tolerance below which solvers evaluate their true residual compensated: at
// 1e-10 and above the plain FP64 residual's rounding floor (~1e-12 relative on these
// systems) is irrelevant and the cheaper product is used
constexpr double kCompensatedResidualBelow = 1e-10;

}  // namespace fgb
