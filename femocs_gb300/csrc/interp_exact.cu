// Point location, interpolation and nodal-field recovery (sm_103a).
//
// Compiled with -fmad=false: every double operation below is rounded on its own, in the
// order the reference evaluates it, so located cells are bit-identical to the reference's
// and interpolated values agree to the last bit except where a libm function (exp) differs.
//
// Location (reference: InterpolatorCells<4>::locate_cell, src/InterpolatorCells.cpp:269-307,
// driven sequentially by SolutionReader::calc_full_interpolation, src/SolutionReader.cpp:136-165):
// the reference checks the previous point's tet, then its neighbour list, then scans every
// tet of the searched region in index order, and finally returns minus the index of the
// tet with the nearest centroid. Its result for point i depends on point i-1 only when
// point i lies in no tet, in more than one tet, or only in tets outside the searched region.
//   k_locate_walk    per point: walk across faces to a tet containing it, then test that
//                    tet's vertex-sharing neighbourhood -> #containing tets, lowest
//                    containing searchable tet V
//   k_locate_scan    exhaustive scan for the rare points the walk could not place
//   k_nearest_ctr    exact nearest centroid (lowest index on ties) for points without V
//   k_resolve        guess-independent points get their final cell in parallel
//   k_chain_runs     each run of guess-dependent points replays the reference's chain
//                    from the last independent point (one warp per run, up to 32
//                    point-in-tet tests of the guess and its neighbours at once)
//   k_interpolate    shape functions of rank 1/2/3 and the weighted nodal solution
//   k_nodal_field, k_smooth: the nodal field and its smoothing; their geometry-only factors
//                    (k_nodal_coef, k_smooth_coef) are kept after a mesh's first
//                    extraction, so later solves only gather and sum (k_*_cached)
#include <climits>
#include <cmath>
#include <algorithm>
#include <deque>
#include <cstring>
#include <mutex>
#include <string>

#include "interp.h"

namespace fgb {

namespace {

constexpr double kZero = 1e-15;  // InterpolatorCells::zero, include/InterpolatorCells.h:241
constexpr int kWalkMax = 4096;

__device__ __forceinline__ double bary_dot(const double* d, int k, double x, double y, double z) {
    // Vec4(point,1).dotProduct(det_k)
    return x * d[1 + 4 * k] + y * d[2 + 4 * k] + z * d[3 + 4 * k] + 1.0 * d[4 + 4 * k];
}

__device__ __forceinline__ bool pic(const double* __restrict__ det, int t, double x, double y, double z) {
    const double* d = det + 17 * (size_t)t;
    const double d0 = d[0];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (d0 * bary_dot(d, k, x, y, z) < -kZero) return false;
    return true;
}

__device__ __forceinline__ void bcc4(const double* __restrict__ det, int t, double x, double y, double z, double* b) {
    const double* d = det + 17 * (size_t)t;
    const double d0 = d[0];
#pragma unroll
    for (int k = 0; k < 4; ++k) b[k] = kZero + d0 * bary_dot(d, k, x, y, z);
}

struct Pts {
    const double* p;
    __device__ __forceinline__ void get(int i, double& x, double& y, double& z) const {
        x = p[3 * (size_t)i];
        y = p[3 * (size_t)i + 1];
        z = p[3 * (size_t)i + 2];
    }
};

struct GridView {
    int dx, dy, dz;
    double ox, oy, oz, sx, sy, sz;
    __device__ __forceinline__ static int clampc(double v, int d) {
        v = floor(v);
        if (!(v >= 0.0)) return 0;  // also NaN
        return v >= (double)(d - 1) ? d - 1 : (int)v;
    }
    __device__ __forceinline__ void cell(double x, double y, double z, int& i, int& j, int& k) const {
        i = clampc((x - ox) / sx, dx);
        j = clampc((y - oy) / sy, dy);
        k = clampc((z - oz) / sz, dz);
    }
};

__global__ void k_locate_walk(int n, Pts P, GridView G, const int32_t* __restrict__ seed, const double* __restrict__ det,
                              const int32_t* __restrict__ fnb, const int32_t* __restrict__ nptr, const int32_t* __restrict__ nidx,
                              const int8_t* __restrict__ search, double lo0, double lo1, double lo2, double hi0, double hi1,
                              double hi2, int32_t* __restrict__ V, int32_t* __restrict__ nin, int32_t* __restrict__ counters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x, y, z;
    P.get(i, x, y, z);
    if (!(x >= lo0 && x <= hi0 && y >= lo1 && y <= hi1 && z >= lo2 && z <= hi2)) {
        // outside the mesh box (with margin): no tet can contain the point
        V[i] = -1;
        nin[i] = 0;
        return;
    }
    int gi, gj, gk;
    G.cell(x, y, z, gi, gj, gk);
    int t = seed[((size_t)gk * G.dy + gj) * G.dx + gi];
    int found = -1;
    for (int step = 0; step < kWalkMax; ++step) {
        const double* d = det + 17 * (size_t)t;
        const double d0 = d[0];
        double bmin = 0.0;
        int kmin = -1;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double b = d0 * bary_dot(d, k, x, y, z);
            if (b < -kZero && (kmin < 0 || b < bmin)) { bmin = b; kmin = k; }
        }
        if (kmin < 0) { found = t; break; }
        const int nx = fnb[4 * (size_t)t + kmin];
        if (nx < 0) break;
        t = nx;
    }
    if (found < 0) {
        V[i] = INT_MIN;  // needs the exhaustive scan
        nin[i] = 0;
        atomicAdd(&counters[0], 1);
        return;
    }
    int cnt = 1;
    int v = search[found] ? found : INT_MAX;
    for (int k = nptr[found]; k < nptr[found + 1]; ++k) {
        const int u = nidx[k];
        if (pic(det, u, x, y, z)) {
            ++cnt;
            if (search[u] && u < v) v = u;
        }
    }
    V[i] = v == INT_MAX ? -1 : v;
    nin[i] = cnt;
}

// one block per unplaced point (grid-stride over points), threads scan all tets
__global__ void k_locate_scan(int n, Pts P, int n_tets, const double* __restrict__ det, const int8_t* __restrict__ search,
                              int32_t* __restrict__ V, int32_t* __restrict__ nin) {
    __shared__ int s_cnt, s_v;
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        if (V[i] != INT_MIN) continue;
        double x, y, z;
        P.get(i, x, y, z);
        if (threadIdx.x == 0) { s_cnt = 0; s_v = INT_MAX; }
        __syncthreads();
        int cnt = 0, v = INT_MAX;
        for (int t = threadIdx.x; t < n_tets; t += blockDim.x)
            if (pic(det, t, x, y, z)) {
                ++cnt;
                if (search[t] && t < v) v = t;
            }
        atomicAdd(&s_cnt, cnt);
        atomicMin(&s_v, v);
        __syncthreads();
        if (threadIdx.x == 0) {
            V[i] = s_v == INT_MAX ? -1 : s_v;
            nin[i] = s_cnt;
        }
        __syncthreads();
    }
}

// exact argmin of the squared centroid distance over all tets, lowest index on ties
__global__ void k_nearest_ctr(int n, Pts P, GridView G, const int32_t* __restrict__ gptr, const int32_t* __restrict__ gtets,
                              const double* __restrict__ gc, const int32_t* __restrict__ V, int32_t* __restrict__ F,
                              int32_t* __restrict__ counters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (V[i] >= 0) { F[i] = -1; return; }
    atomicAdd(&counters[1], 1);
    double x, y, z;
    P.get(i, x, y, z);
    int ci, cj, ck;
    G.cell(x, y, z, ci, cj, ck);
    // like the reference's scan: best starts at 1e100 and the index at 0 (a point with no
    // finite distance, e.g. NaN coordinates, ends at tet 0)
    double best = 1e100;
    int bt = INT_MAX;
    const int rmax = max(G.dx, max(G.dy, G.dz));
    for (int r = 0; r <= rmax; ++r) {
        for (int k = ck - r; k <= ck + r; ++k) {
            if (k < 0 || k >= G.dz) continue;
            for (int j = cj - r; j <= cj + r; ++j) {
                if (j < 0 || j >= G.dy) continue;
                const bool face_kj = (k == ck - r || k == ck + r || j == cj - r || j == cj + r);
                for (int ii = ci - r; ii <= ci + r; ii += (face_kj ? 1 : 2 * r > 0 ? 2 * r : 1)) {
                    if (ii < 0 || ii >= G.dx) continue;
                    const size_t c = ((size_t)k * G.dy + j) * G.dx + ii;
                    for (int q = gptr[c]; q < gptr[c + 1]; ++q) {
                        const double ddx = x - gc[3 * (size_t)q];
                        const double ddy = y - gc[3 * (size_t)q + 1];
                        const double ddz = z - gc[3 * (size_t)q + 2];
                        const double d2 = ddx * ddx + ddy * ddy + ddz * ddz;
                        const int t = gtets[q];
                        if (d2 < best || (d2 == best && t < bt)) { best = d2; bt = t; }
                    }
                    if (r == 0) break;
                }
            }
        }
        if (bt != INT_MAX) {
            // distance from the point to the outside of the (2r+1)^3 block of visited cells
            double lb = 1e300;
            const double lo[3] = {G.ox + (ci - r) * G.sx, G.oy + (cj - r) * G.sy, G.oz + (ck - r) * G.sz};
            const double hi[3] = {G.ox + (ci + r + 1) * G.sx, G.oy + (cj + r + 1) * G.sy, G.oz + (ck + r + 1) * G.sz};
            const double pp[3] = {x, y, z};
            const int cc[3] = {ci, cj, ck};
            const int dd[3] = {G.dx, G.dy, G.dz};
            bool covers_all = true;
            for (int a = 0; a < 3; ++a) {
                if (cc[a] - r > 0) { lb = fmin(lb, pp[a] - lo[a]); covers_all = false; }
                if (cc[a] + r < dd[a] - 1) { lb = fmin(lb, hi[a] - pp[a]); covers_all = false; }
            }
            if (covers_all) break;
            if (lb > 0 && lb * lb * (1.0 - 1e-9) > best) break;
        }
    }
    F[i] = bt == INT_MAX ? 0 : bt;
}

__global__ void k_resolve(int n, const int32_t* __restrict__ V, const int32_t* __restrict__ nin, const int32_t* __restrict__ F,
                          int32_t* __restrict__ res, int32_t* __restrict__ dep, int32_t* __restrict__ counters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool indep = nin[i] == 0 || (nin[i] == 1 && V[i] >= 0);
    dep[i] = indep ? 0 : 1;
    if (indep) res[i] = V[i] >= 0 ? V[i] : -F[i];
    else atomicAdd(&counters[2], 1);
}

// Runs of guess-dependent points replay the reference's chained search from the last
// independent point (the guess, then the tets sharing its nodes in list order, then the scan
// result), one warp per run: for each point lane 0 tests the guess and lanes 1..31 the guess's
// neighbours in list order (further neighbours 31 at a time); the lowest lane whose tet
// contains the point is the reference's first hit, so the result is that of the sequential
// search, with up to 32 point-in-tet tests in flight instead of one
__global__ void k_chain_runs(int n, Pts P, int g0, const double* __restrict__ det, const int32_t* __restrict__ nptr,
                                  const int32_t* __restrict__ nidx, const int32_t* __restrict__ V,
                                  const int32_t* __restrict__ F, const int32_t* __restrict__ dep, int32_t* __restrict__ res,
                                  int32_t* __restrict__ counters) {
    const long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wid >= n) return;  // whole warp leaves together
    const int i = (int)wid;
    if (!dep[i] || (i > 0 && dep[i - 1])) return;
    int g = i == 0 ? g0 : abs(res[i - 1]);
    int j = i;
    for (; j < n && dep[j]; ++j) {
        double x, y, z;
        P.get(j, x, y, z);
        const int k0 = nptr[g], k1 = nptr[g + 1];
        int r = INT_MIN;
        // chunk 0: the guess (lane 0) and the first 31 neighbours; then 31 more per chunk
        for (int base = k0 - 1; base < k1; base += 31) {
            const int k = base + lane;  // lane 0 of chunk 0 is the guess itself
            int cand = -1;
            if (lane == 0) cand = base == k0 - 1 ? g : -1;
            else if (k < k1) cand = nidx[k];
            const bool hit = cand >= 0 && pic(det, cand, x, y, z);
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (m) {
                r = __shfl_sync(0xffffffffu, cand, __ffs(m) - 1);
                break;
            }
        }
        if (r == INT_MIN) r = V[j] >= 0 ? V[j] : -F[j];
        if (lane == 0) res[j] = r;
        g = abs(r);
    }
    if (lane == 0) atomicMax(&counters[3], j - i);
}

// ---------------------------------------------------------------- surface triangles
// LinearTriangles::point_in_cell (src/InterpolatorCells.cpp:1639-1650) on the 19-double rows
// of SurfaceTables::geo: vert0, edge1/D, edge2, pvec/D, normal, |edge2|, centroid
__device__ __forceinline__ bool tri_pic(const double* __restrict__ geo, int f, double x, double y, double z) {
    const double* g = geo + 19 * (size_t)f;
    const double tx = x - g[0], ty = y - g[1], tz = z - g[2];
    const double u = tx * g[9] + ty * g[10] + tz * g[11];
    if (u < -kZero || u > 1 + kZero) return false;
    const double qx = ty * g[5] - tz * g[4], qy = tz * g[3] - tx * g[5], qz = tx * g[4] - ty * g[3];
    const double v = qx * g[12] + qy * g[13] + qz * g[14];
    if (v < -kZero || u + v > 1 + kZero) return false;
    return fabs(qx * g[6] + qy * g[7] + qz * g[8]) < g[15];
}

// LinearTriangles::fast_distance, :1743-1747
__device__ __forceinline__ double tri_fast_distance(const double* __restrict__ geo, int f, double x, double y, double z) {
    const double* g = geo + 19 * (size_t)f;
    const double tx = x - g[0], ty = y - g[1], tz = z - g[2];
    const double qx = ty * g[5] - tz * g[4], qy = tz * g[3] - tx * g[5], qz = tx * g[4] - ty * g[3];
    return g[6] * qx + g[7] * qy + g[8] * qz;
}

// per point: the triangles whose acceptance region meets the point's candidate cell ->
// #containing triangles and the lowest containing one (the result of the reference's scan)
__global__ void k_tri_locate(int n, Pts P, GridView C, double lo0, double lo1, double lo2, double hi0, double hi1,
                             double hi2, const int32_t* __restrict__ cptr, const int32_t* __restrict__ cidx,
                             const double* __restrict__ geo, int32_t* __restrict__ V, int32_t* __restrict__ nin) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x, y, z;
    P.get(i, x, y, z);
    if (!(x >= lo0 && x <= hi0 && y >= lo1 && y <= hi1 && z >= lo2 && z <= hi2)) {
        V[i] = -1;
        nin[i] = 0;
        return;
    }
    int ci, cj, ck;
    C.cell(x, y, z, ci, cj, ck);
    const size_t c = ((size_t)ck * C.dy + cj) * C.dx + ci;
    int cnt = 0, v = INT_MAX;
    for (int q = cptr[c]; q < cptr[c + 1]; ++q) {
        const int f = cidx[q];
        if (tri_pic(geo, f, x, y, z)) {
            ++cnt;
            if (f < v) v = f;
        }
    }
    V[i] = cnt ? v : -1;
    nin[i] = cnt;
}

// runs of guess-dependent points replay the chained triangle search from the last
// independent point: guess, the triangles sharing its nodes, then the scan result
__global__ void k_tri_chain_runs(int n, Pts P, int g0, int n_tris, const double* __restrict__ geo,
                                 const int32_t* __restrict__ nptr, const int32_t* __restrict__ nidx,
                                 const int32_t* __restrict__ V, const int32_t* __restrict__ F,
                                 const int32_t* __restrict__ dep, int32_t* __restrict__ res, int32_t* __restrict__ counters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!dep[i] || (i > 0 && dep[i - 1])) return;
    int g = i == 0 ? g0 : abs(res[i - 1]);
    int j = i;
    for (; j < n && dep[j]; ++j) {
        double x, y, z;
        P.get(j, x, y, z);
        int r = INT_MIN;
        if (g < n_tris) {
            if (tri_pic(geo, g, x, y, z)) {
                r = g;
            } else {
                for (int k = nptr[g]; k < nptr[g + 1]; ++k) {
                    const int u = nidx[k];
                    if (tri_pic(geo, u, x, y, z)) { r = u; break; }
                }
            }
        }
        if (r == INT_MIN) r = V[j] >= 0 ? V[j] : -F[j];
        res[j] = r;
        g = abs(r);
    }
    atomicMax(&counters[3], j - i);
}

// the tet of each located point: the triangle's first tet if the point lies on the triangle
// or inside that tet, otherwise the chained tet search from the second tet
__global__ void k_surface_tet(int n, Pts P, const int32_t* __restrict__ tres, const int32_t* __restrict__ t2t,
                              const double* __restrict__ geo, const double* __restrict__ det,
                              const int32_t* __restrict__ nptr, const int32_t* __restrict__ nidx,
                              const int32_t* __restrict__ V, const int32_t* __restrict__ F, int32_t* __restrict__ tcell) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x, y, z;
    P.get(i, x, y, z);
    const int tri = abs(tres[i]);
    const int t0 = t2t[2 * (size_t)tri], t1 = t2t[2 * (size_t)tri + 1];
    int tet;
    if (fabs(tri_fast_distance(geo, tri, x, y, z)) <= 100.0 * kZero || pic(det, t0, x, y, z)) {
        tet = t0;
    } else if (pic(det, t1, x, y, z)) {
        tet = t1;
    } else {
        tet = INT_MIN;
        for (int k = nptr[t1]; k < nptr[t1 + 1]; ++k) {
            const int u = nidx[k];
            if (pic(det, u, x, y, z)) { tet = u; break; }
        }
        if (tet == INT_MIN) tet = V[i] >= 0 ? V[i] : -F[i];
    }
    tcell[i] = tet;
}

// rank 3 (LinearQuadrangles::locate_cell + interp_solution, src/InterpolatorCells.cpp:1922-1993):
// quadrangle = 3 * triangle + the vertex with the largest barycentric coordinate (sign of the
// triangle result), then the hexes of the triangle's two tets around that vertex: the first if
// the point lies on the triangle or in that hex, else LinearHexahedra::locate_cell from the
// second (tet search from its tet, hex by the largest barycentric coordinate)
__global__ void k_surface_hex(int n, Pts P, const int32_t* __restrict__ tres, const int32_t* __restrict__ tris,
                              const int32_t* __restrict__ t2t, const double* __restrict__ geo,
                              const double* __restrict__ det, const int32_t* __restrict__ tets,
                              const int32_t* __restrict__ nptr, const int32_t* __restrict__ nidx,
                              const int32_t* __restrict__ V, const int32_t* __restrict__ F, int32_t* __restrict__ quad_out,
                              int32_t* __restrict__ hex_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x, y, z;
    P.get(i, x, y, z);
    const int tr = tres[i];
    const int tf = abs(tr);
    {
        // LinearTriangles::shape_functions (:1652-1660)
        const double* g = geo + 19 * (size_t)tf;
        const double tx = x - g[0], ty = y - g[1], tz = z - g[2];
        const double qx = ty * g[5] - tz * g[4], qy = tz * g[3] - tx * g[5], qz = tx * g[4] - ty * g[3];
        const double v = tx * g[9] + ty * g[10] + tz * g[11];
        const double w = qx * g[12] + qy * g[13] + qz * g[14];
        const double u = 1.0 - v - w;
        const double b0 = kZero + u, b1 = kZero + v, b2 = kZero + w;
        int k = -1;
        if (b0 >= b1 && b0 >= b2) k = 0;
        else if (b1 >= b0 && b1 >= b2) k = 1;
        else if (b2 >= b0 && b2 >= b1) k = 2;
        quad_out[i] = k < 0 ? -1 : (tr < 0 ? -1 : 1) * (3 * tf + k);
    }
    const int q = abs(quad_out[i]), tq = q / 3;
    const int vert = tris[3 * (size_t)tq + q % 3];
    int hx[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int t = t2t[2 * (size_t)tq + r];
        int loc = 0;
        while (loc < 4 && tets[4 * (size_t)t + loc] != vert) ++loc;
        hx[r] = 4 * t + (loc < 4 ? loc : 0);
    }
    int hex;
    bool in0 = fabs(tri_fast_distance(geo, tq, x, y, z)) <= 100.0 * kZero;
    if (!in0) {
        // LinearHexahedra::point_in_cell (:1507-1528)
        double b[4];
        bcc4(det, hx[0] / 4, x, y, z, b);
        if (b[0] >= 0 && b[1] >= 0 && b[2] >= 0 && b[3] >= 0) {
            const int s = hx[0] % 4;
            in0 = true;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (j != s && !(b[s] >= b[j])) in0 = false;
        }
    }
    if (in0) {
        hex = hx[0];
    } else {
        const int t1 = hx[1] / 4;
        int tet;
        if (pic(det, t1, x, y, z)) {
            tet = t1;
        } else {
            tet = INT_MIN;
            for (int k = nptr[t1]; k < nptr[t1 + 1]; ++k) {
                const int u = nidx[k];
                if (pic(det, u, x, y, z)) { tet = u; break; }
            }
            if (tet == INT_MIN) tet = V[i] >= 0 ? V[i] : -F[i];
        }
        const int sign = tet < 0 ? -1 : 1;
        const int t = abs(tet);
        double b[4];
        bcc4(det, t, x, y, z, b);
        hex = -1;
        if (b[0] >= b[1] && b[0] >= b[2] && b[0] >= b[3]) hex = sign * (4 * t + 0);
        else if (b[1] >= b[0] && b[1] >= b[2] && b[1] >= b[3]) hex = sign * (4 * t + 1);
        else if (b[2] >= b[0] && b[2] >= b[1] && b[2] >= b[3]) hex = sign * (4 * t + 2);
        else if (b[3] >= b[0] && b[3] >= b[1] && b[3] >= b[2]) hex = sign * (4 * t + 3);
    }
    hex_out[i] = hex;
}

__device__ __forceinline__ void acc5(const double* __restrict__ sol, int node, double w, double* a) {
    const double* s = sol + 5 * (size_t)node;
#pragma unroll
    for (int c = 0; c < 5; ++c) a[c] += s[c] * w;
}

// LinearHexahedra::project_to_nat_coords (src/InterpolatorCells.cpp:1272-1317): Newton on the
// trilinear map x = f0 + f1 u + f2 v + f3 w + f4 uv + f5 uw + f6 vw + f7 uvw, Cramer steps,
// at most 20 iterations, stop when |du|^2 < 1e-15
__device__ __forceinline__ void hex_natural(const double* __restrict__ F, double x, double y, double z, double& u,
                                            double& v, double& ww) {
    const double f0x = x - F[0], f0y = y - F[1], f0z = z - F[2];
    u = 0;
    v = 0;
    ww = 0;
    for (int it = 0; it < 20; ++it) {
        const double uv = u * v, uw = u * ww, vw = v * ww, uvw = uv * ww;
        double f[3], fu[3], fv[3], fw[3];
        const double f0[3] = {f0x, f0y, f0z};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            f[q] = f0[q] - F[3 + q] * u - F[6 + q] * v - F[9 + q] * ww - F[12 + q] * uv - F[15 + q] * uw -
                   F[18 + q] * vw - F[21 + q] * uvw;
            fu[q] = F[3 + q] + F[12 + q] * v + F[15 + q] * ww + F[21 + q] * vw;
            fv[q] = F[6 + q] + F[12 + q] * u + F[18 + q] * ww + F[21 + q] * uw;
            fw[q] = F[9 + q] + F[15 + q] * u + F[18 + q] * v + F[21 + q] * uv;
        }
        // determinant(v1,v2,v3) of the reference, rows = vectors
        auto det3 = [](const double* p, const double* q, const double* r) {
            return p[0] * (q[1] * r[2] - r[1] * q[2]) - q[0] * (p[1] * r[2] - r[1] * p[2]) +
                   r[0] * (p[1] * q[2] - q[1] * p[2]);
        };
        const double D = 1.0 / det3(fu, fv, fw);
        const double du = det3(f, fv, fw) * D, dv = det3(fu, f, fw) * D, dw = det3(fu, fv, f) * D;
        u += du;
        v += dv;
        ww += dw;
        if (du * du + dv * dv + dw * dw < kZero) break;
    }
}

// PoissonSolver::assemble_space_charge_fast (src/PoissonSolver.cpp:300-319): every particle
// adds N_k(p) q/eps0 W_sp to the rhs of its hex's nodes, N = the trilinear shape functions
// at the particle (shape_funs_dealii: the same values in deal.II's vertex order). order 2:
// the 27 Q2 Lagrange functions of the same natural coordinates on the hex's Q2 DoFs. The sum
// over particles uses FP64 atomics (order-dependent rounding at the last bit).
__global__ void k_space_charge(int n, Pts P, const int32_t* __restrict__ hex_of, const double* __restrict__ hexf,
                               const int32_t* __restrict__ hexs, const int32_t* __restrict__ node2dof, int order,
                               const int32_t* __restrict__ hex2cell, const int32_t* __restrict__ cell_dofs, double cf,
                               double* __restrict__ rhs, int32_t* __restrict__ counters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int h = hex_of[i];
    if (h < 0) {  // not inside a vacuum hex: contributes nothing
        atomicAdd(&counters[0], 1);
        return;
    }
    double x, y, z;
    P.get(i, x, y, z);
    double u, v, ww;
    hex_natural(hexf + 24 * (size_t)h, x, y, z, u, v, ww);
    if (order == 1) {
        const double w8[8] = {(1 - u) * (1 - v) * (1 - ww) / 8.0, (1 + u) * (1 - v) * (1 - ww) / 8.0,
                              (1 + u) * (1 + v) * (1 - ww) / 8.0, (1 - u) * (1 + v) * (1 - ww) / 8.0,
                              (1 - u) * (1 - v) * (1 + ww) / 8.0, (1 + u) * (1 - v) * (1 + ww) / 8.0,
                              (1 + u) * (1 + v) * (1 + ww) / 8.0, (1 - u) * (1 + v) * (1 + ww) / 8.0};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int d = node2dof[hexs[8 * (size_t)h + k]];
            if (d >= 0) atomicAdd(&rhs[d], w8[k] * cf);
        }
    } else {
        const int c = hex2cell[h];
        if (c < 0) {
            atomicAdd(&counters[0], 1);
            return;
        }
        const double t[3] = {u, v, ww};
        double l[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            l[a][0] = 0.5 * t[a] * (t[a] - 1.0);
            l[a][1] = 1.0 - t[a] * t[a];
            l[a][2] = 0.5 * t[a] * (t[a] + 1.0);
        }
        for (int L = 0; L < 27; ++L)
            atomicAdd(&rhs[cell_dofs[27 * (size_t)c + L]], l[0][L % 3] * l[1][(L / 3) % 3] * l[2][L / 9] * cf);
    }
}

__global__ void k_interpolate(int n, Pts P, int rank, int from_tets, const int32_t* __restrict__ cells_in,
                              const double* __restrict__ det, const int32_t* __restrict__ tets, const int32_t* __restrict__ quad,
                              const int32_t* __restrict__ hexs, const double* __restrict__ hexf, const double* __restrict__ sol,
                              int32_t* __restrict__ cells_out, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x, y, z;
    P.get(i, x, y, z);
    int cell = cells_in[i];
    if (rank == 3 && from_tets) {
        // LinearHexahedra::locate_cell, src/InterpolatorCells.cpp:1536-1562
        const int sign = cell < 0 ? -1 : 1;
        const int t = abs(cell);
        double b[4];
        bcc4(det, t, x, y, z, b);
        int h = -1;
        if (b[0] >= b[1] && b[0] >= b[2] && b[0] >= b[3]) h = sign * (4 * t + 0);
        else if (b[1] >= b[0] && b[1] >= b[2] && b[1] >= b[3]) h = sign * (4 * t + 1);
        else if (b[2] >= b[0] && b[2] >= b[1] && b[2] >= b[3]) h = sign * (4 * t + 2);
        else if (b[3] >= b[0] && b[3] >= b[1] && b[3] >= b[2]) h = sign * (4 * t + 3);
        cell = h;
    }
    if (cells_out) cells_out[i] = cell;
    const int c = abs(cell);
    double a[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (rank == 1) {
        double b[4];
        bcc4(det, c, x, y, z, b);
        const int32_t* nd = tets + 4 * (size_t)c;
#pragma unroll
        for (int k = 0; k < 4; ++k) acc5(sol, nd[k], b[k], a);
    } else if (rank == 2) {
        double b[4];
        bcc4(det, c, x, y, z, b);
        const double w[10] = {b[0] * (2 * b[0] - 1), b[1] * (2 * b[1] - 1), b[2] * (2 * b[2] - 1), b[3] * (2 * b[3] - 1),
                              4 * b[0] * b[1], 4 * b[1] * b[2], 4 * b[2] * b[0], 4 * b[0] * b[3], 4 * b[1] * b[3],
                              4 * b[2] * b[3]};
        const int32_t* nd = quad + 10 * (size_t)c;
#pragma unroll
        for (int k = 0; k < 10; ++k) acc5(sol, nd[k], w[k], a);
    } else {
        // LinearHexahedra::project_to_nat_coords + shape_functions, :1272-1353
        double u, v, ww;
        hex_natural(hexf + 24 * (size_t)c, x, y, z, u, v, ww);
        const double w8[8] = {(1 - u) * (1 - v) * (1 - ww) / 8.0, (1 + u) * (1 - v) * (1 - ww) / 8.0,
                              (1 + u) * (1 + v) * (1 - ww) / 8.0, (1 - u) * (1 + v) * (1 - ww) / 8.0,
                              (1 - u) * (1 - v) * (1 + ww) / 8.0, (1 + u) * (1 - v) * (1 + ww) / 8.0,
                              (1 + u) * (1 + v) * (1 + ww) / 8.0, (1 - u) * (1 + v) * (1 + ww) / 8.0};
        const int32_t* nd = hexs + 8 * (size_t)c;
#pragma unroll
        for (int k = 0; k < 8; ++k) acc5(sol, nd[k], w8[k], a);
    }
    double* o = out + 5 * (size_t)i;
#pragma unroll
    for (int q = 0; q < 5; ++q) o[q] = a[q];
}

// ---------------------------------------------------------------- nodal solution
__global__ void k_scatter_solution(int n_dofs, const double* __restrict__ phi, const double* __restrict__ charge,
                                   const int32_t* __restrict__ dof2node, double* __restrict__ sol) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n_dofs || dof2node[d] < 0) return;  // Q2 edge/face/interior DoFs have no mesh node
    double* s = sol + 5 * (size_t)dof2node[d];
    s[0] = 0.0;
    s[1] = 0.0;
    s[2] = 0.0;
    s[3] = charge ? charge[d] : 0.0;
    s[4] = phi[d];
}

// local-node tables of LinearHexahedra::project_to_nat_coords(u,v,w,n1,n2,n3,node), :1319-1331
__constant__ int8_t c_uvw[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                   {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
__constant__ int8_t c_nnn[8][3] = {{1, 3, 4}, {0, 2, 5}, {3, 1, 6}, {2, 0, 7}, {5, 7, 0}, {4, 6, 1}, {7, 5, 2}, {6, 4, 3}};

// Interpolator::store_elfield (src/Interpolator.cpp:125-140) with
// LinearHexahedra::shape_fun_grads(hex, node) (:1462-1505) and interp_gradient(cell,node) (:425-439)
__global__ void k_nodal_field(int n_nodes, const int32_t* __restrict__ n2c_ptr, const int32_t* __restrict__ n2c_item,
                              const int32_t* __restrict__ hexs, const double* __restrict__ xyz, double* __restrict__ sol) {
    const int node_id = blockIdx.x * blockDim.x + threadIdx.x;
    if (node_id >= n_nodes) return;
    const int b = n2c_ptr[node_id], e = n2c_ptr[node_id + 1];
    if (b == e) return;
    double mx = 0.0, my = 0.0, mz = 0.0;
    for (int p = b; p < e; ++p) {
        const int hex = n2c_item[p] >> 3, node = n2c_item[p] & 7;
        const int32_t* hx = hexs + 8 * (size_t)hex;
        const double uvw[3] = {(double)c_uvw[node][0], (double)c_uvw[node][1], (double)c_uvw[node][2]};
        const int nn[3] = {c_nnn[node][0], c_nnn[node][1], c_nnn[node][2]};
        const double* v0 = xyz + 3 * (size_t)hx[node];
        double J[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const double* vi = xyz + 3 * (size_t)hx[nn[i]];
            const double f = uvw[i] * 0.5;
            J[i][0] = (v0[0] - vi[0]) * f;
            J[i][1] = (v0[1] - vi[1]) * f;
            J[i][2] = (v0[2] - vi[2]) * f;
        }
        double Jdet = J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) - J[1][0] * (J[0][1] * J[2][2] - J[2][1] * J[0][2]) +
                      J[2][0] * (J[0][1] * J[1][2] - J[1][1] * J[0][2]);
        Jdet = 1.0 / Jdet;
        double Ji[3][3] = {
            {J[1][1] * J[2][2] - J[2][1] * J[1][2], J[2][1] * J[0][2] - J[0][1] * J[2][2], J[0][1] * J[1][2] - J[1][1] * J[0][2]},
            {J[2][0] * J[1][2] - J[1][0] * J[2][2], J[0][0] * J[2][2] - J[2][0] * J[0][2], J[1][0] * J[0][2] - J[0][0] * J[1][2]},
            {J[1][0] * J[2][1] - J[2][0] * J[1][1], J[2][0] * J[0][1] - J[0][0] * J[2][1], J[0][0] * J[1][1] - J[1][0] * J[0][1]}};
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) Ji[i][j] *= Jdet;
        // nonzero shape-function gradients: the node itself and its three edge neighbours
        double gs[3], gn[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            gs[i] = 0.5 * (Ji[i][0] * uvw[0] + Ji[i][1] * uvw[1] + Ji[i][2] * uvw[2]);
#pragma unroll
            for (int j = 0; j < 3; ++j) gn[j][i] = -0.5 * Ji[i][j] * uvw[j];
        }
        // E -= sfg[k] * phi[k] for k = 0..7 in order (zero terms do not change the sum)
        double ex = 0.0, ey = 0.0, ez = 0.0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            double sx, sy, sz;
            if (k == node) { sx = gs[0]; sy = gs[1]; sz = gs[2]; }
            else if (k == nn[0]) { sx = gn[0][0]; sy = gn[0][1]; sz = gn[0][2]; }
            else if (k == nn[1]) { sx = gn[1][0]; sy = gn[1][1]; sz = gn[1][2]; }
            else if (k == nn[2]) { sx = gn[2][0]; sy = gn[2][1]; sz = gn[2][2]; }
            else continue;
            const double ph = sol[5 * (size_t)hx[k] + 4];
            ex -= sx * ph;
            ey -= sy * ph;
            ez -= sz * ph;
        }
        mx += ex;
        my += ey;
        mz += ez;
    }
    const double f = 1.0 / (e - b);
    double* s = sol + 5 * (size_t)node_id;
    s[0] = mx * f;
    s[1] = my * f;
    s[2] = mz * f;
}

// Interpolator::average_nodal_fields (src/Interpolator.cpp:142-170). Tet vertices are
// overwritten from their pseudo-Voronoi neighbours, which are never tet vertices, so the
// in-place sequential loop of the reference is order independent.
__global__ void k_smooth(int n_tn, const int32_t* __restrict__ vptr, const int32_t* __restrict__ vidx,
                         const double* __restrict__ xyz, double decay, double* __restrict__ sol) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_tn) return;
    const int b = vptr[i], e = vptr[i + 1];
    if (b == e) return;
    const double px = xyz[3 * (size_t)i], py = xyz[3 * (size_t)i + 1], pz = xyz[3 * (size_t)i + 2];
    double vx = 0, vy = 0, vz = 0, ws = 0;
    for (int k = b; k < e; ++k) {
        const int nb = vidx[k];
        const double dx = px - xyz[3 * (size_t)nb], dy = py - xyz[3 * (size_t)nb + 1], dz = pz - xyz[3 * (size_t)nb + 2];
        const double w = exp(decay * sqrt(dx * dx + dy * dy + dz * dz));
        ws += w;
        vx += sol[5 * (size_t)nb] * w;
        vy += sol[5 * (size_t)nb + 1] * w;
        vz += sol[5 * (size_t)nb + 2] * w;
    }
    if (ws > 0) {
        const double f = 1.0 / ws;
        sol[5 * (size_t)i] = vx * f;
        sol[5 * (size_t)i + 1] = vy * f;
        sol[5 * (size_t)i + 2] = vz * f;
    }
}

// The geometry-only parts of k_nodal_field and k_smooth, evaluated once per mesh with the same
// expressions (so the same FP64 values), and the per-solve kernels that use them: the same
// sums in the same order, hence bit-identical results.
//
// k_nodal_coef: per (node, hex) item p of n2c, the four nonzero shape-function gradients of
// the hex at that node in ascending local-node order: node ids ids[4p + j] and gradients
// coef[12p + 3j + c]
__global__ void k_nodal_coef(int n_items, const int32_t* __restrict__ n2c_item, const int32_t* __restrict__ hexs,
                             const double* __restrict__ xyz, int32_t* __restrict__ ids, double* __restrict__ coef) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_items) return;
    const int hex = n2c_item[p] >> 3, node = n2c_item[p] & 7;
    const int32_t* hx = hexs + 8 * (size_t)hex;
    const double uvw[3] = {(double)c_uvw[node][0], (double)c_uvw[node][1], (double)c_uvw[node][2]};
    const int nn[3] = {c_nnn[node][0], c_nnn[node][1], c_nnn[node][2]};
    const double* v0 = xyz + 3 * (size_t)hx[node];
    double J[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double* vi = xyz + 3 * (size_t)hx[nn[i]];
        const double f = uvw[i] * 0.5;
        J[i][0] = (v0[0] - vi[0]) * f;
        J[i][1] = (v0[1] - vi[1]) * f;
        J[i][2] = (v0[2] - vi[2]) * f;
    }
    double Jdet = J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) - J[1][0] * (J[0][1] * J[2][2] - J[2][1] * J[0][2]) +
                  J[2][0] * (J[0][1] * J[1][2] - J[1][1] * J[0][2]);
    Jdet = 1.0 / Jdet;
    double Ji[3][3] = {
        {J[1][1] * J[2][2] - J[2][1] * J[1][2], J[2][1] * J[0][2] - J[0][1] * J[2][2], J[0][1] * J[1][2] - J[1][1] * J[0][2]},
        {J[2][0] * J[1][2] - J[1][0] * J[2][2], J[0][0] * J[2][2] - J[2][0] * J[0][2], J[1][0] * J[0][2] - J[0][0] * J[1][2]},
        {J[1][0] * J[2][1] - J[2][0] * J[1][1], J[2][0] * J[0][1] - J[0][0] * J[2][1], J[0][0] * J[1][1] - J[1][0] * J[0][1]}};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Ji[i][j] *= Jdet;
    double gs[3], gn[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        gs[i] = 0.5 * (Ji[i][0] * uvw[0] + Ji[i][1] * uvw[1] + Ji[i][2] * uvw[2]);
#pragma unroll
        for (int j = 0; j < 3; ++j) gn[j][i] = -0.5 * Ji[i][j] * uvw[j];
    }
    int j = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const double* g;
        if (k == node) g = gs;
        else if (k == nn[0]) g = gn[0];
        else if (k == nn[1]) g = gn[1];
        else if (k == nn[2]) g = gn[2];
        else continue;
        ids[4 * (size_t)p + j] = hx[k];
        double* o = coef + 12 * (size_t)p + 3 * j;
        o[0] = g[0];
        o[1] = g[1];
        o[2] = g[2];
        ++j;
    }
}

// k_nodal_field from the per-item gradients of k_nodal_coef
__global__ void k_nodal_field_cached(int n_nodes, const int32_t* __restrict__ n2c_ptr, const int32_t* __restrict__ ids,
                                     const double* __restrict__ coef, double* __restrict__ sol) {
    const int node_id = blockIdx.x * blockDim.x + threadIdx.x;
    if (node_id >= n_nodes) return;
    const int b = n2c_ptr[node_id], e = n2c_ptr[node_id + 1];
    if (b == e) return;
    double mx = 0.0, my = 0.0, mz = 0.0;
    for (int p = b; p < e; ++p) {
        double ex = 0.0, ey = 0.0, ez = 0.0;
        const double* c = coef + 12 * (size_t)p;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const double ph = sol[5 * (size_t)ids[4 * (size_t)p + j] + 4];
            ex -= c[3 * j] * ph;
            ey -= c[3 * j + 1] * ph;
            ez -= c[3 * j + 2] * ph;
        }
        mx += ex;
        my += ey;
        mz += ez;
    }
    const double f = 1.0 / (e - b);
    double* s = sol + 5 * (size_t)node_id;
    s[0] = mx * f;
    s[1] = my * f;
    s[2] = mz * f;
}

// k_smooth's weights exp(decay |x_i - x_nb|) per neighbour item and 1 / (their sum) per tet
// vertex (-1 where the reference skips the vertex: no neighbours or a sum that is not positive)
__global__ void k_smooth_coef(int n_tn, const int32_t* __restrict__ vptr, const int32_t* __restrict__ vidx,
                              const double* __restrict__ xyz, double decay, double* __restrict__ w_out,
                              double* __restrict__ f_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_tn) return;
    const int b = vptr[i], e = vptr[i + 1];
    const double px = xyz[3 * (size_t)i], py = xyz[3 * (size_t)i + 1], pz = xyz[3 * (size_t)i + 2];
    double ws = 0;
    for (int k = b; k < e; ++k) {
        const int nb = vidx[k];
        const double dx = px - xyz[3 * (size_t)nb], dy = py - xyz[3 * (size_t)nb + 1], dz = pz - xyz[3 * (size_t)nb + 2];
        const double w = exp(decay * sqrt(dx * dx + dy * dy + dz * dz));
        w_out[k] = w;
        ws += w;
    }
    f_out[i] = (b != e && ws > 0) ? 1.0 / ws : -1.0;
}

// k_smooth from the weights of k_smooth_coef
__global__ void k_smooth_cached(int n_tn, const int32_t* __restrict__ vptr, const int32_t* __restrict__ vidx,
                                const double* __restrict__ wk, const double* __restrict__ fi, double* __restrict__ sol) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_tn) return;
    const double f = fi[i];
    if (f < 0) return;
    const int b = vptr[i], e = vptr[i + 1];
    double vx = 0, vy = 0, vz = 0;
    for (int k = b; k < e; ++k) {
        const int nb = vidx[k];
        const double w = wk[k];
        vx += sol[5 * (size_t)nb] * w;
        vy += sol[5 * (size_t)nb + 1] * w;
        vz += sol[5 * (size_t)nb + 2] * w;
    }
    sol[5 * (size_t)i] = vx * f;
    sol[5 * (size_t)i + 1] = vy * f;
    sol[5 * (size_t)i + 2] = vz * f;
}

__global__ void k_max_norm2(int n, const double* __restrict__ sol, unsigned long long* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* s = sol + 5 * (size_t)i;
    const double v = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
    // non-negative doubles order like their bit patterns
    atomicMax(out, (unsigned long long)__double_as_longlong(v));
}

}  // namespace

// ==================================================================== allocation-free variant
// Scratch of DeviceMesh::locate_interpolate_noalloc: five int32 per query point (walk result,
// containing-tet count, nearest-centroid tet, resolved cell, dependency flag) plus eight
// counters, for at most kNoAllocMaxPoints points. It is a file-scope device array: every
// GPU that loads this library holds these ~5.2 MB until the process exits, and every call
// shares it, so calls that overlap on the GPU (two streams, or two host threads) race.
constexpr int kNoAllocMaxPoints = 262144;
static __device__ __align__(256) int32_t g_noalloc_scratch[5 * kNoAllocMaxPoints + 8];

namespace {
std::mutex g_noalloc_mutex;
void* g_noalloc_addr[256] = {};  // device address of g_noalloc_scratch, per device ordinal
}  // namespace

// Device address of the scratch array on the current device. The host-side symbol
// g_noalloc_scratch is only a stand-in and must never be passed to a kernel; the address is
// looked up once per device, with that device current, when the first DeviceMesh is built
// there (which also loads this file's module, so the allocation-free calls themselves do no
// set-up). The address is cached per device ordinal: a device reset while the library is
// loaded is unsupported, since the cached address would then be stale.
static int32_t* noalloc_scratch() {
    int dev = 0;
    FGB_CUDA(cudaGetDevice(&dev));
    FGB_REQUIRE(dev >= 0 && dev < 256, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        FGB_REQUIRE(e == cudaSuccess && p, std::string("cudaGetSymbolAddress of the location scratch failed: ") +
                                               cudaGetErrorString(e));
        g_noalloc_addr[dev] = p;
    }
    return static_cast<int32_t*>(g_noalloc_addr[dev]);
}

// ==================================================================== host side
SeedGrid build_seed_grid(const PreparedMesh& pm) {
    SeedGrid g;
    const int nt = pm.tet.n_tets();
    double ext[3];
    for (int c = 0; c < 3; ++c) ext[c] = std::max(1e-9, pm.bbox_max[c] - pm.bbox_min[c]);
    // about four tets per cell on average
    const double cells = std::max(1.0, nt / 4.0);
    const double h = std::cbrt(ext[0] * ext[1] * ext[2] / cells);
    for (int c = 0; c < 3; ++c) {
        g.dim[c] = std::max(1, std::min(1024, (int)std::ceil(ext[c] / h)));
        g.origin[c] = pm.bbox_min[c];
        g.step[c] = ext[c] / g.dim[c];
    }
    const size_t ncell = (size_t)g.dim[0] * g.dim[1] * g.dim[2];
    auto cell_of = [&](const double* p) {
        int ii[3];
        for (int c = 0; c < 3; ++c) {
            int v = (int)std::floor((p[c] - g.origin[c]) / g.step[c]);
            ii[c] = std::min(std::max(v, 0), g.dim[c] - 1);
        }
        return ((size_t)ii[2] * g.dim[1] + ii[1]) * g.dim[0] + ii[0];
    };
    std::vector<size_t> tc(nt);
    g.ptr.assign(ncell + 1, 0);
    for (int t = 0; t < nt; ++t) {
        tc[t] = cell_of(&pm.tt.centroid[3 * (size_t)t]);
        g.ptr[tc[t] + 1]++;
    }
    for (size_t c = 0; c < ncell; ++c) g.ptr[c + 1] += g.ptr[c];
    g.tets.resize(nt);
    g.cxyz.resize(3 * (size_t)nt);
    {
        std::vector<int32_t> pos(g.ptr.begin(), g.ptr.end() - 1);
        for (int t = 0; t < nt; ++t) {
            const int32_t q = pos[tc[t]]++;
            g.tets[q] = t;
            for (int c = 0; c < 3; ++c) g.cxyz[3 * (size_t)q + c] = pm.tt.centroid[3 * (size_t)t + c];
        }
    }
    g.seed.assign(ncell, -1);
    std::deque<size_t> q;
    for (size_t c = 0; c < ncell; ++c)
        if (g.ptr[c + 1] > g.ptr[c]) {
            g.seed[c] = g.tets[g.ptr[c]];
            q.push_back(c);
        }
    while (!q.empty()) {
        const size_t c = q.front();
        q.pop_front();
        const int i = (int)(c % g.dim[0]), j = (int)((c / g.dim[0]) % g.dim[1]), k = (int)(c / ((size_t)g.dim[0] * g.dim[1]));
        const int nb[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k}, {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
        for (auto& v : nb) {
            if (v[0] < 0 || v[1] < 0 || v[2] < 0 || v[0] >= g.dim[0] || v[1] >= g.dim[1] || v[2] >= g.dim[2]) continue;
            const size_t cc = ((size_t)v[2] * g.dim[1] + v[1]) * g.dim[0] + v[0];
            if (g.seed[cc] < 0) {
                g.seed[cc] = g.seed[c];
                q.push_back(cc);
            }
        }
    }
    return g;
}

DeviceMesh::DeviceMesh(const PreparedMesh& pm, cudaStream_t stream)
    : stream_(stream), n_nodes_(pm.hex.n_nodes()), n_tets_(pm.tet.n_tets()), n_tetnodes_(pm.hex.n_tetnodes),
      decay_(pm.decay_factor) {
    cudaStream_t s = stream_;
    for (int c = 0; c < 3; ++c) {
        const double m = 1e-9 * std::max(1.0, pm.bbox_max[c] - pm.bbox_min[c]);
        bb_lo_[c] = pm.bbox_min[c] - m;
        bb_hi_[c] = pm.bbox_max[c] + m;
    }
    grid_ = build_seed_grid(pm);
    tet_nodes_.upload(pm.tet.tets, s);
    face_nbr_.upload(pm.face_nbr, s);
    nbr_ptr_.upload(pm.tt.nbr_ptr, s);
    nbr_idx_.upload(pm.tt.nbr_idx, s);
    quad_.upload(pm.tt.quad_nodes, s);
    search_.upload(pm.tt.search, s);
    det_.upload(pm.tt.det, s);
    centroid_.upload(pm.tt.centroid, s);
    hexs_.upload(pm.hex.hexs, s);
    n2c_ptr_.upload(pm.n2c_ptr, s);
    n2c_item_.upload(pm.n2c_item, s);
    voro_ptr_.upload(pm.voro_ptr, s);
    voro_idx_.upload(pm.voro_idx, s);
    hexf_.upload(pm.hex_coeffs, s);
    xyz_.upload(pm.hex.xyz, s);
    seed_.upload(grid_.seed, s);
    gptr_.upload(grid_.ptr, s);
    gtets_.upload(grid_.tets, s);
    gcxyz_.upload(grid_.cxyz, s);
    sol_.resize(5 * (size_t)n_nodes_);
    sol_.zero(s);
    counters_.resize(8);
    set_surface(pm);
    // set-up of the allocation-free entry point on this device: module load and the scratch
    // array's address, here rather than in a timestep loop or a stream capture
    (void)noalloc_scratch();
    FGB_CUDA(cudaStreamSynchronize(s));
    // host copies of the search tables are no longer needed
    grid_.seed.clear(); grid_.ptr.clear(); grid_.tets.clear(); grid_.cxyz.clear();
}

namespace {
// uniform grid over [lo, hi] with about `per_cell` items per cell (at most 1024 per axis)
void grid_dims(const double* lo, const double* hi, double n_items, double per_cell, int* dim, double* org, double* step) {
    double ext[3];
    for (int c = 0; c < 3; ++c) ext[c] = std::max(1e-9, hi[c] - lo[c]);
    const double cells = std::max(1.0, n_items / per_cell);
    const double h = std::cbrt(ext[0] * ext[1] * ext[2] / cells);
    for (int c = 0; c < 3; ++c) {
        dim[c] = std::max(1, std::min(1024, (int)std::ceil(ext[c] / h)));
        org[c] = lo[c];
        step[c] = ext[c] / dim[c];
    }
}
inline int grid_index(double v, double org, double step, int dim) {
    const int k = (int)std::floor((v - org) / step);
    return std::min(std::max(k, 0), dim - 1);
}
}  // namespace

void DeviceMesh::set_surface(const PreparedMesh& pm) {
    const SurfaceTables& st = pm.surf;
    n_stris_ = st.n_tris();
    if (n_stris_ == 0) return;
    cudaStream_t s = stream_;
    const int nf = n_stris_;
    const double* X = pm.tet.xyz.data();
    // acceptance region of a triangle: inside the prism over it, |distance| < |edge2|; its box
    // is that of the vertices moved by +-|edge2| along the unit normal
    std::vector<double> rlo(3 * (size_t)nf), rhi(3 * (size_t)nf);
    double glo[3] = {1e300, 1e300, 1e300}, ghi[3] = {-1e300, -1e300, -1e300};
    for (int f = 0; f < nf; ++f) {
        const double* g = &st.geo[(size_t)kTriGeoStride * f];
        for (int c = 0; c < 3; ++c) {
            double a = 1e300, b = -1e300;
            for (int k = 0; k < 3; ++k) {
                const double p = X[3 * (size_t)st.tris[3 * (size_t)f + k] + c];
                const double d = std::fabs(g[12 + c]) * g[15];
                a = std::min(a, p - d);
                b = std::max(b, p + d);
            }
            rlo[3 * (size_t)f + c] = a;
            rhi[3 * (size_t)f + c] = b;
            glo[c] = std::min(glo[c], a);
            ghi[c] = std::max(ghi[c], b);
        }
    }
    // margin far above the rounding of the point-in-triangle test
    for (int c = 0; c < 3; ++c) {
        const double m = 1e-9 * std::max(1.0, ghi[c] - glo[c]);
        glo[c] -= m;
        ghi[c] += m;
        scand_lo_[c] = glo[c];
        scand_hi_[c] = ghi[c];
    }
    for (size_t q = 0; q < rlo.size(); ++q) {
        const int c = (int)(q % 3);
        const double m = 1e-9 * std::max(1.0, ghi[c] - glo[c]);
        rlo[q] -= m;
        rhi[q] += m;
    }
    grid_dims(glo, ghi, nf, 0.5, scand_dim_, scand_org_, scand_step_);
    const size_t ncell = (size_t)scand_dim_[0] * scand_dim_[1] * scand_dim_[2];
    std::vector<int32_t> cptr(ncell + 1, 0), cidx;
    for (int pass = 0; pass < 2; ++pass) {
        std::vector<int32_t> pos;
        if (pass == 1) {
            for (size_t c = 0; c < ncell; ++c) cptr[c + 1] += cptr[c];
            cidx.resize(cptr[ncell]);
            pos.assign(cptr.begin(), cptr.end() - 1);
        }
        for (int f = 0; f < nf; ++f) {
            int a[3], b[3];
            for (int c = 0; c < 3; ++c) {
                a[c] = grid_index(rlo[3 * (size_t)f + c], scand_org_[c], scand_step_[c], scand_dim_[c]);
                b[c] = grid_index(rhi[3 * (size_t)f + c], scand_org_[c], scand_step_[c], scand_dim_[c]);
            }
            for (int k = a[2]; k <= b[2]; ++k)
                for (int j = a[1]; j <= b[1]; ++j)
                    for (int i = a[0]; i <= b[0]; ++i) {
                        const size_t c = ((size_t)k * scand_dim_[1] + j) * scand_dim_[0] + i;
                        if (pass == 0) cptr[c + 1]++;
                        else cidx[pos[c]++] = f;
                    }
        }
    }
    // centroid buckets (ascending triangle within a bucket) for the exact nearest centroid
    double clo[3] = {1e300, 1e300, 1e300}, chi[3] = {-1e300, -1e300, -1e300};
    for (int f = 0; f < nf; ++f)
        for (int c = 0; c < 3; ++c) {
            clo[c] = std::min(clo[c], st.geo[(size_t)kTriGeoStride * f + 16 + c]);
            chi[c] = std::max(chi[c], st.geo[(size_t)kTriGeoStride * f + 16 + c]);
        }
    grid_dims(clo, chi, nf, 4.0, sg_dim_, sg_org_, sg_step_);
    const size_t nb = (size_t)sg_dim_[0] * sg_dim_[1] * sg_dim_[2];
    std::vector<int32_t> gptr(nb + 1, 0), gtris(nf);
    std::vector<double> gc(3 * (size_t)nf);
    std::vector<size_t> bc(nf);
    for (int f = 0; f < nf; ++f) {
        const double* cc = &st.geo[(size_t)kTriGeoStride * f + 16];
        bc[f] = ((size_t)grid_index(cc[2], sg_org_[2], sg_step_[2], sg_dim_[2]) * sg_dim_[1] +
                 grid_index(cc[1], sg_org_[1], sg_step_[1], sg_dim_[1])) * sg_dim_[0] +
                grid_index(cc[0], sg_org_[0], sg_step_[0], sg_dim_[0]);
        gptr[bc[f] + 1]++;
    }
    for (size_t c = 0; c < nb; ++c) gptr[c + 1] += gptr[c];
    {
        std::vector<int32_t> pos(gptr.begin(), gptr.end() - 1);
        for (int f = 0; f < nf; ++f) {
            const int32_t q = pos[bc[f]]++;
            gtris[q] = f;
            for (int c = 0; c < 3; ++c) gc[3 * (size_t)q + c] = st.geo[(size_t)kTriGeoStride * f + 16 + c];
        }
    }
    stris_.upload(st.tris, s);
    stri2tet_.upload(st.tri2tet, s);
    snbr_ptr_.upload(st.nbr_ptr, s);
    snbr_idx_.upload(st.nbr_idx.empty() ? std::vector<int32_t>(1, 0) : st.nbr_idx, s);
    sgeo_.upload(st.geo, s);
    scand_ptr_.upload(cptr, s);
    scand_idx_.upload(cidx.empty() ? std::vector<int32_t>(1, 0) : cidx, s);
    sgptr_.upload(gptr, s);
    sgtris_.upload(gtris, s);
    sgcxyz_.upload(gc, s);
    s_counters_.resize(8);
    FGB_CUDA(cudaStreamSynchronize(s));
}

void DeviceMesh::surface_interpolate(int n, const double* d_pts, int rank, int32_t* d_cells, double* d_out) {
    if (n <= 0) return;
    FGB_REQUIRE(rank >= 1 && rank <= 3, "surface interpolation rank must be 1, 2 or 3");
    FGB_REQUIRE(n_stris_ > 0, "the mesh has no surface triangles");
    ensure_scratch(n);
    if (s_scratch_n_ < n) {
        s_tv_.resize(n); s_nin_.resize(n); s_tf_.resize(n); s_res_.resize(n); s_dep_.resize(n);
        s_scratch_n_ = n;
    }
    const int B = 256;
    Pts P{d_pts};
    // tets: the guess-independent results of the chained tet search
    GridView G{grid_.dim[0], grid_.dim[1], grid_.dim[2], grid_.origin[0], grid_.origin[1], grid_.origin[2],
               grid_.step[0], grid_.step[1], grid_.step[2]};
    counters_.zero(stream_);
    s_counters_.zero(stream_);
    FGB_LAUNCH(k_locate_walk<<<grid_for(n, B), B, 0, stream_>>>(n, P, G, seed_.get(), det_.get(), face_nbr_.get(),
                                                                nbr_ptr_.get(), nbr_idx_.get(), search_.get(), bb_lo_[0],
                                                                bb_lo_[1], bb_lo_[2], bb_hi_[0], bb_hi_[1], bb_hi_[2],
                                                                v_.get(), nin_.get(), counters_.get()));
    FGB_LAUNCH(k_locate_scan<<<std::min(n, 1024), B, 0, stream_>>>(n, P, n_tets_, det_.get(), search_.get(), v_.get(),
                                                                   nin_.get()));
    FGB_LAUNCH(k_nearest_ctr<<<grid_for(n, 128), 128, 0, stream_>>>(n, P, G, gptr_.get(), gtets_.get(), gcxyz_.get(),
                                                                    v_.get(), f_.get(), counters_.get()));
    // triangles: scan result, nearest centroid, then the chained search of a fresh reader
    // (first guess abs(-1) = 1)
    GridView C{scand_dim_[0], scand_dim_[1], scand_dim_[2], scand_org_[0], scand_org_[1], scand_org_[2],
               scand_step_[0], scand_step_[1], scand_step_[2]};
    GridView S{sg_dim_[0], sg_dim_[1], sg_dim_[2], sg_org_[0], sg_org_[1], sg_org_[2], sg_step_[0], sg_step_[1],
               sg_step_[2]};
    FGB_LAUNCH(k_tri_locate<<<grid_for(n, B), B, 0, stream_>>>(n, P, C, scand_lo_[0], scand_lo_[1], scand_lo_[2],
                                                               scand_hi_[0], scand_hi_[1], scand_hi_[2], scand_ptr_.get(),
                                                               scand_idx_.get(), sgeo_.get(), s_tv_.get(), s_nin_.get()));
    FGB_LAUNCH(k_nearest_ctr<<<grid_for(n, 128), 128, 0, stream_>>>(n, P, S, sgptr_.get(), sgtris_.get(), sgcxyz_.get(),
                                                                    s_tv_.get(), s_tf_.get(), s_counters_.get()));
    FGB_LAUNCH(k_resolve<<<grid_for(n, B), B, 0, stream_>>>(n, s_tv_.get(), s_nin_.get(), s_tf_.get(), s_res_.get(),
                                                            s_dep_.get(), s_counters_.get()));
    // rank 3 keeps quadrangle cells: its first guess is quadrangle 1's triangle, 0
    FGB_LAUNCH(k_tri_chain_runs<<<grid_for(n, B), B, 0, stream_>>>(n, P, rank == 3 ? 0 : 1, n_stris_, sgeo_.get(),
                                                                   snbr_ptr_.get(), snbr_idx_.get(), s_tv_.get(),
                                                                   s_tf_.get(), s_dep_.get(), s_res_.get(),
                                                                   s_counters_.get()));
    if (rank == 3) {
        FGB_LAUNCH(k_surface_hex<<<grid_for(n, B), B, 0, stream_>>>(n, P, s_res_.get(), stris_.get(), stri2tet_.get(),
                                                                    sgeo_.get(), det_.get(), tet_nodes_.get(),
                                                                    nbr_ptr_.get(), nbr_idx_.get(), v_.get(), f_.get(),
                                                                    s_tv_.get(), res_.get()));
    } else {
        FGB_LAUNCH(k_surface_tet<<<grid_for(n, B), B, 0, stream_>>>(n, P, s_res_.get(), stri2tet_.get(), sgeo_.get(),
                                                                    det_.get(), nbr_ptr_.get(), nbr_idx_.get(), v_.get(),
                                                                    f_.get(), res_.get()));
    }
    FGB_LAUNCH(k_interpolate<<<grid_for(n, 128), 128, 0, stream_>>>(n, P, rank, 0, res_.get(), det_.get(), tet_nodes_.get(),
                                                                    quad_.get(), hexs_.get(), hexf_.get(), sol_.get(),
                                                                    nullptr, d_out));
    // cells: triangles (ranks 1, 2) or quadrangles (rank 3, computed into s_tv_)
    if (d_cells)
        FGB_CUDA(cudaMemcpyAsync(d_cells, rank == 3 ? s_tv_.get() : s_res_.get(), sizeof(int32_t) * n,
                                 cudaMemcpyDeviceToDevice, stream_));
    FGB_CUDA(cudaGetLastError());
}

void DeviceMesh::ensure_scratch(int n) {
    if (n <= scratch_n_) return;
    v_.resize(n); nin_.resize(n); f_.resize(n); res_.resize(n); dep_.resize(n);
    scratch_n_ = n;
}

void DeviceMesh::extract_solution(const double* d_phi, const int32_t* d_dof2node, int n_dofs, bool smoothen,
                                  const double* d_charge) {
    const int B = 256;
    sol_.zero(stream_);
    FGB_LAUNCH(k_scatter_solution<<<grid_for(n_dofs, B), B, 0, stream_>>>(n_dofs, d_phi, d_charge, d_dof2node, sol_.get()));
    if (geo_cache_) {
        // the geometry-only factors are built at the first extraction of this mesh
        if (!nodal_ids_.size()) {
            const int n_items = (int)n2c_item_.size();
            nodal_ids_.resize(4 * (size_t)std::max(1, n_items));
            nodal_coef_.resize(12 * (size_t)std::max(1, n_items));
            if (n_items > 0)
                FGB_LAUNCH(k_nodal_coef<<<grid_for(n_items, B), B, 0, stream_>>>(n_items, n2c_item_.get(), hexs_.get(),
                                                                                 xyz_.get(), nodal_ids_.get(),
                                                                                 nodal_coef_.get()));
            const int n_vor = (int)voro_idx_.size();
            smooth_w_.resize(std::max(1, n_vor));
            smooth_f_.resize(std::max(1, n_tetnodes_));
            if (n_tetnodes_ > 0)
                FGB_LAUNCH(k_smooth_coef<<<grid_for(n_tetnodes_, B), B, 0, stream_>>>(n_tetnodes_, voro_ptr_.get(),
                                                                                     voro_idx_.get(), xyz_.get(), decay_,
                                                                                     smooth_w_.get(), smooth_f_.get()));
        }
        FGB_LAUNCH(k_nodal_field_cached<<<grid_for(n_nodes_, B), B, 0, stream_>>>(n_nodes_, n2c_ptr_.get(), nodal_ids_.get(),
                                                                                 nodal_coef_.get(), sol_.get()));
        if (smoothen && n_tetnodes_ > 0)
            FGB_LAUNCH(k_smooth_cached<<<grid_for(n_tetnodes_, B), B, 0, stream_>>>(n_tetnodes_, voro_ptr_.get(), voro_idx_.get(),
                                                                                   smooth_w_.get(), smooth_f_.get(), sol_.get()));
    } else {
        FGB_LAUNCH(k_nodal_field<<<grid_for(n_nodes_, B), B, 0, stream_>>>(n_nodes_, n2c_ptr_.get(), n2c_item_.get(), hexs_.get(),
                                                                          xyz_.get(), sol_.get()));
        if (smoothen)
            FGB_LAUNCH(k_smooth<<<grid_for(n_tetnodes_, B), B, 0, stream_>>>(n_tetnodes_, voro_ptr_.get(), voro_idx_.get(),
                                                                            xyz_.get(), decay_, sol_.get()));
    }
    FGB_CUDA(cudaGetLastError());
}

double DeviceMesh::max_field_norm() {
    counters_.zero(stream_);
    unsigned long long* acc = reinterpret_cast<unsigned long long*>(counters_.get());
    FGB_LAUNCH(k_max_norm2<<<grid_for(n_nodes_, 256), 256, 0, stream_>>>(n_nodes_, sol_.get(), acc));
    unsigned long long h = 0;
    FGB_CUDA(cudaMemcpyAsync(&h, acc, sizeof(h), cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
    double v;
    memcpy(&v, &h, sizeof(v));
    return std::sqrt(v);
}

void DeviceMesh::set_solution(const double* h) {
    FGB_CUDA(cudaMemcpyAsync(sol_.get(), h, sol_.bytes(), cudaMemcpyHostToDevice, stream_));
}
void DeviceMesh::get_solution(double* h) {
    FGB_CUDA(cudaMemcpyAsync(h, sol_.get(), sol_.bytes(), cudaMemcpyDeviceToHost, stream_));
    FGB_CUDA(cudaStreamSynchronize(stream_));
}

void DeviceMesh::locate_interpolate(int n, const double* d_pts, int rank, int32_t* d_cells, double* d_out,
                                    LocateStats* stats) {
    if (n <= 0) return;
    FGB_REQUIRE(rank >= 1 && rank <= 3, "interpolation rank must be 1, 2 or 3");
    ensure_scratch(n);
    const int B = 256;
    Pts P{d_pts};
    GridView G{grid_.dim[0], grid_.dim[1], grid_.dim[2], grid_.origin[0], grid_.origin[1], grid_.origin[2],
               grid_.step[0], grid_.step[1], grid_.step[2]};
    counters_.zero(stream_);
    FGB_LAUNCH(k_locate_walk<<<grid_for(n, B), B, 0, stream_>>>(n, P, G, seed_.get(), det_.get(), face_nbr_.get(), nbr_ptr_.get(),
                                                     nbr_idx_.get(), search_.get(), bb_lo_[0], bb_lo_[1], bb_lo_[2], bb_hi_[0],
                                                     bb_hi_[1], bb_hi_[2], v_.get(), nin_.get(), counters_.get()));
    FGB_LAUNCH(k_locate_scan<<<std::min(n, 1024), B, 0, stream_>>>(n, P, n_tets_, det_.get(), search_.get(), v_.get(), nin_.get()));
    FGB_LAUNCH(k_nearest_ctr<<<grid_for(n, 128), 128, 0, stream_>>>(n, P, G, gptr_.get(), gtets_.get(), gcxyz_.get(), v_.get(), f_.get(),
                                                         counters_.get()));
    FGB_LAUNCH(k_resolve<<<grid_for(n, B), B, 0, stream_>>>(n, v_.get(), nin_.get(), f_.get(), res_.get(), dep_.get(), counters_.get()));
    // first guess of a fresh reader: abs(-1) = 1 for tets, abs(-1)/4 = 0 for hexes
    const int g0 = rank == 3 ? 0 : std::min(1, n_tets_ - 1);
    FGB_LAUNCH(k_chain_runs<<<grid_for(32LL * n, B), B, 0, stream_>>>(n, P, g0, det_.get(), nbr_ptr_.get(), nbr_idx_.get(), v_.get(), f_.get(),
                                                    dep_.get(), res_.get(), counters_.get()));
    FGB_LAUNCH(k_interpolate<<<grid_for(n, 128), 128, 0, stream_>>>(n, P, rank, 1, res_.get(), det_.get(), tet_nodes_.get(), quad_.get(),
                                                         hexs_.get(), hexf_.get(), sol_.get(), d_cells, d_out));
    FGB_CUDA(cudaGetLastError());
    if (stats) {
        int32_t h[8];
        FGB_CUDA(cudaMemcpyAsync(h, counters_.get(), sizeof(h), cudaMemcpyDeviceToHost, stream_));
        FGB_CUDA(cudaStreamSynchronize(stream_));
        stats->n_points = n;
        stats->n_walk_failed = h[0];
        stats->n_fallback = h[1];
        stats->n_dependent = h[2];
        stats->longest_run = h[3];
    }
}

void DeviceMesh::locate_interpolate_noalloc(int n, const double* d_pts, int rank, int32_t* d_cells, double* d_out) {
    if (n <= 0) return;
    FGB_REQUIRE(rank >= 1 && rank <= 3, "interpolation rank must be 1, 2 or 3");
    FGB_REQUIRE(n <= kNoAllocMaxPoints, "the allocation-free interpolation takes at most " +
                                            std::to_string(kNoAllocMaxPoints) + " points per call, got " +
                                            std::to_string(n));
    int32_t* base = noalloc_scratch();
    int32_t* V = base;
    int32_t* nin = base + kNoAllocMaxPoints;
    int32_t* F = base + 2 * kNoAllocMaxPoints;
    int32_t* res = base + 3 * kNoAllocMaxPoints;
    int32_t* dep = base + 4 * kNoAllocMaxPoints;
    int32_t* counters = base + 5 * kNoAllocMaxPoints;
    // the per-point slots are fully rewritten before they are read; only the counters must
    // start at zero (the array keeps the previous call's contents)
    FGB_CUDA(cudaMemsetAsync(counters, 0, 8 * sizeof(int32_t), stream_));
    const int B = 256;
    Pts P{d_pts};
    GridView G{grid_.dim[0], grid_.dim[1], grid_.dim[2], grid_.origin[0], grid_.origin[1], grid_.origin[2],
               grid_.step[0], grid_.step[1], grid_.step[2]};
    FGB_LAUNCH(k_locate_walk<<<grid_for(n, B), B, 0, stream_>>>(n, P, G, seed_.get(), det_.get(), face_nbr_.get(), nbr_ptr_.get(),
                                                     nbr_idx_.get(), search_.get(), bb_lo_[0], bb_lo_[1], bb_lo_[2], bb_hi_[0],
                                                     bb_hi_[1], bb_hi_[2], V, nin, counters));
    FGB_LAUNCH(k_locate_scan<<<std::min(n, 1024), B, 0, stream_>>>(n, P, n_tets_, det_.get(), search_.get(), V, nin));
    FGB_LAUNCH(k_nearest_ctr<<<grid_for(n, 128), 128, 0, stream_>>>(n, P, G, gptr_.get(), gtets_.get(), gcxyz_.get(), V, F,
                                                                    counters));
    FGB_LAUNCH(k_resolve<<<grid_for(n, B), B, 0, stream_>>>(n, V, nin, F, res, dep, counters));
    const int g0 = rank == 3 ? 0 : std::min(1, n_tets_ - 1);
    FGB_LAUNCH(k_chain_runs<<<grid_for(32LL * n, B), B, 0, stream_>>>(n, P, g0, det_.get(), nbr_ptr_.get(), nbr_idx_.get(), V, F, dep,
                                                              res, counters));
    FGB_LAUNCH(k_interpolate<<<grid_for(n, 128), 128, 0, stream_>>>(n, P, rank, 1, res, det_.get(), tet_nodes_.get(),
                                                                    quad_.get(), hexs_.get(), hexf_.get(), sol_.get(), d_cells,
                                                                    d_out));
    FGB_CUDA(cudaGetLastError());
}

void DeviceMesh::space_charge(int n, const double* d_pts, const int32_t* d_hex, int order, const int32_t* d_node2dof,
                              const int32_t* d_hex2cell, const int32_t* d_cell_dofs, double charge_factor,
                              double* d_rhs, int* n_skipped) {
    if (n <= 0) return;
    FGB_REQUIRE(order == 1 || order == 2, "element order must be 1 or 2");
    counters_.zero(stream_);
    Pts P{d_pts};
    FGB_LAUNCH(k_space_charge<<<grid_for(n, 256), 256, 0, stream_>>>(n, P, d_hex, hexf_.get(), hexs_.get(), d_node2dof,
                                                                     order, d_hex2cell, d_cell_dofs, charge_factor,
                                                                     d_rhs, counters_.get()));
    FGB_CUDA(cudaGetLastError());
    if (n_skipped) {
        int32_t h = 0;
        FGB_CUDA(cudaMemcpyAsync(&h, counters_.get(), sizeof(int32_t), cudaMemcpyDeviceToHost, stream_));
        FGB_CUDA(cudaStreamSynchronize(stream_));
        *n_skipped = h;
    }
}

void DeviceMesh::interpolate_known(int n, const double* d_pts, int rank, const int32_t* d_cells, double* d_out) {
    if (n <= 0) return;
    Pts P{d_pts};
    FGB_LAUNCH(k_interpolate<<<grid_for(n, 128), 128, 0, stream_>>>(n, P, rank, 0, d_cells, det_.get(), tet_nodes_.get(), quad_.get(),
                                                         hexs_.get(), hexf_.get(), sol_.get(), nullptr, d_out));
    FGB_CUDA(cudaGetLastError());
}

}  // namespace fgb
