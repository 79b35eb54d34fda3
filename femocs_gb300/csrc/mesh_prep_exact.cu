// Device preparation of a tetrahedral mesh: every table of prepare_mesh (mesh.cpp,
// prepared.cpp) built by kernels from the tets and their vertices, then downloaded into a
// PreparedMesh. Compiled with -fmad=false: coordinates, determinants and trilinear
// coefficients come from the same IEEE operation sequence as the host (mesh_math.h), and
// every integer table has the same order, so the two builders agree bit for bit.
//
// Reference steps reproduced:
//   * edges numbered by ascending (max, min) vertex pair, faces by first encounter while
//     walking tets, their local edges and the vertices opposite to each edge; nodes = tet
//     vertices, then edge, face and tet centroids (src/Tethex.cpp:965-1035, 1244-1342);
//   * hex 4t+k around tet vertex k, front and back swapped when its volume is negative
//     (src/Tethex.cpp:1037-1102), markers +-(1+vertex) (src/TetgenMesh.cpp:353-385);
//   * per tet 1/D and the barycentric minors, the centroid and the location candidates:
//     face neighbours, then the tets sharing each vertex (src/InterpolatorCells.cpp:523-629);
//   * per hex the trilinear coefficients f0..f7 (src/InterpolatorCells.cpp:1205-1267);
//   * vacuum vertex compaction (src/DealSolver.cpp:192-208) and the pseudo-Voronoi stencils
//     of the nodal-field smoothing (src/TetgenMesh.cpp:819-837).
// Grouping uses the stable radix sort of dprim.cuh. The first-encounter face order comes
// from the face neighbours: a face is first met in the lower-numbered tet that holds it, at
// the first (local edge, opposite vertex) slot of that tet spanning it.
#include "mesh_prep.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "dprim.cuh"
#include "mesh_math.h"

namespace fgb {
using namespace dprim;

namespace {

constexpr int kB = 256;
enum : int { kErrDegenerate = 1, kErrNonManifold = 2, kErrEdges = 4, kErrLookup = 8 };

inline unsigned blocks(int64_t n) { return (unsigned)std::max<int64_t>(1, (n + kB - 1) / kB); }

__device__ __forceinline__ int64_t gid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }

__device__ __forceinline__ void load4(const int32_t* __restrict__ T, int64_t t, int32_t v[4]) {
    const int4 q = reinterpret_cast<const int4*>(T)[t];
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
}

__device__ __forceinline__ void sort3(int32_t& a, int32_t& b, int32_t& c) {
    int32_t t;
    if (a > b) { t = a; a = b; b = t; }
    if (b > c) { t = b; b = c; c = t; }
    if (a > b) { t = a; a = b; b = t; }
}

// the three vertices of tet face j (opposite local vertex j), ascending
__device__ __forceinline__ void face_of(const int32_t v[4], int j, int32_t f[3]) {
    int m = 0;
    for (int k = 0; k < 4; ++k)
        if (k != j) f[m++] = v[k];
    sort3(f[0], f[1], f[2]);
}

__device__ __forceinline__ int find_key(const uint64_t* __restrict__ a, int n, uint64_t key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ int edge_index(const uint64_t* __restrict__ ek, int ne, int nb, int32_t x, int32_t y,
                                          int* err) {
    const int32_t hi = max(x, y), lo = min(x, y);
    const uint64_t key = ((uint64_t)hi << nb) | (uint64_t)lo;
    const int e = find_key(ek, ne, key);
    if (e >= ne || ek[e] != key) {
        atomicOr(err, kErrLookup);
        return 0;
    }
    return e;
}

// ---------------------------------------------------------------- edges
__global__ void k_edge_keys(int nt, const int32_t* __restrict__ T, int nb, uint64_t* __restrict__ keys, int* err) {
    const int64_t t = gid();
    if (t >= nt) return;
    int32_t v[4];
    load4(T, t, v);
    int s = 0;
    for (int i = 0; i < 4; ++i)
        for (int j = i + 1; j < 4; ++j) {
            const int32_t hi = max(v[i], v[j]), lo = min(v[i], v[j]);
            if (hi == lo) atomicOr(err, kErrDegenerate);
            keys[6 * t + s++] = ((uint64_t)hi << nb) | (uint64_t)lo;
        }
}

__global__ void k_head_flags(int64_t n, const uint64_t* __restrict__ k, int* __restrict__ flag) {
    const int64_t i = gid();
    if (i < n) flag[i] = (i == 0 || k[i] != k[i - 1]) ? 1 : 0;
}

__global__ void k_compact_heads(int64_t n, const uint64_t* __restrict__ k, const int* __restrict__ pos,
                                uint64_t* __restrict__ out) {
    const int64_t i = gid();
    if (i < n && (i == 0 || k[i] != k[i - 1])) out[pos[i]] = k[i];
}

// ---------------------------------------------------------------- faces
__global__ void k_face_keys(int nt, const int32_t* __restrict__ T, int nb, uint64_t* __restrict__ keys,
                            int32_t* __restrict__ slots) {
    const int64_t i = gid();
    if (i >= 4LL * nt) return;
    int32_t v[4], f[3];
    load4(T, i >> 2, v);
    face_of(v, (int)(i & 3), f);
    keys[i] = ((uint64_t)f[0] << (2 * nb)) | ((uint64_t)f[1] << nb) | (uint64_t)f[2];
    slots[i] = (int32_t)i;
}

// sorted face keys: equal neighbours are the two tets of an interior face
__global__ void k_face_pairs(int64_t n, const uint64_t* __restrict__ k, const int32_t* __restrict__ slot,
                             int32_t* __restrict__ nbr, int* err) {
    const int64_t i = gid();
    if (i >= n || (i > 0 && k[i - 1] == k[i])) return;
    if (i + 1 < n && k[i + 1] == k[i]) {
        if (i + 2 < n && k[i + 2] == k[i]) {
            atomicOr(err, kErrNonManifold);
            return;
        }
        nbr[slot[i]] = slot[i + 1] / 4;
        nbr[slot[i + 1]] = slot[i] / 4;
    }
}

// first (local edge, third vertex) slot of the tet at which each face is met
__device__ __forceinline__ void face_first_slots(const int32_t v[4], int ms[4]) {
    const mm::LocalEdges le = mm::local_edges(v);
    for (int j = 0; j < 4; ++j) ms[j] = 1 << 20;
    int slot = 0;
    for (int e = 0; e < le.n; ++e)
        for (int k = 0; k < 4; ++k) {
            if (k == le.a[e] || k == le.b[e]) continue;
            const int opp = 6 - le.a[e] - le.b[e] - k;
            if (ms[opp] > slot) ms[opp] = slot;
            ++slot;
        }
}

__device__ __forceinline__ bool owns(const int32_t* __restrict__ nbr, int64_t t, int j) {
    const int32_t u = nbr[4 * t + j];
    return u < 0 || u > t;
}

__global__ void k_face_count(int nt, const int32_t* __restrict__ nbr, int* __restrict__ cnt) {
    const int64_t t = gid();
    if (t >= nt) return;
    int c = 0;
    for (int j = 0; j < 4; ++j) c += owns(nbr, t, j) ? 1 : 0;
    cnt[t] = c;
}

__global__ void k_face_owned(int nt, const int32_t* __restrict__ T, const int32_t* __restrict__ nbr,
                             const int* __restrict__ off, int32_t* __restrict__ tet_face, int32_t* __restrict__ fv) {
    const int64_t t = gid();
    if (t >= nt) return;
    int32_t v[4];
    load4(T, t, v);
    int ms[4];
    face_first_slots(v, ms);
    for (int j = 0; j < 4; ++j) {
        if (!owns(nbr, t, j)) continue;
        int r = 0;
        for (int j2 = 0; j2 < 4; ++j2)
            if (j2 != j && owns(nbr, t, j2) && ms[j2] < ms[j]) ++r;
        const int f = off[t] + r;
        tet_face[4 * t + j] = f;
        int32_t fa[3];
        face_of(v, j, fa);
        fv[3 * (int64_t)f] = fa[0];
        fv[3 * (int64_t)f + 1] = fa[1];
        fv[3 * (int64_t)f + 2] = fa[2];
    }
}

__global__ void k_face_shared(int nt, const int32_t* __restrict__ T, const int32_t* __restrict__ nbr,
                              int32_t* __restrict__ tet_face, int* err) {
    const int64_t t = gid();
    if (t >= nt) return;
    int32_t v[4];
    load4(T, t, v);
    for (int j = 0; j < 4; ++j) {
        if (owns(nbr, t, j)) continue;
        const int32_t u = nbr[4 * t + j];
        int32_t f[3], w[4], g[3];
        face_of(v, j, f);
        load4(T, u, w);
        int found = -1;
        for (int j2 = 0; j2 < 4 && found < 0; ++j2) {
            face_of(w, j2, g);
            if (g[0] == f[0] && g[1] == f[1] && g[2] == f[2]) found = tet_face[4 * (int64_t)u + j2];
        }
        if (found < 0) atomicOr(err, kErrLookup);
        tet_face[4 * t + j] = found < 0 ? 0 : found;
    }
}

// ---------------------------------------------------------------- nodes and hexes
__global__ void k_nodes(int n_old, int ne, int nf, int nt, int nb, const double* __restrict__ X,
                        const uint64_t* __restrict__ ek, const int32_t* __restrict__ fv, const int32_t* __restrict__ T,
                        double* __restrict__ xyz, int8_t* __restrict__ marker, int32_t* __restrict__ par) {
    const int64_t i = gid();
    const int64_t n = (int64_t)n_old + ne + nf + nt;
    if (i >= n) return;
    int32_t p[4] = {-1, -1, -1, -1};
    double o[3];
    int8_t mk;
    if (i < n_old) {
        for (int c = 0; c < 3; ++c) o[c] = X[3 * i + c];
        mk = kTetNode;
        p[0] = (int32_t)i;
    } else if (i < (int64_t)n_old + ne) {
        const int64_t e = i - n_old;
        const int32_t hi = (int32_t)(ek[e] >> nb), lo = (int32_t)(ek[e] & ((1ull << nb) - 1));
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            s += X[3 * (int64_t)lo + c];
            s += X[3 * (int64_t)hi + c];
            o[c] = s / 2;
        }
        mk = kEdgeCentroid;
        p[0] = lo;
        p[1] = hi;
    } else if (i < (int64_t)n_old + ne + nf) {
        const int64_t f = i - n_old - ne;
        for (int k = 0; k < 3; ++k) p[k] = fv[3 * f + k];
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += X[3 * (int64_t)p[k] + c];
            o[c] = s / 3;
        }
        mk = kFaceCentroid;
    } else {
        const int64_t t = i - n_old - ne - nf;
        load4(T, t, p);
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += X[3 * (int64_t)p[k] + c];
            o[c] = s / 4;
        }
        mk = kTetCentroid;
    }
    for (int c = 0; c < 3; ++c) xyz[3 * i + c] = o[c];
    marker[i] = mk;
    for (int k = 0; k < 4; ++k) par[4 * i + k] = p[k];
}

__global__ void k_hexes(int nt, int n_old, int ne, int nf, int nb, const int32_t* __restrict__ T,
                        const int32_t* __restrict__ tmarker, const uint64_t* __restrict__ ek,
                        const int32_t* __restrict__ tet_face, const double* __restrict__ xyz, int32_t* __restrict__ hexs,
                        int32_t* __restrict__ hmarker, int* err) {
    const int64_t idx = gid();
    if (idx >= 4LL * nt) return;
    const int64_t t = idx >> 2;
    const int ver = (int)(idx & 3);
    int32_t v[4];
    load4(T, t, v);
    const mm::LocalEdges le = mm::local_edges(v);
    int other[3], ns = 0;
    for (int e = 0; e < le.n && ns < 3; ++e) {
        if (le.a[e] == ver) other[ns++] = le.b[e];
        else if (le.b[e] == ver) other[ns++] = le.a[e];
    }
    if (ns != 3) {  // degenerate tets are rejected before this kernel; keep the ids in range anyway
        atomicOr(err, kErrEdges);
        for (int i = 0; i < 8; ++i) hexs[8 * idx + i] = v[ver];
        hmarker[idx] = -1 - v[ver];
        return;
    }
    auto edge_node = [&](int k) { return n_old + edge_index(ek, ne, nb, v[ver], v[other[k]], err); };
    auto face_node = [&](int k1, int k2) {
        return n_old + ne + tet_face[4 * t + (6 - ver - other[k1] - other[k2])];
    };
    int32_t h[8];
    h[0] = v[ver];
    h[1] = edge_node(0);
    h[2] = face_node(0, 1);
    h[3] = edge_node(1);
    h[4] = edge_node(2);
    h[5] = face_node(0, 2);
    h[6] = (int32_t)(n_old + ne + nf + t);
    h[7] = face_node(1, 2);
    double d[24];
    for (int i = 0; i < 8; ++i)
        for (int c = 0; c < 3; ++c) d[3 * mm::to_deal(i) + c] = xyz[3 * (int64_t)h[i] + c];
    if (mm::hex_orientation(d) < 0)
        for (int i = 0; i < 4; ++i) {
            const int32_t q = h[i];
            h[i] = h[i + 4];
            h[i + 4] = q;
        }
    for (int i = 0; i < 8; ++i) hexs[8 * idx + i] = h[i];
    hmarker[idx] = tmarker[t] == kVacuum ? (1 + v[ver]) : (-1 - v[ver]);
}

// ---------------------------------------------------------------- per-tet tables
__global__ void k_n2t_entries(int nt, const int32_t* __restrict__ T, uint32_t* __restrict__ keys,
                              int32_t* __restrict__ vals, int* __restrict__ cnt) {
    const int64_t i = gid();
    if (i >= 4LL * nt) return;
    const int32_t v = T[i];
    keys[i] = (uint32_t)v;
    vals[i] = (int32_t)(i >> 2);
    atomicAdd(&cnt[v], 1);
}

// location candidates of tet t: face neighbours, then the tets of each vertex in ascending
// order that were not listed yet (a tet is listed already iff it is t, a face neighbour, or
// holds one of the earlier vertices)
template <bool kFill>
__global__ void k_nbr_lists(int nt, const int32_t* __restrict__ T, const int32_t* __restrict__ nbr,
                            const int* __restrict__ ptr, const int32_t* __restrict__ n2t, int* __restrict__ cnt,
                            const int* __restrict__ out_ptr, int32_t* __restrict__ out) {
    const int64_t t = gid();
    if (t >= nt) return;
    int32_t v[4], fn[4];
    load4(T, t, v);
    load4(nbr, t, fn);
    int32_t* o = kFill ? out + out_ptr[t] : nullptr;
    int c = 0;
    for (int j = 0; j < 4; ++j)
        if (fn[j] >= 0) {
            if (kFill) o[c] = fn[j];
            ++c;
        }
    for (int k = 0; k < 4; ++k)
        for (int p = ptr[v[k]]; p < ptr[v[k] + 1]; ++p) {
            const int32_t u = n2t[p];
            if (u == t || u == fn[0] || u == fn[1] || u == fn[2] || u == fn[3]) continue;
            bool seen = false;
            if (k > 0) {
                int32_t w[4];
                load4(T, u, w);
                for (int kk = 0; kk < k && !seen; ++kk)
                    seen = w[0] == v[kk] || w[1] == v[kk] || w[2] == v[kk] || w[3] == v[kk];
            }
            if (seen) continue;
            if (kFill) o[c] = u;
            ++c;
        }
    if (!kFill) cnt[t] = c;
}

__global__ void k_tet_tables(int nt, int n_old, int ne, int nb, const int32_t* __restrict__ T,
                             const int32_t* __restrict__ tmarker, const double* __restrict__ X,
                             const uint64_t* __restrict__ ek, double* __restrict__ det, double* __restrict__ ctr,
                             int8_t* __restrict__ search, int32_t* __restrict__ quad, int* err) {
    const int64_t t = gid();
    if (t >= nt) return;
    int32_t v[4];
    load4(T, t, v);
    const mm::V3 p1{X[3 * (int64_t)v[0]], X[3 * (int64_t)v[0] + 1], X[3 * (int64_t)v[0] + 2]};
    const mm::V3 p2{X[3 * (int64_t)v[1]], X[3 * (int64_t)v[1] + 1], X[3 * (int64_t)v[1] + 2]};
    const mm::V3 p3{X[3 * (int64_t)v[2]], X[3 * (int64_t)v[2] + 1], X[3 * (int64_t)v[2] + 2]};
    const mm::V3 p4{X[3 * (int64_t)v[3]], X[3 * (int64_t)v[3] + 1], X[3 * (int64_t)v[3] + 2]};
    double d[kTetDetStride];
    mm::tet_det_table(p1, p2, p3, p4, d);
    for (int k = 0; k < kTetDetStride; ++k) det[kTetDetStride * t + k] = d[k];
    double cx = 0.0, cy = 0.0, cz = 0.0;
    for (int k = 0; k < 4; ++k) {
        cx += X[3 * (int64_t)v[k]];
        cy += X[3 * (int64_t)v[k] + 1];
        cz += X[3 * (int64_t)v[k] + 2];
    }
    ctr[3 * t] = cx * 0.25;
    ctr[3 * t + 1] = cy * 0.25;
    ctr[3 * t + 2] = cz * 0.25;
    search[t] = tmarker[t] == kVacuum ? 1 : 0;
    // quadratic tet: vertices, then the mid-edge nodes of edges 01, 12, 20, 03, 13, 23
    const int ea[6] = {0, 1, 2, 0, 1, 2}, eb[6] = {1, 2, 0, 3, 3, 3};
    for (int k = 0; k < 4; ++k) quad[10 * t + k] = v[k];
    for (int k = 0; k < 6; ++k) quad[10 * t + 4 + k] = n_old + edge_index(ek, ne, nb, v[ea[k]], v[eb[k]], err);
}

__global__ void k_hex_coeffs(int64_t nh, const int32_t* __restrict__ hexs, const double* __restrict__ xyz,
                             double* __restrict__ f) {
    const int64_t h = gid();
    if (h >= nh) return;
    const double* nodes[8];
    for (int k = 0; k < 8; ++k) nodes[k] = xyz + 3 * (int64_t)hexs[8 * h + k];
    double o[24];
    mm::hex_coefficients(nodes, o);
    for (int k = 0; k < 24; ++k) f[24 * h + k] = o[k];
}

__global__ void k_edgemax(int nt, const int32_t* __restrict__ T, const double* __restrict__ X,
                          unsigned long long* m) {
    const int64_t t = gid();
    if (t >= nt) return;
    int32_t v[4];
    load4(T, t, v);
    double best = 0.0;
    for (int i = 0; i < 4; ++i)
        for (int j = i + 1; j < 4; ++j) {
            const double dx = X[3 * (int64_t)v[i]] - X[3 * (int64_t)v[j]];
            const double dy = X[3 * (int64_t)v[i] + 1] - X[3 * (int64_t)v[j] + 1];
            const double dz = X[3 * (int64_t)v[i] + 2] - X[3 * (int64_t)v[j] + 2];
            const double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 > best) best = d2;
        }
    // non-negative doubles order like their bit patterns
    atomicMax(m, (unsigned long long)__double_as_longlong(best));
}

// ---------------------------------------------------------------- vacuum grouping
__global__ void k_vac_mark(int64_t nh, const int32_t* __restrict__ hm, const int32_t* __restrict__ hexs,
                           int* __restrict__ nflag, int* __restrict__ hflag) {
    const int64_t h = gid();
    if (h >= nh) return;
    const bool vac = hm[h] > 0;
    hflag[h] = vac ? 1 : 0;
    if (vac)
        for (int k = 0; k < 8; ++k) nflag[hexs[8 * h + k]] = 1;
}

__global__ void k_vac_nodes(int64_t nn, const int* __restrict__ flag, const int* __restrict__ pos,
                            int32_t* __restrict__ n2v, int32_t* __restrict__ v2n) {
    const int64_t i = gid();
    if (i >= nn) return;
    if (flag[i]) {
        n2v[i] = pos[i];
        v2n[pos[i]] = (int32_t)i;
    } else {
        n2v[i] = -1;
    }
}

__global__ void k_compact_index(int64_t n, const int* __restrict__ flag, const int* __restrict__ pos,
                                int32_t* __restrict__ out) {
    const int64_t i = gid();
    if (i < n && flag[i]) out[pos[i]] = (int32_t)i;
}

// pseudo-Voronoi stencil of tet vertex tn: the non-vertex nodes of its vacuum hexes, hexes in
// ascending order
template <bool kFill>
__global__ void k_voro(int n_old, const int* __restrict__ ptr, const int32_t* __restrict__ n2t,
                       const int32_t* __restrict__ T, const int32_t* __restrict__ hm, const int32_t* __restrict__ hexs,
                       const int8_t* __restrict__ nmarker, int* __restrict__ cnt, const int* __restrict__ out_ptr,
                       int32_t* __restrict__ out) {
    const int64_t tn = gid();
    if (tn >= n_old) return;
    int c = 0;
    for (int p = ptr[tn]; p < ptr[tn + 1]; ++p) {
        const int32_t t = n2t[p];
        int32_t v[4];
        load4(T, t, v);
        const int ver = v[0] == tn ? 0 : v[1] == tn ? 1 : v[2] == tn ? 2 : 3;
        const int64_t h = 4 * (int64_t)t + ver;
        if (hm[h] <= 0) continue;
        for (int k = 0; k < 8; ++k) {
            const int32_t nd = hexs[8 * h + k];
            if (nd != tn && nmarker[nd] >= kEdgeCentroid) {
                if (kFill) out[out_ptr[tn] + c] = nd;
                ++c;
            }
        }
    }
    if (!kFill) cnt[tn] = c;
}

__global__ void k_n2c_entries(int64_t nvc, const int32_t* __restrict__ cells, const int32_t* __restrict__ hexs,
                              uint32_t* __restrict__ keys, int32_t* __restrict__ vals, int* __restrict__ cnt) {
    const int64_t i = gid();
    if (i >= 8 * nvc) return;
    const int64_t h = cells[i >> 3];
    const int k = (int)(i & 7);
    const int32_t nd = hexs[8 * h + k];
    keys[i] = (uint32_t)nd;
    vals[i] = (int32_t)(8 * h + k);
    atomicAdd(&cnt[nd], 1);
}

void check_errors(const SBuf<int>& err, cudaStream_t s) {
    int h = 0;
    FGB_CUDA(cudaMemcpyAsync(&h, err.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
    FGB_CUDA(cudaStreamSynchronize(s));
    FGB_REQUIRE(!(h & kErrDegenerate), "degenerate tetrahedron");
    FGB_REQUIRE(!(h & kErrNonManifold), "non-manifold face shared by more than two tets");
    FGB_REQUIRE(!(h & kErrEdges), "tet vertex without three edges");
    FGB_REQUIRE(!(h & kErrLookup), "inconsistent edge or face tables");
}

template <typename T>
void upload(SBuf<T>& d, const std::vector<T>& h, cudaStream_t s) {
    if (!h.empty()) FGB_CUDA(cudaMemcpyAsync(d.get(), h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

}  // namespace

PreparedMesh prepare_mesh_device(TetMesh&& tm, cudaStream_t s, MeshPrepTiming* timing) {
    const auto w0 = std::chrono::steady_clock::now();
    FGB_REQUIRE(tm.n_tets() > 0 && tm.n_nodes() > 0, "empty mesh");
    FGB_REQUIRE(tm.marker.size() == (size_t)tm.n_tets(), "one marker per tet is required");
    for (int32_t v : tm.tets) FGB_REQUIRE(v >= 0 && v < tm.n_nodes(), "tet references a node out of range");
    const int n_old = tm.n_nodes(), nt = tm.n_tets();
    const int nb = bits_for((uint64_t)(n_old - 1));
    FGB_REQUIRE(3 * nb <= 63, "device mesh preparation supports up to 2^21 tet vertices");

    cudaEvent_t e0, e1;
    FGB_CUDA(cudaEventCreate(&e0));
    FGB_CUDA(cudaEventCreate(&e1));
    SBuf<double> X(3 * (size_t)n_old, s);
    SBuf<int32_t> T(4 * (size_t)nt, s), TM(nt, s);
    upload(X, tm.xyz, s);
    upload(T, tm.tets, s);
    upload(TM, tm.marker, s);
    FGB_CUDA(cudaEventRecord(e0, s));
    SBuf<int> err(1, s);
    err.fill_bytes(0);

    // ---- edges: sorted unique (max, min) vertex pairs
    const int64_t n6 = 6LL * nt, n4 = 4LL * nt;
    SBuf<uint64_t> ek(n6, s);
    FGB_LAUNCH(k_edge_keys<<<blocks(nt), kB, 0, s>>>(nt, T.get(), nb, ek.get(), err.get()));
    check_errors(err, s);
    radix_sort(ek, (SBuf<int32_t>*)nullptr, n6, 2 * nb, s);
    int ne = 0;
    SBuf<uint64_t> edges;
    {
        SBuf<int> flag(n6, s), pos(n6, s);
        FGB_LAUNCH(k_head_flags<<<blocks(n6), kB, 0, s>>>(n6, ek.get(), flag.get()));
        ne = exclusive_scan_total(flag.get(), pos.get(), n6, s);
        edges = SBuf<uint64_t>(ne, s);
        FGB_LAUNCH(k_compact_heads<<<blocks(n6), kB, 0, s>>>(n6, ek.get(), pos.get(), edges.get()));
    }
    ek = SBuf<uint64_t>();

    // ---- face neighbours, then face numbering by first encounter
    SBuf<int32_t> nbr(n4, s);
    nbr.fill_bytes(0xff);
    {
        SBuf<uint64_t> fk(n4, s);
        SBuf<int32_t> fs(n4, s);
        FGB_LAUNCH(k_face_keys<<<blocks(n4), kB, 0, s>>>(nt, T.get(), nb, fk.get(), fs.get()));
        radix_sort(fk, &fs, n4, 3 * nb, s);
        FGB_LAUNCH(k_face_pairs<<<blocks(n4), kB, 0, s>>>(n4, fk.get(), fs.get(), nbr.get(), err.get()));
    }
    check_errors(err, s);
    SBuf<int32_t> tet_face(n4, s);
    int nf = 0;
    SBuf<int32_t> fverts;
    {
        SBuf<int> cnt(nt, s), off(nt, s);
        FGB_LAUNCH(k_face_count<<<blocks(nt), kB, 0, s>>>(nt, nbr.get(), cnt.get()));
        nf = exclusive_scan_total(cnt.get(), off.get(), nt, s);
        fverts = SBuf<int32_t>(3 * (size_t)nf, s);
        FGB_LAUNCH(k_face_owned<<<blocks(nt), kB, 0, s>>>(nt, T.get(), nbr.get(), off.get(), tet_face.get(),
                                                           fverts.get()));
        FGB_LAUNCH(k_face_shared<<<blocks(nt), kB, 0, s>>>(nt, T.get(), nbr.get(), tet_face.get(), err.get()));
    }

    // ---- nodes and hexahedra
    const int64_t nn = (int64_t)n_old + ne + nf + nt, nh = 4LL * nt;
    FGB_REQUIRE(nn < INT32_MAX && 8 * nh < INT32_MAX, "mesh too large for 32-bit node and hex ids");
    SBuf<double> xyz(3 * nn, s);
    SBuf<int8_t> nmark(nn, s);
    SBuf<int32_t> par(4 * nn, s);
    FGB_LAUNCH(k_nodes<<<blocks(nn), kB, 0, s>>>(n_old, ne, nf, nt, nb, X.get(), edges.get(), fverts.get(), T.get(),
                                                  xyz.get(), nmark.get(), par.get()));
    SBuf<int32_t> hexs(8 * nh, s), hmark(nh, s);
    FGB_LAUNCH(k_hexes<<<blocks(nh), kB, 0, s>>>(nt, n_old, ne, nf, nb, T.get(), TM.get(), edges.get(),
                                                  tet_face.get(), xyz.get(), hexs.get(), hmark.get(), err.get()));

    // ---- node -> tets (ascending), location candidates, per-tet tables
    SBuf<int> tptr(n_old + 1, s);
    SBuf<int32_t> n2t;
    {
        SBuf<uint32_t> tk(n4, s);
        n2t = SBuf<int32_t>(n4, s);
        SBuf<int> cnt(n_old + 1, s);
        cnt.fill_bytes(0);
        FGB_LAUNCH(k_n2t_entries<<<blocks(n4), kB, 0, s>>>(nt, T.get(), tk.get(), n2t.get(), cnt.get()));
        radix_sort(tk, &n2t, n4, nb, s);
        exclusive_scan(cnt.get(), tptr.get(), n_old + 1, (int*)nullptr, s);
    }
    SBuf<int> nptr(nt + 1, s);
    int n_nbr = 0;
    SBuf<int32_t> nidx;
    {
        SBuf<int> cnt(nt + 1, s);
        cnt.fill_bytes(0);
        FGB_LAUNCH(k_nbr_lists<false><<<blocks(nt), kB, 0, s>>>(nt, T.get(), nbr.get(), tptr.get(), n2t.get(),
                                                                 cnt.get(), nullptr, nullptr));
        n_nbr = exclusive_scan_total(cnt.get(), nptr.get(), nt + 1, s);
        nidx = SBuf<int32_t>(n_nbr, s);
        FGB_LAUNCH(k_nbr_lists<true><<<blocks(nt), kB, 0, s>>>(nt, T.get(), nbr.get(), tptr.get(), n2t.get(),
                                                                nullptr, nptr.get(), nidx.get()));
    }
    SBuf<double> det((size_t)kTetDetStride * nt, s), ctr(3 * (size_t)nt, s);
    SBuf<int8_t> search(nt, s);
    SBuf<int32_t> quad(10 * (size_t)nt, s);
    FGB_LAUNCH(k_tet_tables<<<blocks(nt), kB, 0, s>>>(nt, n_old, ne, nb, T.get(), TM.get(), X.get(), edges.get(),
                                                       det.get(), ctr.get(), search.get(), quad.get(), err.get()));
    SBuf<double> hf(24 * nh, s);
    FGB_LAUNCH(k_hex_coeffs<<<blocks(nh), kB, 0, s>>>(nh, hexs.get(), xyz.get(), hf.get()));
    SBuf<unsigned long long> emax(1, s);
    emax.fill_bytes(0);
    FGB_LAUNCH(k_edgemax<<<blocks(nt), kB, 0, s>>>(nt, T.get(), X.get(), emax.get()));

    // ---- vacuum vertices and cells
    SBuf<int32_t> n2v(nn, s), v2n, cells;
    int nv = 0, nvc = 0;
    {
        SBuf<int> nflag(nn, s), npos(nn, s), hflag(nh, s), hpos(nh, s);
        nflag.fill_bytes(0);
        FGB_LAUNCH(k_vac_mark<<<blocks(nh), kB, 0, s>>>(nh, hmark.get(), hexs.get(), nflag.get(), hflag.get()));
        nv = exclusive_scan_total(nflag.get(), npos.get(), nn, s);
        v2n = SBuf<int32_t>(nv, s);
        FGB_LAUNCH(k_vac_nodes<<<blocks(nn), kB, 0, s>>>(nn, nflag.get(), npos.get(), n2v.get(), v2n.get()));
        nvc = exclusive_scan_total(hflag.get(), hpos.get(), nh, s);
        cells = SBuf<int32_t>(nvc, s);
        FGB_LAUNCH(k_compact_index<<<blocks(nh), kB, 0, s>>>(nh, hflag.get(), hpos.get(), cells.get()));
    }

    // ---- smoothing stencils of the tet vertices
    SBuf<int> vptr(n_old + 1, s);
    int n_voro = 0;
    SBuf<int32_t> vidx;
    {
        SBuf<int> cnt(n_old + 1, s);
        cnt.fill_bytes(0);
        FGB_LAUNCH(k_voro<false><<<blocks(n_old), kB, 0, s>>>(n_old, tptr.get(), n2t.get(), T.get(), hmark.get(),
                                                               hexs.get(), nmark.get(), cnt.get(), nullptr, nullptr));
        n_voro = exclusive_scan_total(cnt.get(), vptr.get(), n_old + 1, s);
        vidx = SBuf<int32_t>(n_voro, s);
        FGB_LAUNCH(k_voro<true><<<blocks(n_old), kB, 0, s>>>(n_old, tptr.get(), n2t.get(), T.get(), hmark.get(),
                                                              hexs.get(), nmark.get(), nullptr, vptr.get(), vidx.get()));
    }

    // ---- node -> (vacuum hex, local node), hexes ascending
    SBuf<int> cptr(nn + 1, s);
    const int64_t n8 = 8LL * nvc;
    SBuf<int32_t> citem(n8, s);
    {
        SBuf<uint32_t> ck(n8, s);
        SBuf<int> cnt(nn + 1, s);
        cnt.fill_bytes(0);
        FGB_LAUNCH(k_n2c_entries<<<blocks(n8), kB, 0, s>>>(nvc, cells.get(), hexs.get(), ck.get(), citem.get(),
                                                            cnt.get()));
        radix_sort(ck, &citem, n8, bits_for((uint64_t)(nn - 1)), s);
        exclusive_scan(cnt.get(), cptr.get(), nn + 1, (int*)nullptr, s);
    }
    FGB_CUDA(cudaEventRecord(e1, s));
    check_errors(err, s);
    float kms = 0;
    FGB_CUDA(cudaEventElapsedTime(&kms, e0, e1));

    // ---- download
    PreparedMesh pm;
    HexMesh& hm = pm.hex;
    hm.n_tetnodes = n_old;
    hm.n_edges = ne;
    hm.n_faces = nf;
    hm.n_tets = nt;
    xyz.to_host(hm.xyz, 3 * nn);
    nmark.to_host(hm.node_marker, nn);
    hexs.to_host(hm.hexs, 8 * nh);
    hmark.to_host(hm.hex_marker, nh);
    par.to_host(hm.parents, 4 * nn);
    nbr.to_host(pm.face_nbr, n4);
    det.to_host(pm.tt.det, (size_t)kTetDetStride * nt);
    ctr.to_host(pm.tt.centroid, 3 * (size_t)nt);
    search.to_host(pm.tt.search, nt);
    nptr.to_host(pm.tt.nbr_ptr, nt + 1);
    nidx.to_host(pm.tt.nbr_idx, n_nbr);
    quad.to_host(pm.tt.quad_nodes, 10 * (size_t)nt);
    hf.to_host(pm.hex_coeffs, 24 * nh);
    n2v.to_host(pm.vac.node2vertex, nn);
    v2n.to_host(pm.vac.vertex2node, nv);
    cells.to_host(pm.vac.cells, nvc);
    vptr.to_host(pm.voro_ptr, n_old + 1);
    vidx.to_host(pm.voro_idx, n_voro);
    cptr.to_host(pm.n2c_ptr, nn + 1);
    citem.to_host(pm.n2c_item, n8);
    unsigned long long em = 0;
    FGB_CUDA(cudaMemcpyAsync(&em, emax.get(), sizeof(em), cudaMemcpyDeviceToHost, s));
    FGB_CUDA(cudaStreamSynchronize(s));
    FGB_CUDA(cudaEventDestroy(e0));
    FGB_CUDA(cudaEventDestroy(e1));

    double m2;
    static_assert(sizeof(m2) == sizeof(em), "double is 64 bits");
    std::memcpy(&m2, &em, sizeof(m2));
    pm.edgemax = std::sqrt(m2);
    pm.decay_factor = -1.0 / pm.edgemax;
    for (int c = 0; c < 3; ++c) {
        pm.bbox_min[c] = 1e300;
        pm.bbox_max[c] = -1e300;
    }
    for (int i = 0; i < n_old; ++i)
        for (int c = 0; c < 3; ++c) {
            pm.bbox_min[c] = std::min(pm.bbox_min[c], tm.xyz[3 * (size_t)i + c]);
            pm.bbox_max[c] = std::max(pm.bbox_max[c], tm.xyz[3 * (size_t)i + c]);
        }
    pm.tet = std::move(tm);
    attach_interface_surface(pm);
    if (timing) {
        timing->kernel_ms = kms;
        timing->total_ms =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
    }
    return pm;
}

}  // namespace fgb
