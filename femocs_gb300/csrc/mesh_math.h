// Arithmetic of the mesh preparation shared by the host builder (mesh.cpp, compiled with
// -ffp-contract=off) and the device builder (mesh_prep_exact.cu, compiled with -fmad=false):
// one definition, one IEEE operation sequence, so both produce the same bits.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define FGB_HD __host__ __device__ __forceinline__
#else
#define FGB_HD inline
#endif

namespace fgb {
namespace mm {

// Local edges of a tet in the order the reference enumerates them (src/Tethex.cpp:1244-1262):
// all ordered pairs (i, j) of local vertices with v[i] > v[j], i outer, j inner.
struct LocalEdges {
    int n;
    int a[6], b[6];  // local vertex indices, v[a] > v[b]
};
FGB_HD LocalEdges local_edges(const int32_t* v) {
    LocalEdges le;
    le.n = 0;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            if (v[i] > v[j]) {
                le.a[le.n] = i;
                le.b[le.n] = j;
                ++le.n;
            }
    return le;
}

// sign of the trilinear-hex volume for vertices given in deal.II lexicographic order,
// from the Jacobian at the cell centre (sufficient for the convex tet corners produced here)
FGB_HD double hex_orientation(const double* d) {
    double ex[3], ey[3], ez[3];
    for (int c = 0; c < 3; ++c) {
        ex[c] = (d[3 * 1 + c] - d[3 * 0 + c]) + (d[3 * 3 + c] - d[3 * 2 + c]) +
                (d[3 * 5 + c] - d[3 * 4 + c]) + (d[3 * 7 + c] - d[3 * 6 + c]);
        ey[c] = (d[3 * 2 + c] - d[3 * 0 + c]) + (d[3 * 3 + c] - d[3 * 1 + c]) +
                (d[3 * 6 + c] - d[3 * 4 + c]) + (d[3 * 7 + c] - d[3 * 5 + c]);
        ez[c] = (d[3 * 4 + c] - d[3 * 0 + c]) + (d[3 * 5 + c] - d[3 * 1 + c]) +
                (d[3 * 6 + c] - d[3 * 2 + c]) + (d[3 * 7 + c] - d[3 * 3 + c]);
    }
    return ex[0] * (ey[1] * ez[2] - ey[2] * ez[1]) - ex[1] * (ey[0] * ez[2] - ey[2] * ez[0]) +
           ex[2] * (ey[0] * ez[1] - ey[1] * ez[0]);
}

// position of femocs hex vertex i in the deal.II lexicographic order used by hex_orientation
FGB_HD int to_deal(int i) {
    switch (i) {
        case 0: return 0;
        case 1: return 1;
        case 2: return 5;
        case 3: return 4;
        case 4: return 2;
        case 5: return 3;
        case 6: return 7;
        default: return 6;
    }
}

struct V3 {
    double x, y, z;
};

// 2x3 "determinant" helper of the barycentric minors: a.x*(b.y-b.z) - a.y*(b.x-b.z) + a.z*(b.x-b.y)
FGB_HD double minor2(const V3& a, const V3& b) { return a.x * (b.y - b.z) - a.y * (b.x - b.z) + a.z * (b.x - b.y); }
FGB_HD double minor3(const V3& a, const V3& b, const V3& c) {
    return a.x * (b.y * c.z - c.y * b.z) - b.x * (a.y * c.z - c.y * a.z) + c.x * (a.y * b.z - b.y * a.z);
}
// |x y z 1| determinant of four points, expanded along the column of ones
FGB_HD double det4(const V3& p1, const V3& p2, const V3& p3, const V3& p4) {
    const double a = minor3(p2, p3, p4);
    const double b = minor3(p1, p3, p4);
    const double c = minor3(p1, p2, p4);
    const double d = minor3(p1, p2, p3);
    return d - c + b - a;
}
// Minor vector of the barycentric coordinate that replaces point `skip` by (x,y,z,1);
// `sgn` = +1 for coordinates 1 and 3, -1 for 2 and 4.
// The 3x3 minor of the last coordinate is evaluated on the transposed vectors for the first
// three coordinates and on the points themselves for the fourth, as the reference does
// (src/InterpolatorCells.cpp:586-626); both are the same determinant but round differently.
FGB_HD void bary_minor(const V3& p, const V3& q, const V3& r, int sgn, bool rows, double* out) {
    const double m1 = minor2({p.y, q.y, r.y}, {p.z, q.z, r.z});
    const double m2 = minor2({p.x, q.x, r.x}, {p.z, q.z, r.z});
    const double m3 = minor2({p.x, q.x, r.x}, {p.y, q.y, r.y});
    const double m4 = rows ? minor3(p, q, r) : minor3({p.x, q.x, r.x}, {p.y, q.y, r.y}, {p.z, q.z, r.z});
    if (sgn > 0) {
        out[0] = m1; out[1] = -m2; out[2] = m3; out[3] = -m4;
    } else {
        out[0] = -m1; out[1] = m2; out[2] = -m3; out[3] = m4;
    }
}

// The 17 location doubles of a tet with corners p1..p4: 1/D, then the four minor vectors.
FGB_HD void tet_det_table(const V3& p1, const V3& p2, const V3& p3, const V3& p4, double* d) {
    d[0] = 1.0 / det4(p1, p2, p3, p4);
    bary_minor(p2, p3, p4, +1, false, d + 1);
    bary_minor(p1, p3, p4, -1, false, d + 5);
    bary_minor(p1, p2, p4, +1, false, d + 9);
    bary_minor(p1, p2, p3, -1, true, d + 13);
}

// Sign of hex node k in trilinear coefficient f_r (rows 1, x, y, z, xy, xz, yz, xyz of the
// expansion over the femocs vertex signs hx = -+ +- -+ +-, hy = --++--++, hz = ----++++).
FGB_HD int trilinear_sign(int r, int k) {
    const int hx = ((k ^ (k >> 1)) & 1) ? 1 : -1;
    const int hy = (k & 2) ? 1 : -1;
    const int hz = (k & 4) ? 1 : -1;
    switch (r) {
        case 0: return 1;
        case 1: return hx;
        case 2: return hy;
        case 3: return hz;
        case 4: return hx * hy;
        case 5: return hx * hz;
        case 6: return hy * hz;
        default: return hx * hy * hz;
    }
}

// Trilinear map coefficients f0..f7 (3 doubles each) of a hex from its 8 node positions:
// left-to-right signed sum starting from the first node, then /8.
FGB_HD void hex_coefficients(const double* const nodes[8], double* f) {
    for (int r = 0; r < 8; ++r)
        for (int c = 0; c < 3; ++c) {
            double s = nodes[0][c] * (double)trilinear_sign(r, 0);
            for (int k = 1; k < 8; ++k) {
                const double x = nodes[k][c];
                s = trilinear_sign(r, k) > 0 ? s + x : s - x;
            }
            f[3 * r + c] = s / 8.0;
        }
}

}  // namespace mm
}  // namespace fgb
