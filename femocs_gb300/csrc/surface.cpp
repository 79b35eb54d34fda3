// Surface triangles and their location tables (see surface.h). Compiled with
// -ffp-contract=off: every product and sum is rounded on its own, in the reference's order.
#include "surface.h"

#include <cmath>

namespace fgb {

namespace {
struct D3 {
    double x, y, z;
};
inline D3 sub(const D3& a, const D3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 scale(const D3& a, double s) { return {a.x * s, a.y * s, a.z * s}; }
// Vec3::crossProduct / dotProduct (include/Primitives.h:307-313)
inline D3 cross(const D3& a, const D3& v) { return {a.y * v.z - a.z * v.y, a.z * v.x - a.x * v.z, a.x * v.y - a.y * v.x}; }
inline double dot(const D3& a, const D3& v) { return a.x * v.x + a.y * v.y + a.z * v.z; }
inline D3 node(const double* xyz, int32_t i) { return {xyz[3 * (size_t)i], xyz[3 * (size_t)i + 1], xyz[3 * (size_t)i + 2]}; }
}  // namespace

void interface_triangles(const std::vector<int32_t>& tets, const std::vector<int32_t>& marker,
                         const std::vector<int32_t>& face_nbr, const std::vector<double>& xyz,
                         std::vector<int32_t>& tris, std::vector<int32_t>& tri2tet) {
    tris.clear();
    tri2tet.clear();
    const int nt = (int)marker.size();
    for (int t = 0; t < nt; ++t) {
        if (marker[t] != kVacuum) continue;
        const int32_t* v = &tets[4 * (size_t)t];
        for (int j = 0; j < 4; ++j) {
            const int32_t u = face_nbr[4 * (size_t)t + j];
            if (u < 0 || marker[u] == kVacuum) continue;
            int32_t f[3], m = 0;
            for (int k = 0; k < 4; ++k)
                if (k != j) f[m++] = v[k];
            const D3 p0 = node(xyz.data(), f[0]);
            const D3 n = cross(sub(node(xyz.data(), f[1]), p0), sub(node(xyz.data(), f[2]), p0));
            if (dot(n, sub(node(xyz.data(), v[j]), p0)) < 0) std::swap(f[1], f[2]);
            tris.insert(tris.end(), f, f + 3);
            tri2tet.push_back(t);
            tri2tet.push_back(u);
        }
    }
}

SurfaceTables build_surface_tables(const double* xyz, int n_nodes, int n_tets, std::vector<int32_t> tris,
                                   std::vector<int32_t> tri2tet) {
    FGB_REQUIRE(tris.size() % 3 == 0 && tri2tet.size() == tris.size() / 3 * 2, "3 nodes and 2 tets per triangle");
    for (int32_t v : tris) FGB_REQUIRE(v >= 0 && v < n_nodes, "surface triangle node out of range");
    for (int32_t t : tri2tet) FGB_REQUIRE(t >= 0 && t < n_tets, "surface triangle needs two tets in range");
    SurfaceTables st;
    st.tris = std::move(tris);
    st.tri2tet = std::move(tri2tet);
    const int nf = st.n_tris();
    st.geo.resize((size_t)kTriGeoStride * nf);
    for (int f = 0; f < nf; ++f) {
        const D3 v0 = node(xyz, st.tris[3 * (size_t)f]);
        const D3 v1 = node(xyz, st.tris[3 * (size_t)f + 1]);
        const D3 v2 = node(xyz, st.tris[3 * (size_t)f + 2]);
        // TetgenFaces::calc_appendices: unit normal (Vec3::normalize) and centroid
        const D3 e1 = sub(v1, v0), e2 = sub(v2, v0);
        D3 nrm = cross(e1, e2);
        const double nn = std::sqrt(nrm.x * nrm.x + nrm.y * nrm.y + nrm.z * nrm.z);
        if (nn > 0) {
            const double factor = 1 / nn;
            nrm = scale(nrm, factor);
        }
        const D3 ctr = {(v0.x + v1.x + v2.x) / 3.0, (v0.y + v1.y + v2.y) / 3.0, (v0.z + v1.z + v2.z) / 3.0};
        // LinearTriangles::precompute
        const D3 pv = cross(nrm, e2);
        const double i_det = 1.0 / dot(e1, pv);
        const D3 e1d = scale(e1, i_det), pvd = scale(pv, i_det);
        double* g = &st.geo[(size_t)kTriGeoStride * f];
        const double vals[kTriGeoStride] = {v0.x,  v0.y,  v0.z,  e1d.x, e1d.y, e1d.z, e2.x,  e2.y,  e2.z, pvd.x,
                                            pvd.y, pvd.z, nrm.x, nrm.y, nrm.z, std::sqrt(e2.x * e2.x + e2.y * e2.y + e2.z * e2.z),
                                            ctr.x, ctr.y, ctr.z};
        for (int k = 0; k < kTriGeoStride; ++k) g[k] = vals[k];
    }
    // node -> triangles (ascending), then each triangle's candidate list
    std::vector<int32_t> cnt(n_nodes + 1, 0);
    for (int32_t v : st.tris) cnt[v + 1]++;
    for (int i = 0; i < n_nodes; ++i) cnt[i + 1] += cnt[i];
    std::vector<int32_t> n2t(cnt[n_nodes]);
    {
        std::vector<int32_t> pos(cnt.begin(), cnt.end() - 1);
        for (int f = 0; f < nf; ++f)
            for (int k = 0; k < 3; ++k) n2t[pos[st.tris[3 * (size_t)f + k]]++] = f;
    }
    st.nbr_ptr.assign(nf + 1, 0);
    for (int f = 0; f < nf; ++f) {
        for (int k = 0; k < 3; ++k) {
            const int32_t v = st.tris[3 * (size_t)f + k];
            for (int p = cnt[v]; p < cnt[v + 1]; ++p)
                if (n2t[p] != f) st.nbr_idx.push_back(n2t[p]);
        }
        st.nbr_ptr[f + 1] = (int32_t)st.nbr_idx.size();
    }
    return st;
}

}  // namespace fgb
