// Host construction of the Q1 FEM structure of the vacuum (field) or the bulk (current/heat)
// hexahedra.
//
// DoF numbering: the reference lets deal.II number DoFs (DoFHandler::distribute_dofs) and
// maps them back to mesh vertices (src/DealSolver.cpp:318-341); only the per-vertex
// solution is observable. Here the vacuum vertices are ordered along a Morton curve and,
// inside windows of 256 rows, by decreasing row length, so that (a) rows close in index are
// close in space (the SpMV gathers hit cache) and (b) each 32-row SELL slice holds rows of
// similar length (little padding).
#include "fem.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <parallel/algorithm>

namespace fgb {

namespace {

inline uint64_t spread3(uint64_t v) {
    v &= 0x1fffff;
    v = (v | v << 32) & 0x1f00000000ffffull;
    v = (v | v << 16) & 0x1f0000ff0000ffull;
    v = (v | v << 8) & 0x100f00f00f00f00full;
    v = (v | v << 4) & 0x10c30c30c30c30c3ull;
    v = (v | v << 2) & 0x1249249249249249ull;
    return v;
}

// the six faces of a femocs-ordered hex, vertices in cyclic order
const int kHexFace[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}, {0, 1, 5, 4}, {3, 2, 6, 7}};

struct BFace {
    int32_t s[4];  // sorted dofs
    int32_t cell;
    int8_t face;
};

}  // namespace

RegionCells region_cells(const PreparedMesh& pm, int region) {
    if (region == kRegionVacuum) return {pm.vac.cells, pm.vac.node2vertex, pm.vac.vertex2node};
    FGB_REQUIRE(region == kRegionBulk, "region must be vacuum or bulk");
    RegionCells rc;
    rc.node2vertex.assign(pm.hex.n_nodes(), -1);
    for (int h = 0; h < pm.hex.n_hexs(); ++h)
        if (pm.hex.hex_marker[h] < 0) {
            rc.cells.push_back(h);
            for (int k = 0; k < 8; ++k) rc.node2vertex[pm.hex.hexs[8 * (size_t)h + k]] = -2;
        }
    for (int i = 0; i < pm.hex.n_nodes(); ++i)
        if (rc.node2vertex[i] == -2) {
            rc.node2vertex[i] = (int32_t)rc.vertex2node.size();
            rc.vertex2node.push_back(i);
        }
    return rc;
}

FemStructure build_fem_structure(const PreparedMesh& pm, int region) {
    FemStructure fs;
    SetupPhases phase("q1 structure");
    const RegionCells rcs = region_cells(pm, region);
    const int nv = (int)rcs.vertex2node.size();
    const int nc = (int)rcs.cells.size();
    FGB_REQUIRE(nv > 0 && nc > 0, region == kRegionBulk ? "mesh has no bulk hexahedra" : "mesh has no vacuum hexahedra");
    fs.n_dofs = nv;
    fs.n_cells = nc;
    fs.region = region;
    const std::vector<double>& X = pm.hex.xyz;

    // cells in vertex numbering
    std::vector<int32_t> cv(8 * (size_t)nc);
    for (int c = 0; c < nc; ++c)
        for (int k = 0; k < 8; ++k)
            cv[8 * (size_t)c + k] = rcs.node2vertex[pm.hex.hexs[8 * (size_t)rcs.cells[c] + k]];

    phase("region, cells");
    // vertex -> cells
    std::vector<int32_t> v2c_ptr(nv + 1, 0);
    for (int32_t v : cv) v2c_ptr[v + 1]++;
    for (int i = 0; i < nv; ++i) v2c_ptr[i + 1] += v2c_ptr[i];
    std::vector<int32_t> v2c(v2c_ptr[nv]);
    {
        std::vector<int32_t> pos(v2c_ptr.begin(), v2c_ptr.end() - 1);
        for (int c = 0; c < nc; ++c)
            for (int k = 0; k < 8; ++k) v2c[pos[cv[8 * (size_t)c + k]]++] = 8 * c + k;
    }

    phase("vertex -> cells");
    // neighbour sets (vertex numbering) and degrees, as one flat array: the sorted, unique
    // vertices of each vertex's cells, counted in a first pass and written in a second
    std::vector<int32_t> deg(nv);
    auto neighbours = [&](int v, std::vector<int32_t>& l) {
        l.clear();
        for (int p = v2c_ptr[v]; p < v2c_ptr[v + 1]; ++p) {
            const int c = v2c[p] / 8;
            for (int k = 0; k < 8; ++k) l.push_back(cv[8 * (size_t)c + k]);
        }
        std::sort(l.begin(), l.end());
        l.erase(std::unique(l.begin(), l.end()), l.end());
    };
#pragma omp parallel
    {
        std::vector<int32_t> l;
#pragma omp for schedule(dynamic, 1024)
        for (int v = 0; v < nv; ++v) {
            neighbours(v, l);
            deg[v] = (int32_t)l.size();
        }
    }
    std::vector<int64_t> nb_ptr(nv + 1, 0);
    for (int v = 0; v < nv; ++v) nb_ptr[v + 1] = nb_ptr[v] + deg[v];
    std::vector<int32_t> nb_col(nb_ptr[nv]);
#pragma omp parallel
    {
        std::vector<int32_t> l;
#pragma omp for schedule(dynamic, 1024)
        for (int v = 0; v < nv; ++v) {
            neighbours(v, l);
            std::copy(l.begin(), l.end(), nb_col.begin() + nb_ptr[v]);
        }
    }

    phase("neighbour sets");
    // Morton order, then windows of 256 sorted by decreasing degree
    double mn0 = 1e300, mn1 = 1e300, mn2 = 1e300, mx0 = -1e300, mx1 = -1e300, mx2 = -1e300;
#pragma omp parallel for schedule(static) reduction(min : mn0, mn1, mn2) reduction(max : mx0, mx1, mx2)
    for (int v = 0; v < nv; ++v) {
        const double* p = &X[3 * (size_t)rcs.vertex2node[v]];
        mn0 = std::min(mn0, p[0]);
        mn1 = std::min(mn1, p[1]);
        mn2 = std::min(mn2, p[2]);
        mx0 = std::max(mx0, p[0]);
        mx1 = std::max(mx1, p[1]);
        mx2 = std::max(mx2, p[2]);
    }
    const double mn[3] = {mn0, mn1, mn2}, mx[3] = {mx0, mx1, mx2};
    std::vector<std::pair<uint64_t, int32_t>> key(nv);
#pragma omp parallel for schedule(static)
    for (int v = 0; v < nv; ++v) {
        uint64_t code = 0;
        for (int c = 0; c < 3; ++c) {
            const double span = mx[c] > mn[c] ? mx[c] - mn[c] : 1.0;
            double t = (X[3 * (size_t)rcs.vertex2node[v] + c] - mn[c]) / span;
            uint64_t q = (uint64_t)std::min(2097151.0, std::max(0.0, std::floor(t * 2097151.0)));
            code |= spread3(q) << c;
        }
        key[v] = {code, v};
    }
    __gnu_parallel::sort(key.begin(), key.end());
    std::vector<int32_t> dof2v(nv);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nv; ++i) dof2v[i] = key[i].second;
    const int W = 256;
#pragma omp parallel for schedule(dynamic, 64)
    for (int w0 = 0; w0 < nv; w0 += W) {
        const int w1 = std::min(nv, w0 + W);
        std::stable_sort(dof2v.begin() + w0, dof2v.begin() + w1,
                         [&](int32_t a, int32_t b) { return deg[a] > deg[b]; });
    }
    std::vector<int32_t> v2dof(nv);
    for (int d = 0; d < nv; ++d) v2dof[dof2v[d]] = d;

    phase("Morton order, windows");
    fs.dof2node.resize(nv);
    fs.node2dof.assign(pm.hex.n_nodes(), -1);
    for (int d = 0; d < nv; ++d) {
        fs.dof2node[d] = rcs.vertex2node[dof2v[d]];
        fs.node2dof[fs.dof2node[d]] = d;
    }
    fs.cell_dofs.resize(8 * (size_t)nc);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)cv.size(); ++i) fs.cell_dofs[i] = v2dof[cv[i]];

    // CSR in dof numbering
    fs.rowptr.assign(nv + 1, 0);
    fs.row_len.resize(nv);
    for (int d = 0; d < nv; ++d) {
        fs.row_len[d] = deg[dof2v[d]];
        fs.rowptr[d + 1] = fs.rowptr[d] + fs.row_len[d];
    }
    fs.col.resize(fs.rowptr[nv]);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int d = 0; d < nv; ++d) {
        const int v = dof2v[d];
        const int64_t b = nb_ptr[v], len = nb_ptr[v + 1] - b;
        int32_t* o = &fs.col[fs.rowptr[d]];
        for (int64_t k = 0; k < len; ++k) o[k] = v2dof[nb_col[b + k]];
        std::sort(o, o + len);
    }
    std::vector<int32_t>().swap(nb_col);

    phase("CSR columns");
    // row -> (cell, local), ascending cell
    fs.r2c_ptr.assign(nv + 1, 0);
    for (int d = 0; d < nv; ++d) fs.r2c_ptr[d + 1] = fs.r2c_ptr[d] + (v2c_ptr[dof2v[d] + 1] - v2c_ptr[dof2v[d]]);
    fs.r2c_item.resize(fs.r2c_ptr[nv]);
#pragma omp parallel for schedule(static)
    for (int d = 0; d < nv; ++d) {
        const int v = dof2v[d];
        std::copy(v2c.begin() + v2c_ptr[v], v2c.begin() + v2c_ptr[v + 1], fs.r2c_item.begin() + fs.r2c_ptr[d]);
    }

    phase("row -> cells");
    // ---- boundary faces (src/DealSolver.cpp:461-518 via PoissonSolver::mark_mesh)
    std::vector<BFace> faces(6 * (size_t)nc);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nc; ++c)
        for (int f = 0; f < 6; ++f) {
            BFace& b = faces[6 * (size_t)c + f];
            for (int q = 0; q < 4; ++q) b.s[q] = fs.cell_dofs[8 * (size_t)c + kHexFace[f][q]];
            std::sort(b.s, b.s + 4);
            b.cell = c;
            b.face = (int8_t)f;
        }
    // sorted by (corner DoFs, cell): buckets by the smallest corner DoF (atomic counts and
    // cursors), then each bucket by the full key; the order is total, so the result is the
    // comparison sort's at any thread count
    {
        auto face_less = [](const BFace& a, const BFace& b) {
            for (int k = 0; k < 4; ++k)
                if (a.s[k] != b.s[k]) return a.s[k] < b.s[k];
            return a.cell < b.cell;
        };
        const long long nf = (long long)faces.size();
        std::vector<int32_t> bstart(nv + 1, 0);
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < nf; ++i) __atomic_fetch_add(&bstart[faces[i].s[0] + 1], 1, __ATOMIC_RELAXED);
        for (int v = 0; v < nv; ++v) bstart[v + 1] += bstart[v];
        std::vector<int32_t> cur(bstart.begin(), bstart.end() - 1);
        std::vector<BFace> sorted(faces.size());
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < nf; ++i) sorted[__atomic_fetch_add(&cur[faces[i].s[0]], 1, __ATOMIC_RELAXED)] = faces[i];
#pragma omp parallel for schedule(dynamic, 2048)
        for (int v = 0; v < nv; ++v) std::sort(sorted.begin() + bstart[v], sorted.begin() + bstart[v + 1], face_less);
        faces.swap(sorted);
    }
    std::vector<BFace> bnd;
    for (size_t i = 0; i < faces.size();) {
        size_t j = i + 1;
        while (j < faces.size() && std::equal(faces[j].s, faces[j].s + 4, faces[i].s)) ++j;
        if (j - i == 1) bnd.push_back(faces[i]);
        i = j;
    }
    faces.clear();
    faces.shrink_to_fit();
    // vacuum: (cell, face) order; bulk: the reference's per-face order of the boundary values,
    // cells ascending and deal.II faces x-, x+, y-, y+, z-, z+ (kHexFace 2, 3, 0, 1, 4, 5)
    static const int kDealRank[6] = {2, 3, 0, 1, 4, 5};
    std::sort(bnd.begin(), bnd.end(), [&](const BFace& a, const BFace& b) {
        if (a.cell != b.cell) return a.cell < b.cell;
        return region == kRegionBulk ? kDealRank[a.face] < kDealRank[b.face] : a.face < b.face;
    });
    auto dof_x = [&](int32_t d, int c) { return X[3 * (size_t)fs.dof2node[d] + c]; };
    double bmn[3] = {1e16, 1e16, 1e16}, bmx[3] = {-1e16, -1e16, -1e16};
    std::vector<double> ctr(3 * bnd.size());
    for (size_t i = 0; i < bnd.size(); ++i) {
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int q = 0; q < 4; ++q) s += dof_x(fs.cell_dofs[8 * (size_t)bnd[i].cell + kHexFace[bnd[i].face][q]], c);
            ctr[3 * i + c] = s / 4.0;
            bmn[c] = std::min(bmn[c], ctr[3 * i + c]);
            bmx[c] = std::max(bmx[c], ctr[3 * i + c]);
        }
    }
    const double eps = 1e-6;
    fs.bc_kind.assign(nv, 0);
    std::vector<int32_t> top;
    for (size_t i = 0; i < bnd.size(); ++i) {
        const double x = ctr[3 * i], y = ctr[3 * i + 1], z = ctr[3 * i + 2];
        const bool side = std::fabs(x - bmn[0]) <= eps || std::fabs(x - bmx[0]) <= eps ||
                          std::fabs(y - bmn[1]) <= eps || std::fabs(y - bmx[1]) <= eps;
        if (side) continue;
        int32_t fd[4];
        for (int q = 0; q < 4; ++q) fd[q] = fs.cell_dofs[8 * (size_t)bnd[i].cell + kHexFace[bnd[i].face][q]];
        // vacuum (PoissonSolver::mark_mesh): z max -> top (Neumann), the rest -> copper (phi = 0);
        // bulk (CurrentHeatSolver::mark_mesh, src/CurrentHeatSolver.cpp:535-539): z min -> copper
        // bottom (Dirichlet), z max and the rest -> copper surface (Neumann, per-face values)
        const bool neumann = region == kRegionBulk ? !(std::fabs(z - bmn[2]) <= eps) : std::fabs(z - bmx[2]) <= eps;
        if (neumann) {
            top.insert(top.end(), fd, fd + 4);
            fs.top_face_cells.push_back(bnd[i].cell);
            fs.top_face_local.push_back(bnd[i].face);
        } else {
            for (int q = 0; q < 4; ++q) fs.bc_kind[fd[q]] = 1;
        }
    }
    fs.top_faces = top;
    for (int32_t d : top)
        if (fs.bc_kind[d] == 0) fs.bc_kind[d] = 2;
    const int nt = fs.n_top_faces();
    fs.r2f_ptr.assign(nv + 1, 0);
    for (int32_t d : top) fs.r2f_ptr[d + 1]++;
    for (int i = 0; i < nv; ++i) fs.r2f_ptr[i + 1] += fs.r2f_ptr[i];
    fs.r2f_item.resize(fs.r2f_ptr[nv]);
    {
        std::vector<int32_t> pos(fs.r2f_ptr.begin(), fs.r2f_ptr.end() - 1);
        for (int f = 0; f < nt; ++f)
            for (int q = 0; q < 4; ++q) fs.r2f_item[pos[top[4 * (size_t)f + q]]++] = 4 * f + q;
    }

    phase("boundary faces");
    // ---- SELL-32 with 4-wide row chunks: slice s holds rows 32s..32s+31, padded to a length
    // that is a multiple of 4; entry j of lane l sits at ptr[s] + ((j/4)*32 + l)*4 + j%4, so a
    // warp reads 32 x 16 contiguous bytes of values (and of columns) per chunk
    const int C = 32, W4 = 4;
    const int ns = (nv + C - 1) / C;
    fs.slice_ptr.assign(ns + 1, 0);
    fs.slice_len.assign(ns, 0);
    for (int s = 0; s < ns; ++s) {
        int m = 0;
        for (int r = s * C; r < std::min(nv, (s + 1) * C); ++r) m = std::max(m, fs.row_len[r]);
        m = (m + W4 - 1) / W4 * W4;
        fs.slice_len[s] = m;
        fs.slice_ptr[s + 1] = fs.slice_ptr[s] + (int64_t)m * C;
    }
    fs.sell_col.assign(fs.slice_ptr[ns], 0);
    fs.csr2sell.resize(fs.nnz());
#pragma omp parallel for schedule(dynamic, 256)
    for (int s = 0; s < ns; ++s)
        for (int lane = 0; lane < C; ++lane) {
            const int r = s * C + lane;
            for (int j = 0; j < fs.slice_len[s]; ++j) {
                const int64_t pos = fs.slice_ptr[s] + ((int64_t)(j / W4) * C + lane) * W4 + j % W4;
                if (r < nv && j < fs.row_len[r]) {
                    fs.sell_col[pos] = fs.col[fs.rowptr[r] + j];
                    fs.csr2sell[fs.rowptr[r] + j] = pos;
                } else {
                    fs.sell_col[pos] = r < nv ? r : 0;
                }
            }
        }
    phase("SELL layout");
    return fs;
}

}  // namespace fgb
