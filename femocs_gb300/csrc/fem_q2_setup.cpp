// Host construction of the Q2 (27-node hexahedron) structure on the vacuum hexes.
//
// The reference solves with Q1 elements only (DealSolver<3> builds FE_Q<3>(1), its Q2 path
// is absent: include/DealSolver.h:130); this is the higher-order element of the same mesh,
// same boundary marking (src/DealSolver.cpp:461-518) and same vertex hand-off to the
// interpolator: a Q2 DoF sits on every vacuum vertex, hex edge, hex face and hex interior;
// vertex DoFs carry phi at the mesh nodes. Numbering: Morton order of the DoF positions, then
// windows of 256 rows by decreasing row length (as the Q1 structure).
#include "fem.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <numeric>
#include <parallel/algorithm>

#include <omp.h>

namespace fgb {

namespace {

const int kHx[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
const int kHy[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
const int kHz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};

inline uint64_t spread3q(uint64_t v) {
    v &= 0x1fffff;
    v = (v | v << 32) & 0x1f00000000ffffull;
    v = (v | v << 16) & 0x1f0000ff0000ffull;
    v = (v | v << 8) & 0x100f00f00f00f00full;
    v = (v | v << 4) & 0x10c30c30c30c30c3ull;
    v = (v | v << 2) & 0x1249249249249249ull;
    return v;
}

// lattice corners of the entity that local node L belongs to (1, 2, 4 or 8 corners)
int corners_of(int L, int out[8]) {
    int a, b, c;
    q2_lattice(L, a, b, c);
    const int ra[2] = {a == 1 ? 0 : a, a == 1 ? 2 : a};
    const int rb[2] = {b == 1 ? 0 : b, b == 1 ? 2 : b};
    const int rc[2] = {c == 1 ? 0 : c, c == 1 ? 2 : c};
    int n = 0;
    for (int k = 0; k < (c == 1 ? 2 : 1); ++k)
        for (int j = 0; j < (b == 1 ? 2 : 1); ++j)
            for (int i = 0; i < (a == 1 ? 2 : 1); ++i) out[n++] = q2_corner_vertex(ra[i], rb[j], rc[k]);
    return n;
}

struct EntityKey {
    std::array<int32_t, 4> k;  // sorted global node ids of the entity's corners (unused: INT32_MAX)
    int32_t cell;
    int8_t local;
    bool operator<(const EntityKey& o) const { return k != o.k ? k < o.k : cell < o.cell; }
};

}  // namespace

int q2_entity_corners(int L, int out[8]) { return corners_of(L, out); }

int q2_corner_vertex(int a, int b, int c) {
    for (int k = 0; k < 8; ++k)
        if (kHx[k] + 1 == a && kHy[k] + 1 == b && kHz[k] + 1 == c) return k;
    return -1;
}

FemStructure build_q2_structure(const PreparedMesh& pm, bool sell_columns) {
    FemStructure fs;
    SetupPhases phase("q2 structure");
    fs.order = 2;
    fs.npc = 27;
    fs.nfc = 9;
    const int nc = (int)pm.vac.cells.size();
    const int nvx = (int)pm.vac.vertex2node.size();
    FGB_REQUIRE(nvx > 0 && nc > 0, "mesh has no vacuum hexahedra");
    fs.n_cells = nc;
    const std::vector<double>& X = pm.hex.xyz;
    auto cell_node = [&](int c, int k) { return pm.hex.hexs[8 * (size_t)pm.vac.cells[c] + k]; };

    // ---- entities: vertices by compact vertex index, edges/faces by sorted corner nodes,
    // interiors by cell
    std::vector<int32_t> ent(27 * (size_t)nc, -1);  // entity id per (cell, L)
    // 12 edges and 6 faces per cell, at fixed slots so that cells fill in parallel
    int slot_of[27], n_corner[27], corner_tab[27][8];
    {
        int k = 0;
        for (int L = 0; L < 27; ++L) {
            n_corner[L] = corners_of(L, corner_tab[L]);
            slot_of[L] = (n_corner[L] == 2 || n_corner[L] == 4) ? k++ : -1;
        }
        FGB_REQUIRE(k == 18, "Q2 lattice: 12 edges and 6 faces per cell");
    }
    std::vector<EntityKey> ek(18 * (size_t)nc);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nc; ++c) {
        int32_t cn[8];  // the cell's corner nodes, read once
        for (int k = 0; k < 8; ++k) cn[k] = cell_node(c, k);
        for (int L = 0; L < 27; ++L) {
            const int n = n_corner[L];
            if (n == 1) {
                ent[27 * (size_t)c + L] = pm.vac.node2vertex[cn[corner_tab[L][0]]];
            } else if (n == 2 || n == 4) {
                EntityKey& e = ek[18 * (size_t)c + slot_of[L]];
                int32_t k[4] = {INT32_MAX, INT32_MAX, INT32_MAX, INT32_MAX};
                for (int q = 0; q < n; ++q) k[q] = cn[corner_tab[L][q]];
                // four keys in ascending order (a five-exchange sorting network)
                auto cx = [&](int a, int b) {
                    if (k[b] < k[a]) std::swap(k[a], k[b]);
                };
                cx(0, 1);
                cx(2, 3);
                cx(0, 2);
                cx(1, 3);
                cx(1, 2);
                e.k = {k[0], k[1], k[2], k[3]};
                e.cell = c;
                e.local = (int8_t)L;
            }
        }
    }
    phase("entity keys");
    // sort by (corner nodes, cell): buckets by the smallest corner node (atomic counts and
    // cursors), then each bucket by the full key. The order is total (a cell has one record
    // per entity), so the result is the comparison sort's at any thread count.
    {
        const size_t ne0 = ek.size();
        const int n_nodes = (int)(X.size() / 3);
        FGB_REQUIRE(ne0 < (size_t)INT32_MAX, "Q2 structure: too many edge and face records");
        std::vector<int32_t> bstart(n_nodes + 1, 0);
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < (long long)ne0; ++i) __atomic_fetch_add(&bstart[ek[i].k[0] + 1], 1, __ATOMIC_RELAXED);
        for (int v = 0; v < n_nodes; ++v) bstart[v + 1] += bstart[v];
        std::vector<int32_t> cur(bstart.begin(), bstart.end() - 1);
        std::vector<EntityKey> sorted(ne0);
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < (long long)ne0; ++i)
            sorted[__atomic_fetch_add(&cur[ek[i].k[0]], 1, __ATOMIC_RELAXED)] = ek[i];
#pragma omp parallel for schedule(dynamic, 2048)
        for (int v = 0; v < n_nodes; ++v) std::sort(sorted.begin() + bstart[v], sorted.begin() + bstart[v + 1]);
        ek.swap(sorted);
    }
    phase("entity sort");
    // runs of equal keys in the sorted list are one entity each, numbered in order: run heads
    // flagged and counted per thread block of the list, an exclusive scan over the blocks, then
    // each record takes its run's id (the numbering of a sequential pass, in parallel)
    const size_t ne = ek.size();
    std::vector<int32_t> run_id(ne);
    int n_shared = 0;
    {
        const int nt = std::max(1, omp_get_max_threads());
        std::vector<int64_t> heads(nt + 1, 0);
#pragma omp parallel num_threads(nt)
        {
            const int t = omp_get_thread_num();
            const size_t a0 = ne * t / nt, a1 = ne * (t + 1) / nt;
            int64_t h = 0;
            for (size_t i = a0; i < a1; ++i) h += (i == 0 || !(ek[i].k == ek[i - 1].k));
            heads[t + 1] = h;
#pragma omp barrier
#pragma omp single
            for (int u = 0; u < nt; ++u) heads[u + 1] += heads[u];
            int64_t id = heads[t] - 1;
            for (size_t i = a0; i < a1; ++i) {
                if (i == 0 || !(ek[i].k == ek[i - 1].k)) ++id;
                run_id[i] = (int32_t)id;
            }
        }
        n_shared = (int)heads[nt];
    }
    std::vector<int32_t> face_count(n_shared);  // occurrences of each face entity (boundary faces: 1)
    std::vector<int32_t> ent_first(n_shared);   // first (cell, L) of each shared entity
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)ne; ++i) {
        const int r = run_id[i];
        ent[27 * (size_t)ek[i].cell + ek[i].local] = nvx + r;
        if (i == 0 || run_id[i - 1] != r) {
            size_t j = i + 1;
            while (j < ne && run_id[j] == r) ++j;
            face_count[r] = ek[i].k[2] == INT32_MAX ? 0 : (int32_t)(j - i);
            ent_first[r] = 27 * ek[i].cell + ek[i].local;
        }
    }
    const int n_ent = nvx + n_shared + nc;
    for (int c = 0; c < nc; ++c) ent[27 * (size_t)c + 13] = nvx + n_shared + c;
    fs.n_dofs = n_ent;

    phase("entity ids");
    // entity -> cells: the (cell, L) items of each entity in ascending item order, entities in
    // id order (vertices, edges and faces, interiors). Vertices: a counting sort of the 8 corner
    // items per cell. Edges and faces: the runs of the sorted records, which are already in
    // (entity, cell) order. Interiors: one item per cell.
    std::vector<int32_t> e2c_ptr(n_ent + 1, 0);
    std::vector<int32_t> e2c(ent.size());
    {
        int corner_L[8], nl = 0;
        for (int L = 0; L < 27; ++L)
            if (n_corner[L] == 1) corner_L[nl++] = L;
        FGB_REQUIRE(nl == 8, "Q2 lattice: 8 corner nodes per cell");
        for (int c = 0; c < nc; ++c)
            for (int j = 0; j < 8; ++j) e2c_ptr[ent[27 * (size_t)c + corner_L[j]] + 1]++;
        for (int v = 0; v < nvx; ++v) e2c_ptr[v + 1] += e2c_ptr[v];
        const int64_t nv_items = e2c_ptr[nvx];
        FGB_REQUIRE(nv_items == 8 * (int64_t)nc, "Q2 structure: vertex items");
        {
            std::vector<int32_t> cur(e2c_ptr.begin(), e2c_ptr.begin() + nvx);
            for (int c = 0; c < nc; ++c)
                for (int j = 0; j < 8; ++j) {
                    const int32_t item = 27 * c + corner_L[j];
                    e2c[cur[ent[item]]++] = item;
                }
        }
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < (long long)ne; ++i) {
            e2c[nv_items + i] = 27 * ek[i].cell + ek[i].local;
            if (i == 0 || run_id[i - 1] != run_id[i]) e2c_ptr[nvx + run_id[i]] = (int32_t)(nv_items + i);
        }
#pragma omp parallel for schedule(static)
        for (int c = 0; c < nc; ++c) {
            e2c_ptr[nvx + n_shared + c] = (int32_t)(nv_items + (int64_t)ne + c);
            e2c[nv_items + ne + c] = 27 * c + 13;
        }
        e2c_ptr[n_ent] = (int32_t)(nv_items + (int64_t)ne + nc);
    }
    ek.clear();
    ek.shrink_to_fit();
    phase("entity -> cells");
    // entity -> its first (cell, L) in item order (the head of its stable list) and position
    std::vector<int32_t> e_cell(n_ent, -1);
    std::vector<int8_t> e_loc(n_ent, 0);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < n_ent; ++e) {
        if (e2c_ptr[e] == e2c_ptr[e + 1]) continue;
        const int32_t item = e2c[e2c_ptr[e]];
        e_cell[e] = item / 27;
        e_loc[e] = (int8_t)(item % 27);
    }
    std::vector<double> exyz(3 * (size_t)n_ent);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < n_ent; ++e) {
        const int L = e_loc[e], n = n_corner[L];  // the lattice corners of L, tabulated above
        int32_t nd[8];
        for (int q = 0; q < n; ++q) nd[q] = cell_node(e_cell[e], corner_tab[L][q]);
        for (int d = 0; d < 3; ++d) {
            double s = 0.0;
            for (int q = 0; q < n; ++q) s += X[3 * (size_t)nd[q] + d];
            exyz[3 * (size_t)e + d] = s / n;
        }
    }

    phase("entity positions");
    // row length = number of distinct entities of the incident cells, counted with a stamped
    // open-addressing set per thread (no sort: the columns themselves are built later)
    int max_inc = 1;
    for (int e = 0; e < n_ent; ++e) max_inc = std::max(max_inc, e2c_ptr[e + 1] - e2c_ptr[e]);
    int tab = 64;
    while (tab < 2 * 27 * max_inc) tab *= 2;
    std::vector<int32_t> deg(n_ent);
#pragma omp parallel
    {
        std::vector<int32_t> key(tab);
        std::vector<uint32_t> stamp(tab, 0);
        uint32_t cur = 0;
        const uint32_t mask = (uint32_t)tab - 1;
#pragma omp for schedule(dynamic, 4096)
        for (int e = 0; e < n_ent; ++e) {
            ++cur;
            int cnt = 0;
            for (int p = e2c_ptr[e]; p < e2c_ptr[e + 1]; ++p) {
                const int32_t* ce = &ent[27 * (size_t)(e2c[p] / 27)];
                for (int L = 0; L < 27; ++L) {
                    const int32_t k = ce[L];
                    uint32_t h = ((uint32_t)k * 2654435761u) & mask;
                    while (stamp[h] == cur && key[h] != k) h = (h + 1) & mask;
                    if (stamp[h] != cur) {
                        stamp[h] = cur;
                        key[h] = k;
                        ++cnt;
                    }
                }
            }
            deg[e] = cnt;
        }
    }

    phase("row lengths");
    // ---- numbering: Morton order, then windows of 256 by decreasing row length
    double mn0 = 1e300, mn1 = 1e300, mn2 = 1e300, mx0 = -1e300, mx1 = -1e300, mx2 = -1e300;
#pragma omp parallel for schedule(static) reduction(min : mn0, mn1, mn2) reduction(max : mx0, mx1, mx2)
    for (int e = 0; e < n_ent; ++e) {
        const double* p = &exyz[3 * (size_t)e];
        mn0 = std::min(mn0, p[0]);
        mn1 = std::min(mn1, p[1]);
        mn2 = std::min(mn2, p[2]);
        mx0 = std::max(mx0, p[0]);
        mx1 = std::max(mx1, p[1]);
        mx2 = std::max(mx2, p[2]);
    }
    const double mn[3] = {mn0, mn1, mn2}, mx[3] = {mx0, mx1, mx2};
    std::vector<std::pair<uint64_t, int32_t>> key(n_ent);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < n_ent; ++e) {
        uint64_t code = 0;
        for (int d = 0; d < 3; ++d) {
            const double span = mx[d] > mn[d] ? mx[d] - mn[d] : 1.0;
            const double t = (exyz[3 * (size_t)e + d] - mn[d]) / span;
            const uint64_t q = (uint64_t)std::min(2097151.0, std::max(0.0, std::floor(t * 2097151.0)));
            code |= spread3q(q) << d;
        }
        key[e] = {code, e};
    }
    // sorted by (code, entity): buckets by the top 16 bits of the 63-bit code (atomic counts
    // and cursors), then each bucket; the keys are unique, so the order is the full sort's
    {
        constexpr int kBits = 16, kShift = 63 - kBits;
        std::vector<int32_t> bstart((1 << kBits) + 1, 0);
#pragma omp parallel for schedule(static)
        for (int e = 0; e < n_ent; ++e) __atomic_fetch_add(&bstart[(key[e].first >> kShift) + 1], 1, __ATOMIC_RELAXED);
        for (int b = 0; b < (1 << kBits); ++b) bstart[b + 1] += bstart[b];
        std::vector<int32_t> cur(bstart.begin(), bstart.end() - 1);
        std::vector<std::pair<uint64_t, int32_t>> sorted(n_ent);
#pragma omp parallel for schedule(static)
        for (int e = 0; e < n_ent; ++e)
            sorted[__atomic_fetch_add(&cur[key[e].first >> kShift], 1, __ATOMIC_RELAXED)] = key[e];
#pragma omp parallel for schedule(dynamic, 16)
        for (int b = 0; b < (1 << kBits); ++b) std::sort(sorted.begin() + bstart[b], sorted.begin() + bstart[b + 1]);
        key.swap(sorted);
    }
    std::vector<int32_t> dof2e(n_ent), e2dof(n_ent);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n_ent; ++i) dof2e[i] = key[i].second;
    key.clear();
    key.shrink_to_fit();
    // Q2 rows range from 27 (interiors) to several hundred (tet vertices shared by many
    // hexes); windows of 4096 keep SELL padding near 5 % (256: 44 %) while the gathers stay
    // inside a 32 KB stretch of the vector
    const int kWin = 4096;
#pragma omp parallel for schedule(dynamic, 16)
    for (int w0 = 0; w0 < n_ent; w0 += kWin) {
        const int w1 = std::min(n_ent, w0 + kWin);
        std::stable_sort(dof2e.begin() + w0, dof2e.begin() + w1, [&](int32_t a, int32_t b) { return deg[a] > deg[b]; });
    }
#pragma omp parallel for schedule(static)
    for (int d = 0; d < n_ent; ++d) e2dof[dof2e[d]] = d;

    phase("Morton order, windows");
    fs.cell_dofs.resize(27 * (size_t)nc);
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < ent.size(); ++i) fs.cell_dofs[i] = e2dof[ent[i]];
    fs.dof2node.assign(n_ent, -1);
    fs.node2dof.assign(pm.hex.n_nodes(), -1);
    for (int v = 0; v < nvx; ++v) {
        const int d = e2dof[v];
        fs.dof2node[d] = pm.vac.vertex2node[v];
        fs.node2dof[pm.vac.vertex2node[v]] = d;
    }
    fs.dof_xyz.resize(3 * (size_t)n_ent);
    fs.dof_cell.resize(n_ent);
    fs.dof_local.resize(n_ent);
    fs.row_len.resize(n_ent);
#pragma omp parallel for schedule(static)
    for (int d = 0; d < n_ent; ++d) {
        const int e = dof2e[d];
        for (int k = 0; k < 3; ++k) fs.dof_xyz[3 * (size_t)d + k] = exyz[3 * (size_t)e + k];
        fs.dof_cell[d] = e_cell[e];
        fs.dof_local[d] = e_loc[e];
        fs.row_len[d] = deg[e];
    }
    exyz.clear();
    exyz.shrink_to_fit();

    phase("dof tables");
    // row -> (cell, local), ascending cell
    // row pointers: lengths in parallel, then a blocked prefix sum (per-block totals, a scan
    // over the blocks, each block offset by its predecessors)
    fs.r2c_ptr.assign(n_ent + 1, 0);
    {
        const int nt = std::max(1, omp_get_max_threads());
        std::vector<int64_t> bsum(nt + 1, 0);
#pragma omp parallel num_threads(nt)
        {
            const int t = omp_get_thread_num();
            const int d0 = (int)((int64_t)n_ent * t / nt), d1 = (int)((int64_t)n_ent * (t + 1) / nt);
            int64_t run = 0;
            for (int d = d0; d < d1; ++d) {
                run += e2c_ptr[dof2e[d] + 1] - e2c_ptr[dof2e[d]];
                fs.r2c_ptr[d + 1] = (int32_t)run;
            }
            bsum[t + 1] = run;
#pragma omp barrier
#pragma omp single
            for (int u = 0; u < nt; ++u) bsum[u + 1] += bsum[u];
            const int32_t off = (int32_t)bsum[t];
            for (int d = d0; d < d1; ++d) fs.r2c_ptr[d + 1] += off;
        }
    }
    fs.r2c_item.resize(fs.r2c_ptr[n_ent]);
#pragma omp parallel for schedule(static)
    for (int d = 0; d < n_ent; ++d) {
        const int e = dof2e[d];
        int32_t* o = &fs.r2c_item[fs.r2c_ptr[d]];
        std::copy(e2c.begin() + e2c_ptr[e], e2c.begin() + e2c_ptr[e + 1], o);
        std::sort(o, o + (e2c_ptr[e + 1] - e2c_ptr[e]));
    }

    phase("row -> cells");
    // ---- SELL-32 with 4-wide row chunks, filled directly (second pass over the row sets)
    const int C = 32, W4 = 4;
    const int ns = (n_ent + C - 1) / C;
    fs.slice_ptr.assign(ns + 1, 0);
    fs.slice_len.assign(ns, 0);
    int64_t nz = 0;
    for (int s = 0; s < ns; ++s) {
        int m = 0;
        for (int r = s * C; r < std::min(n_ent, (s + 1) * C); ++r) {
            m = std::max(m, fs.row_len[r]);
            nz += fs.row_len[r];
        }
        m = (m + W4 - 1) / W4 * W4;
        fs.slice_len[s] = m;
        fs.slice_ptr[s + 1] = fs.slice_ptr[s] + (int64_t)m * C;
    }
    fs.n_entries = nz;
    if (sell_columns) fs.sell_col.assign(fs.slice_ptr[ns], 0);
#pragma omp parallel if (sell_columns)
    if (sell_columns) {
        std::vector<int32_t> l;
#pragma omp for schedule(dynamic, 256)
        for (int s = 0; s < ns; ++s)
            for (int lane = 0; lane < C; ++lane) {
                const int r = s * C + lane;
                if (r < n_ent) {
                    // the row's columns: the DoFs of its cells (already renumbered), sorted, unique
                    l.clear();
                    for (int p = fs.r2c_ptr[r]; p < fs.r2c_ptr[r + 1]; ++p) {
                        const int32_t* cdr = &fs.cell_dofs[27 * (size_t)(fs.r2c_item[p] / 27)];
                        l.insert(l.end(), cdr, cdr + 27);
                    }
                    std::sort(l.begin(), l.end());
                    l.erase(std::unique(l.begin(), l.end()), l.end());
                }
                for (int j = 0; j < fs.slice_len[s]; ++j) {
                    const int64_t pos = fs.slice_ptr[s] + ((int64_t)(j / W4) * C + lane) * W4 + j % W4;
                    fs.sell_col[pos] = (r < n_ent && j < (int)l.size()) ? l[j] : (r < n_ent ? r : 0);
                }
            }
    }

    phase("SELL columns");
    // ---- boundary faces: face entities owned by one vacuum cell (src/DealSolver.cpp:461-518)
    struct BF {
        int32_t cell;
        int8_t L;
        double ctr[3];
    };
    std::vector<BF> bnd;
    for (size_t i = 0; i < face_count.size(); ++i)
        if (face_count[i] == 1) {
            BF b;
            b.cell = ent_first[i] / 27;
            b.L = (int8_t)(ent_first[i] % 27);
            const int d = e2dof[nvx + (int)i];
            for (int k = 0; k < 3; ++k) b.ctr[k] = fs.dof_xyz[3 * (size_t)d + k];
            bnd.push_back(b);
        }
    std::sort(bnd.begin(), bnd.end(), [](const BF& a, const BF& b) { return a.cell != b.cell ? a.cell < b.cell : a.L < b.L; });
    double bmn[3] = {1e16, 1e16, 1e16}, bmx[3] = {-1e16, -1e16, -1e16};
    for (const BF& b : bnd)
        for (int k = 0; k < 3; ++k) {
            bmn[k] = std::min(bmn[k], b.ctr[k]);
            bmx[k] = std::max(bmx[k], b.ctr[k]);
        }
    const double eps = 1e-6;
    fs.bc_kind.assign(n_ent, 0);
    std::vector<int32_t> top;
    for (const BF& b : bnd) {
        const double x = b.ctr[0], y = b.ctr[1], z = b.ctr[2];
        const bool side = std::fabs(x - bmn[0]) <= eps || std::fabs(x - bmx[0]) <= eps ||
                          std::fabs(y - bmn[1]) <= eps || std::fabs(y - bmx[1]) <= eps;
        if (side) continue;
        // the 9 lattice nodes of the face: its fixed axis keeps the face node's value
        int a0, b0, c0;
        q2_lattice(b.L, a0, b0, c0);
        int fd[9];
        for (int v = 0; v < 3; ++v)
            for (int u = 0; u < 3; ++u) {
                int a = a0, bb = b0, c = c0;
                if (a0 != 1) { bb = u; c = v; }        // face normal along a
                else if (b0 != 1) { a = u; c = v; }    // normal along b
                else { a = u; bb = v; }                // normal along c
                fd[u + 3 * v] = fs.cell_dofs[27 * (size_t)b.cell + a + 3 * bb + 9 * c];
            }
        if (std::fabs(z - bmx[2]) <= eps) {
            top.insert(top.end(), fd, fd + 9);
        } else {
            for (int q = 0; q < 9; ++q) fs.bc_kind[fd[q]] = 1;
        }
    }
    fs.top_faces = top;
    for (int32_t d : top)
        if (fs.bc_kind[d] == 0) fs.bc_kind[d] = 2;
    const int nt = fs.n_top_faces();
    fs.r2f_ptr.assign(n_ent + 1, 0);
    for (int32_t d : top) fs.r2f_ptr[d + 1]++;
    for (int i = 0; i < n_ent; ++i) fs.r2f_ptr[i + 1] += fs.r2f_ptr[i];
    fs.r2f_item.resize(fs.r2f_ptr[n_ent]);
    {
        std::vector<int32_t> pos(fs.r2f_ptr.begin(), fs.r2f_ptr.end() - 1);
        for (int f = 0; f < nt; ++f)
            for (int q = 0; q < 9; ++q) fs.r2f_item[pos[top[9 * (size_t)f + q]]++] = 9 * f + q;
    }
    phase("boundary, r2f");
    return fs;
}

}  // namespace fgb
