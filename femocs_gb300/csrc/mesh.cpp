// Host-side mesh preparation (see mesh.h). Compiled with -ffp-contract=off so that every
// coordinate and table entry is produced by the same IEEE operation sequence on x86 and Arm.
#include "mesh.h"
#include "mesh_math.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <fstream>
#include <sstream>
#include <unordered_map>

namespace fgb {

namespace {
thread_local std::string g_last_error;
}
void set_last_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }

// ------------------------------------------------------------------------------------
// Gmsh 2.2 ASCII reader (tetrahedra only; first tag = region marker), the input format of
// the reference's `mesh_file` path (src/Tethex.cpp:478-586).
TetMesh read_gmsh(const std::string& path) {
    std::ifstream in(path);
    FGB_REQUIRE(in.is_open(), "cannot open mesh file " + path);
    TetMesh tm;
    std::unordered_map<long long, int> id2idx;
    std::string tok;
    in >> tok;
    FGB_REQUIRE(tok == "$MeshFormat", "not a Gmsh file: " + path);
    double version = 0;
    int binary = 0, dsize = 0;
    in >> version >> binary >> dsize;
    FGB_REQUIRE(version >= 2.2 && binary == 0, "only ASCII Gmsh 2.2+ meshes are supported");
    while (in >> tok) {
        if (tok == "$Nodes") {
            long long n = 0;
            in >> n;
            tm.xyz.resize(3 * (size_t)n);
            for (long long i = 0; i < n; ++i) {
                long long id;
                double x, y, z;
                in >> id >> x >> y >> z;
                id2idx[id] = (int)i;
                tm.xyz[3 * i] = x;
                tm.xyz[3 * i + 1] = y;
                tm.xyz[3 * i + 2] = z;
            }
        } else if (tok == "$Elements") {
            long long n = 0;
            in >> n;
            std::string line;
            std::getline(in, line);
            for (long long e = 0; e < n; ++e) {
                std::getline(in, line);
                std::istringstream ls(line);
                long long serial;
                int type, ntags;
                ls >> serial >> type >> ntags;
                std::vector<long long> tags(ntags);
                for (int k = 0; k < ntags; ++k) ls >> tags[k];
                if (type != 4) continue;
                FGB_REQUIRE(ntags >= 1, "tetrahedron without region tag");
                for (int k = 0; k < 4; ++k) {
                    long long v;
                    ls >> v;
                    auto it = id2idx.find(v);
                    FGB_REQUIRE(it != id2idx.end(), "element references unknown node");
                    tm.tets.push_back(it->second);
                }
                tm.marker.push_back((int32_t)tags[0]);
            }
        }
    }
    FGB_REQUIRE(tm.n_tets() > 0, "mesh has no tetrahedra: " + path);
    return tm;
}

// ------------------------------------------------------------------------------------
namespace {

using mm::LocalEdges;
using mm::local_edges;

inline uint64_t edge_key(int32_t hi, int32_t lo) { return ((uint64_t)(uint32_t)hi << 32) | (uint32_t)lo; }

struct FaceRec {
    int32_t v0, v1, v2;  // sorted ascending
    int64_t order;       // first-encounter order
    int32_t tet;
    int32_t opp;         // local index of the vertex opposite to this face in `tet`
};

}  // namespace

HexMesh tethex_split(const TetMesh& tm) {
    const int n_old = tm.n_nodes();
    const int n_tets = tm.n_tets();
    const int32_t* T = tm.tets.data();

    // ---- edges: all vertex pairs of the tets, numbered by ascending (max, min)
    std::vector<uint64_t> ekeys;
    ekeys.reserve(6 * (size_t)n_tets);
    for (int t = 0; t < n_tets; ++t) {
        const int32_t* v = T + 4 * t;
        for (int i = 0; i < 4; ++i)
            for (int j = i + 1; j < 4; ++j) {
                int32_t hi = std::max(v[i], v[j]), lo = std::min(v[i], v[j]);
                FGB_REQUIRE(hi != lo, "degenerate tetrahedron " + std::to_string(t));
                ekeys.push_back(edge_key(hi, lo));
            }
    }
    std::sort(ekeys.begin(), ekeys.end());
    ekeys.erase(std::unique(ekeys.begin(), ekeys.end()), ekeys.end());
    const int n_edges = (int)ekeys.size();
    auto edge_id = [&](int32_t x, int32_t y) -> int {
        uint64_t k = edge_key(std::max(x, y), std::min(x, y));
        return (int)(std::lower_bound(ekeys.begin(), ekeys.end(), k) - ekeys.begin());
    };

    // ---- faces: numbered in the order they are first met while walking tets, their local
    // edges and the vertices opposite to each edge (src/Tethex.cpp:1272-1342)
    std::vector<FaceRec> recs;
    recs.reserve(12 * (size_t)n_tets);
    for (int t = 0; t < n_tets; ++t) {
        const int32_t* v = T + 4 * t;
        LocalEdges le = local_edges(v);
        int slot = 0;
        for (int e = 0; e < le.n; ++e)
            for (int k = 0; k < 4; ++k) {
                if (k == le.a[e] || k == le.b[e]) continue;
                int32_t f[3] = {v[le.a[e]], v[le.b[e]], v[k]};
                std::sort(f, f + 3);
                int opp = 6 - le.a[e] - le.b[e] - k;
                recs.push_back({f[0], f[1], f[2], (int64_t)t * 12 + slot, t, opp});
                ++slot;
            }
    }
    std::sort(recs.begin(), recs.end(), [](const FaceRec& x, const FaceRec& y) {
        if (x.v0 != y.v0) return x.v0 < y.v0;
        if (x.v1 != y.v1) return x.v1 < y.v1;
        if (x.v2 != y.v2) return x.v2 < y.v2;
        return x.order < y.order;
    });
    // unique faces with their first-encounter order
    std::vector<std::pair<int64_t, size_t>> firsts;  // (order, first index in recs)
    for (size_t i = 0; i < recs.size(); ++i) {
        if (i == 0 || recs[i].v0 != recs[i - 1].v0 || recs[i].v1 != recs[i - 1].v1 ||
            recs[i].v2 != recs[i - 1].v2)
            firsts.push_back({recs[i].order, i});
    }
    std::sort(firsts.begin(), firsts.end());
    const int n_faces = (int)firsts.size();
    std::vector<int32_t> face_of_group(recs.size());
    std::vector<std::array<int32_t, 3>> face_verts(n_faces);
    {
        std::vector<int32_t> gid(recs.size());
        // group index of each rec (by position of its group's first rec)
        std::vector<int32_t> group_start(recs.size());
        size_t g0 = 0;
        for (size_t i = 0; i < recs.size(); ++i) {
            if (i == 0 || recs[i].v0 != recs[i - 1].v0 || recs[i].v1 != recs[i - 1].v1 ||
                recs[i].v2 != recs[i - 1].v2)
                g0 = i;
            group_start[i] = (int32_t)g0;
        }
        std::vector<int32_t> id_of_first(recs.size(), -1);
        for (int f = 0; f < n_faces; ++f) {
            id_of_first[firsts[f].second] = f;
            const FaceRec& r = recs[firsts[f].second];
            face_verts[f] = {r.v0, r.v1, r.v2};
        }
        for (size_t i = 0; i < recs.size(); ++i) face_of_group[i] = id_of_first[group_start[i]];
    }
    std::vector<int32_t> tet_face(4 * (size_t)n_tets, -1);  // face opposite local vertex
    for (size_t i = 0; i < recs.size(); ++i) tet_face[4 * (size_t)recs[i].tet + recs[i].opp] = face_of_group[i];

    // ---- nodes
    HexMesh hm;
    hm.n_tetnodes = n_old;
    hm.n_edges = n_edges;
    hm.n_faces = n_faces;
    hm.n_tets = n_tets;
    const size_t n_nodes = (size_t)n_old + n_edges + n_faces + n_tets;
    hm.xyz.resize(3 * n_nodes);
    hm.node_marker.resize(n_nodes);
    hm.parents.assign(4 * n_nodes, -1);
    const double* X = tm.xyz.data();
    for (int i = 0; i < n_old; ++i) {
        for (int c = 0; c < 3; ++c) hm.xyz[3 * i + c] = X[3 * i + c];
        hm.node_marker[i] = kTetNode;
        hm.parents[4 * (size_t)i] = i;
    }
    for (int e = 0; e < n_edges; ++e) {
        const int32_t hi = (int32_t)(ekeys[e] >> 32), lo = (int32_t)(ekeys[e] & 0xffffffffu);
        const size_t o = (size_t)n_old + e;
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            s += X[3 * (size_t)lo + c];
            s += X[3 * (size_t)hi + c];
            hm.xyz[3 * o + c] = s / 2;
        }
        hm.node_marker[o] = kEdgeCentroid;
        hm.parents[4 * o] = lo;
        hm.parents[4 * o + 1] = hi;
    }
    for (int f = 0; f < n_faces; ++f) {
        const size_t o = (size_t)n_old + n_edges + f;
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += X[3 * (size_t)face_verts[f][k] + c];
            hm.xyz[3 * o + c] = s / 3;
        }
        hm.node_marker[o] = kFaceCentroid;
        for (int k = 0; k < 3; ++k) hm.parents[4 * o + k] = face_verts[f][k];
    }
    for (int t = 0; t < n_tets; ++t) {
        const size_t o = (size_t)n_old + n_edges + n_faces + t;
        for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += X[3 * (size_t)T[4 * t + k] + c];
            hm.xyz[3 * o + c] = s / 4;
        }
        hm.node_marker[o] = kTetCentroid;
        for (int k = 0; k < 4; ++k) hm.parents[4 * o + k] = T[4 * t + k];
    }

    // ---- hexahedra, four per tet, in the reference's vertex order
    hm.hexs.resize(32 * (size_t)n_tets);
    hm.hex_marker.resize(4 * (size_t)n_tets);
    for (int t = 0; t < n_tets; ++t) {
        const int32_t* v = T + 4 * t;
        LocalEdges le = local_edges(v);
        const bool vac = tm.marker[t] == kVacuum;
        for (int ver = 0; ver < 4; ++ver) {
            int se[3], other[3], ns = 0;
            for (int e = 0; e < le.n && ns < 3; ++e) {
                if (le.a[e] == ver) { se[ns] = e; other[ns] = le.b[e]; ++ns; }
                else if (le.b[e] == ver) { se[ns] = e; other[ns] = le.a[e]; ++ns; }
            }
            FGB_REQUIRE(ns == 3, "tet vertex without three edges");
            auto edge_node = [&](int k) { return n_old + edge_id(v[ver], v[other[k]]); };
            auto face_node = [&](int k1, int k2) {
                int opp = 6 - ver - other[k1] - other[k2];
                return n_old + n_edges + tet_face[4 * (size_t)t + opp];
            };
            (void)se;
            int32_t h[8];
            h[0] = v[ver];
            h[1] = edge_node(0);
            h[2] = face_node(0, 1);
            h[3] = edge_node(1);
            h[4] = edge_node(2);
            h[5] = face_node(0, 2);
            h[6] = n_old + n_edges + n_faces + t;
            h[7] = face_node(1, 2);
            double d[24];
            for (int i = 0; i < 8; ++i)
                for (int c = 0; c < 3; ++c) d[3 * mm::to_deal(i) + c] = hm.xyz[3 * (size_t)h[i] + c];
            if (mm::hex_orientation(d) < 0)
                for (int i = 0; i < 4; ++i) std::swap(h[i], h[i + 4]);
            const size_t hx = 4 * (size_t)t + ver;
            for (int i = 0; i < 8; ++i) hm.hexs[8 * hx + i] = h[i];
            hm.hex_marker[hx] = vac ? (1 + v[ver]) : (-1 - v[ver]);
        }
    }
    return hm;
}

std::vector<int32_t> tet_face_neighbours(const TetMesh& tm) {
    const int n_tets = tm.n_tets();
    struct R { int32_t a, b, c; int32_t slot; };
    std::vector<R> rs;
    rs.reserve(4 * (size_t)n_tets);
    for (int t = 0; t < n_tets; ++t) {
        const int32_t* v = &tm.tets[4 * (size_t)t];
        for (int j = 0; j < 4; ++j) {
            int32_t f[3], n = 0;
            for (int k = 0; k < 4; ++k)
                if (k != j) f[n++] = v[k];
            std::sort(f, f + 3);
            rs.push_back({f[0], f[1], f[2], 4 * t + j});
        }
    }
    std::sort(rs.begin(), rs.end(), [](const R& x, const R& y) {
        if (x.a != y.a) return x.a < y.a;
        if (x.b != y.b) return x.b < y.b;
        if (x.c != y.c) return x.c < y.c;
        return x.slot < y.slot;
    });
    std::vector<int32_t> nb(4 * (size_t)n_tets, -1);
    for (size_t i = 0; i + 1 < rs.size(); ++i) {
        const R& x = rs[i];
        const R& y = rs[i + 1];
        if (x.a == y.a && x.b == y.b && x.c == y.c) {
            FGB_REQUIRE(i + 2 >= rs.size() || !(rs[i + 2].a == x.a && rs[i + 2].b == x.b && rs[i + 2].c == x.c),
                        "non-manifold face shared by more than two tets");
            nb[x.slot] = y.slot / 4;
            nb[y.slot] = x.slot / 4;
            ++i;
        }
    }
    return nb;
}

double tet_edgemax(const TetMesh& tm) {
    double m = -1e300;
    const double* X = tm.xyz.data();
    for (int t = 0; t < tm.n_tets(); ++t) {
        const int32_t* v = &tm.tets[4 * (size_t)t];
        for (int i = 0; i < 4; ++i)
            for (int j = i + 1; j < 4; ++j) {
                double dx = X[3 * v[i]] - X[3 * v[j]];
                double dy = X[3 * v[i] + 1] - X[3 * v[j] + 1];
                double dz = X[3 * v[i] + 2] - X[3 * v[j] + 2];
                double d2 = dx * dx + dy * dy + dz * dz;
                if (d2 > m) m = d2;
            }
    }
    return std::sqrt(m);
}

// ------------------------------------------------------------------------------------
using mm::V3;

TetTables build_tet_tables(const TetMesh& tm, const HexMesh& hm, const std::vector<int32_t>& face_nbr) {
    const int n_tets = tm.n_tets();
    const int n_nodes = tm.n_nodes();
    const double* X = tm.xyz.data();
    TetTables tt;
    tt.det.resize((size_t)kTetDetStride * n_tets);
    tt.centroid.resize(3 * (size_t)n_tets);
    tt.search.resize(n_tets);
    tt.quad_nodes.resize(10 * (size_t)n_tets);

    // node -> tets, ascending tet order
    std::vector<int32_t> cnt(n_nodes + 1, 0);
    for (int t = 0; t < n_tets; ++t)
        for (int k = 0; k < 4; ++k) cnt[tm.tets[4 * (size_t)t + k] + 1]++;
    for (int i = 0; i < n_nodes; ++i) cnt[i + 1] += cnt[i];
    std::vector<int32_t> n2t(cnt[n_nodes]);
    {
        std::vector<int32_t> pos(cnt.begin(), cnt.end() - 1);
        for (int t = 0; t < n_tets; ++t)
            for (int k = 0; k < 4; ++k) n2t[pos[tm.tets[4 * (size_t)t + k]]++] = t;
    }

    tt.nbr_ptr.resize(n_tets + 1);
    tt.nbr_ptr[0] = 0;
    tt.nbr_idx.clear();
    tt.nbr_idx.reserve(40 * (size_t)n_tets);
    std::vector<int32_t> seen_stamp(n_tets, -1);
    for (int t = 0; t < n_tets; ++t) {
        const int32_t* v = &tm.tets[4 * (size_t)t];
        const int32_t* fn = &face_nbr[4 * (size_t)t];
        for (int j = 0; j < 4; ++j)
            if (fn[j] >= 0) {
                tt.nbr_idx.push_back(fn[j]);
                seen_stamp[fn[j]] = t;
            }
        seen_stamp[t] = t;
        for (int k = 0; k < 4; ++k)
            for (int p = cnt[v[k]]; p < cnt[v[k] + 1]; ++p) {
                int32_t u = n2t[p];
                if (seen_stamp[u] == t) continue;
                seen_stamp[u] = t;
                tt.nbr_idx.push_back(u);
            }
        tt.nbr_ptr[t + 1] = (int32_t)tt.nbr_idx.size();

        V3 p1{X[3 * v[0]], X[3 * v[0] + 1], X[3 * v[0] + 2]};
        V3 p2{X[3 * v[1]], X[3 * v[1] + 1], X[3 * v[1] + 2]};
        V3 p3{X[3 * v[2]], X[3 * v[2] + 1], X[3 * v[2] + 2]};
        V3 p4{X[3 * v[3]], X[3 * v[3] + 1], X[3 * v[3] + 2]};
        mm::tet_det_table(p1, p2, p3, p4, &tt.det[(size_t)kTetDetStride * t]);

        double cx = 0.0, cy = 0.0, cz = 0.0;
        for (int k = 0; k < 4; ++k) {
            cx += X[3 * v[k]];
            cy += X[3 * v[k] + 1];
            cz += X[3 * v[k] + 2];
        }
        tt.centroid[3 * (size_t)t] = cx * 0.25;
        tt.centroid[3 * (size_t)t + 1] = cy * 0.25;
        tt.centroid[3 * (size_t)t + 2] = cz * 0.25;
        tt.search[t] = tm.marker[t] == kVacuum ? 1 : 0;

        // quadratic tet: 4 vertices, then the mid-edge nodes of edges 01,12,20,03,13,23
        // (src/InterpolatorCells.cpp:1151-1174 finds them as the edge nodes shared by the
        // corner hexes of the two end vertices)
        int32_t* q = &tt.quad_nodes[10 * (size_t)t];
        static const int ea[6] = {0, 1, 2, 0, 1, 2}, eb[6] = {1, 2, 0, 3, 3, 3};
        for (int k = 0; k < 4; ++k) q[k] = v[k];
        for (int k = 0; k < 6; ++k) {
            // hex 4t+ea holds the edge nodes around vertex ea; find the one shared with 4t+eb
            const int32_t* ha = &hm.hexs[8 * (4 * (size_t)t + ea[k])];
            const int32_t* hb = &hm.hexs[8 * (4 * (size_t)t + eb[k])];
            int32_t found = -1;
            for (int i = 0; i < 8 && found < 0; ++i) {
                if (hm.node_marker[ha[i]] != kEdgeCentroid) continue;
                for (int j = 0; j < 8; ++j)
                    if (hb[j] == ha[i]) { found = ha[i]; break; }
            }
            q[4 + k] = found;
        }
    }
    return tt;
}

std::vector<double> build_hex_coeffs(const HexMesh& hm) {
    const int n = hm.n_hexs();
    std::vector<double> f(24 * (size_t)n);
    for (int h = 0; h < n; ++h) {
        const double* nodes[8];
        for (int k = 0; k < 8; ++k) nodes[k] = &hm.xyz[3 * (size_t)hm.hexs[8 * (size_t)h + k]];
        mm::hex_coefficients(nodes, &f[24 * (size_t)h]);
    }
    return f;
}

VacuumMap build_vacuum_map(const HexMesh& hm) {
    VacuumMap vm;
    const int n_nodes = hm.n_nodes();
    vm.node2vertex.assign(n_nodes, -1);
    for (int h = 0; h < hm.n_hexs(); ++h)
        if (hm.hex_marker[h] > 0) {
            vm.cells.push_back(h);
            for (int k = 0; k < 8; ++k) vm.node2vertex[hm.hexs[8 * (size_t)h + k]] = -2;
        }
    int nv = 0;
    for (int i = 0; i < n_nodes; ++i)
        if (vm.node2vertex[i] == -2) {
            vm.node2vertex[i] = nv++;
            vm.vertex2node.push_back(i);
        }
    return vm;
}

void build_vorocells(const HexMesh& hm, std::vector<int32_t>& ptr, std::vector<int32_t>& idx) {
    const int n_tn = hm.n_tetnodes;
    std::vector<std::vector<int32_t>> cells(n_tn);
    for (int h = 0; h < hm.n_hexs(); ++h) {
        int tn = hm.hex_marker[h];
        if (tn <= 0) continue;
        tn -= 1;
        for (int k = 0; k < 8; ++k) {
            int32_t nd = hm.hexs[8 * (size_t)h + k];
            if (nd != tn && hm.node_marker[nd] >= kEdgeCentroid) cells[tn].push_back(nd);
        }
    }
    ptr.assign(n_tn + 1, 0);
    idx.clear();
    for (int i = 0; i < n_tn; ++i) {
        idx.insert(idx.end(), cells[i].begin(), cells[i].end());
        ptr[i + 1] = (int32_t)idx.size();
    }
}

}  // namespace fgb
