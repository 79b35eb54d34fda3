// Test-oracle driver for the reference's own mesh-split, cell-precompute, point-location
// and interpolation code (tetgen/, src/Tethex.cpp, src/TetgenMesh.cpp, src/TetgenCells.cpp,
// src/InterpolatorCells.cpp), compiled unmodified by oracle/Makefile.ref.
//
// THIS IS TEST INFRASTRUCTURE. It only produces golden vectors that the tests compare the
// femocs_gb300 host preparation and CUDA kernels against; nothing in the product links it.
//
// usage: ref_driver <mesh.msh> <points.bin> <out.bin>
//   mesh.msh   : Gmsh 2.2 ASCII tetrahedral mesh, physical tag 3 = vacuum, 1 = bulk
//   points.bin : int32 n, then n*3 float64 (x,y,z interleaved)
//   out.bin    : sequence of records {char name[16]; char type ('i'|'d'); int64 count; data}
//
// The mesh is read the way the reference reads `mesh_file` (ProjectRunaway::generate_mesh,
// src/ProjectRunaway.cpp:180: TetgenMesh::read(file, "rQnn")), the vacuum interpolator is
// initialised the way Interpolator::initialize does it (src/Interpolator.cpp:28-77), and the
// query loop replays SolutionReader::calc_full_interpolation (src/SolutionReader.cpp:136-165)
// for interpolation ranks 1, 2 and 3 with the chained cell guess.
//
// Nodal solution used for interpolation: a fixed smooth test field evaluated at every mesh
// node (test_solution below); the same formula lives in tests/golden/make_golden.py.
// Nodal E recovery (src/Interpolator.cpp:125-140) and smoothing (:142-170) are restated
// here in a few lines on top of the reference's compiled LinearHexahedra::interp_gradient
// and TetgenMesh::calc_pseudo_3D_vorocells, because Interpolator.cpp itself needs deal.II.

#define MAINFILE
#include "Globals.h"
#include "Config.h"
#include "TetgenMesh.h"
#include "InterpolatorCells.h"

#include <cstdio>
#include <cstring>
#include <cstdint>
#include <vector>
#include <string>

using namespace femocs;

static void put(FILE* f, const char* name, char type, int64_t count, const void* data) {
    char nm[16];
    std::memset(nm, 0, sizeof(nm));
    std::strncpy(nm, name, 15);
    std::fwrite(nm, 1, 16, f);
    std::fwrite(&type, 1, 1, f);
    std::fwrite(&count, sizeof(int64_t), 1, f);
    size_t es = (type == 'd') ? sizeof(double) : sizeof(int32_t);
    if (count > 0) std::fwrite(data, es, (size_t)count, f);
}

// smooth test field: phi and a vector, polynomials of the node coordinates (IEEE +,-,* only,
// so every platform evaluates it identically)
static Solution test_solution(const Point3& p) {
    const double phi = 0.25 * p.x - 0.5 * p.y + 0.125 * p.z + 1e-3 * p.x * p.z + 2e-4 * p.x * p.y * p.y
                     - 3e-5 * p.z * p.z * p.y;
    const Vec3 e(0.1 + 1e-3 * p.y, -0.2 + 2e-3 * p.z, 0.3 + 1e-3 * p.x);
    const double rho = 1.0 + 1e-2 * p.z;
    return Solution(e, rho, phi);
}

int main(int argc, char** argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: %s mesh.msh points.bin out.bin\n", argv[0]);
        return 2;
    }
    MODES.MUTE = true;
    MODES.VERBOSE = false;
    MODES.WRITELOG = false;

    Config conf;
    TetgenMesh mesh(&conf.mesh);
    if (mesh.read(argv[1], "rQnn")) {
        std::fprintf(stderr, "mesh read failed\n");
        return 1;
    }

    // ---------------- points
    FILE* fp = std::fopen(argv[2], "rb");
    if (!fp) return 1;
    int32_t n_pts = 0;
    if (std::fread(&n_pts, 4, 1, fp) != 1) return 1;
    std::vector<double> pts(3 * (size_t)n_pts);
    if (n_pts > 0 && std::fread(pts.data(), 8, pts.size(), fp) != pts.size()) return 1;
    std::fclose(fp);

    // ---------------- interpolator set-up as in Interpolator::initialize (vacuum search region)
    InterpolatorNodes nodes("elfield", "charge_density", "potential");
    LinearTetrahedra lintet(&nodes);
    QuadraticTetrahedra quadtet(&nodes, &lintet);
    LinearHexahedra linhex(&nodes, &lintet);
    nodes.set_mesh(&mesh);
    lintet.set_mesh(&mesh);
    quadtet.set_mesh(&mesh);
    linhex.set_mesh(&mesh);
    nodes.precompute(TYPES.VACUUM);
    lintet.precompute();
    quadtet.precompute();
    linhex.precompute(TYPES.VACUUM);
    lintet.narrow_search_to(TYPES.VACUUM);

    const int n_nodes = mesh.nodes.size();
    const int n_tets = mesh.tets.size();
    const int n_hexs = mesh.hexs.size();
    for (int i = 0; i < n_nodes; ++i) nodes.append_solution(Solution(0.0));
    for (int i = 0; i < n_nodes; ++i) nodes.set_solution(i, test_solution(mesh.nodes[i]));

    FILE* fo = std::fopen(argv[3], "wb");
    if (!fo) return 1;

    // ---------------- mesh as the reference holds it
    {
        std::vector<double> xyz(3 * (size_t)n_nodes);
        std::vector<int32_t> nmark(n_nodes);
        for (int i = 0; i < n_nodes; ++i) {
            Point3 p = mesh.nodes[i];
            xyz[3 * i] = p.x; xyz[3 * i + 1] = p.y; xyz[3 * i + 2] = p.z;
            nmark[i] = mesh.nodes.get_marker(i);
        }
        put(fo, "node_xyz", 'd', xyz.size(), xyz.data());
        put(fo, "node_marker", 'i', nmark.size(), nmark.data());

        std::vector<int32_t> tv(4 * (size_t)n_tets), tm(n_tets), tn(4 * (size_t)n_tets);
        for (int t = 0; t < n_tets; ++t) {
            SimpleElement e = mesh.tets[t];
            for (int k = 0; k < 4; ++k) tv[4 * t + k] = e[k];
            tm[t] = mesh.tets.get_marker(t);
            std::vector<int> nb = mesh.tets.get_neighbours(t);
            for (int k = 0; k < 4; ++k) tn[4 * t + k] = nb[k];
        }
        put(fo, "tet_nodes", 'i', tv.size(), tv.data());
        put(fo, "tet_marker", 'i', tm.size(), tm.data());
        put(fo, "tet_nbor", 'i', tn.size(), tn.data());

        std::vector<int32_t> hv(8 * (size_t)n_hexs), hm(n_hexs);
        for (int h = 0; h < n_hexs; ++h) {
            SimpleHex e = mesh.hexs[h];
            for (int k = 0; k < 8; ++k) hv[8 * h + k] = e[k];
            hm[h] = mesh.hexs.get_marker(h);
        }
        put(fo, "hex_nodes", 'i', hv.size(), hv.data());
        put(fo, "hex_marker", 'i', hm.size(), hm.data());

        double em = mesh.tets.stat.edgemax;
        put(fo, "tet_edgemax", 'd', 1, &em);
        double df = lintet.decay_factor;
        put(fo, "decay_factor", 'd', 1, &df);
    }

    // ---------------- locate + interpolate, ranks 1..3, chained guesses as in
    // SolutionReader::calc_full_interpolation with a fresh reader (cell starts at -1)
    for (int rank = 1; rank <= 3; ++rank) {
        std::vector<int32_t> cells(n_pts);
        std::vector<double> sol(5 * (size_t)n_pts);
        int cell = -1;
        for (int i = 0; i < n_pts; ++i) {
            Point3 p(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
            Solution s;
            if (rank == 1) s = lintet.locate_interpolate(p, cell);
            else if (rank == 2) s = quadtet.locate_interpolate(p, cell);
            else s = linhex.locate_interpolate(p, cell);
            cells[i] = cell;
            sol[5 * i] = s.vector.x; sol[5 * i + 1] = s.vector.y; sol[5 * i + 2] = s.vector.z;
            sol[5 * i + 3] = s.scalar1; sol[5 * i + 4] = s.scalar2;
        }
        char nm[16];
        if (rank == 1) {
            std::vector<double> bc(4 * (size_t)n_pts);
            for (int i = 0; i < n_pts; ++i) {
                Point3 p(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
                std::array<double, 4> b = lintet.shape_functions(Vec3(p), std::abs(cells[i]));
                for (int k = 0; k < 4; ++k) bc[4 * i + k] = b[k];
            }
            put(fo, "bcc_r1", 'd', bc.size(), bc.data());
        }
        std::snprintf(nm, sizeof(nm), "cells_r%d", rank);
        put(fo, nm, 'i', cells.size(), cells.data());
        std::snprintf(nm, sizeof(nm), "interp_r%d", rank);
        put(fo, nm, 'd', sol.size(), sol.data());
    }

    // ---------------- surface (2-D) location and interpolation, when the mesh file carries
    // surface triangles: TetGen's tri->tet mapping of the read (calc_tri2tet2tri_mapping,
    // src/TetgenMesh.cpp:592-612), LinearTriangles / QuadraticTriangles set up as in
    // Interpolator::initialize, and the chained query loop of calc_full_interpolation with
    // dim = 2 (src/SolutionReader.cpp:43-55)
    const int n_tris = mesh.tris.size();
    if (n_tris > 0) {
        LinearTriangles lintri(&nodes, &lintet);
        QuadraticTriangles quadtri(&nodes, &lintri, &quadtet);
        LinearQuadrangles linquad(&nodes, &lintri, &linhex);
        lintri.set_mesh(&mesh);
        quadtri.set_mesh(&mesh);
        linquad.set_mesh(&mesh);
        lintri.precompute();
        quadtri.precompute();
        linquad.precompute();
        std::vector<int32_t> tv(3 * (size_t)n_tris), t2t(2 * (size_t)n_tris);
        std::vector<double> tn(3 * (size_t)n_tris);
        for (int f = 0; f < n_tris; ++f) {
            SimpleFace sf = mesh.tris[f];
            for (int k = 0; k < 3; ++k) tv[3 * f + k] = sf[k];
            std::array<int, 2> tt = mesh.tris.to_tets(f);
            t2t[2 * f] = tt[0];
            t2t[2 * f + 1] = tt[1];
            Vec3 nv = lintri.get_norm(f);
            tn[3 * f] = nv.x; tn[3 * f + 1] = nv.y; tn[3 * f + 2] = nv.z;
        }
        put(fo, "tri_nodes", 'i', tv.size(), tv.data());
        put(fo, "tri2tet", 'i', t2t.size(), t2t.data());
        put(fo, "tri_norm", 'd', tn.size(), tn.data());
        for (int rank = 1; rank <= 3; ++rank) {
            std::vector<int32_t> cells(n_pts);
            std::vector<double> sol(5 * (size_t)n_pts);
            int cell = -1;
            for (int i = 0; i < n_pts; ++i) {
                Point3 p(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
                Solution s = rank == 1 ? lintri.locate_interpolate(p, cell)
                             : rank == 2 ? quadtri.locate_interpolate(p, cell) : linquad.locate_interpolate(p, cell);
                cells[i] = cell;
                sol[5 * i] = s.vector.x; sol[5 * i + 1] = s.vector.y; sol[5 * i + 2] = s.vector.z;
                sol[5 * i + 3] = s.scalar1; sol[5 * i + 4] = s.scalar2;
            }
            char nm[16];
            std::snprintf(nm, sizeof(nm), "cells_s%d", rank);
            put(fo, nm, 'i', cells.size(), cells.data());
            std::snprintf(nm, sizeof(nm), "interp_s%d", rank);
            put(fo, nm, 'd', sol.size(), sol.data());
        }
    }

    // ---------------- nodal field recovery (vacuum hexes) and smoothing
    {
        std::vector<std::vector<std::pair<int, int>>> node2cells(n_nodes);
        for (int hex = 0; hex < n_hexs; ++hex)
            if (mesh.hexs.get_marker(hex) > 0) {
                SimpleHex shex = mesh.hexs[hex];
                for (int node = 0; node < 8; ++node)
                    node2cells[shex[node]].push_back(std::make_pair(hex, node));
            }
        std::vector<Vec3> efield(n_nodes, Vec3(0.0));
        for (int node = 0; node < n_nodes; ++node) {
            if (nodes.femocs2deal(node) < 0) continue;
            Vec3 mean_field(0);
            int nf = node2cells[node].size();
            if (nf > 0) {
                for (auto pr : node2cells[node]) mean_field += linhex.interp_gradient(pr.first, pr.second);
                mean_field *= (1.0 / nf);
            }
            efield[node] = mean_field;
        }
        std::vector<double> e_raw(3 * (size_t)n_nodes);
        for (int i = 0; i < n_nodes; ++i) {
            e_raw[3 * i] = efield[i].x; e_raw[3 * i + 1] = efield[i].y; e_raw[3 * i + 2] = efield[i].z;
        }
        put(fo, "nodal_E_raw", 'd', e_raw.size(), e_raw.data());

        std::vector<std::vector<unsigned>> nborlist;
        mesh.calc_pseudo_3D_vorocells(nborlist, true);
        std::vector<int32_t> vptr(1, 0), vidx;
        for (auto& l : nborlist) {
            for (unsigned v : l) vidx.push_back((int32_t)v);
            vptr.push_back((int32_t)vidx.size());
        }
        put(fo, "voro_ptr", 'i', vptr.size(), vptr.data());
        put(fo, "voro_idx", 'i', vidx.size(), vidx.data());

        for (unsigned i = 0; i < nborlist.size(); ++i) {
            if (nborlist[i].size() == 0) continue;
            Point3 tetnode = mesh.nodes[i];
            Vec3 vec(0);
            double w_sum = 0;
            for (unsigned nbor : nborlist[i]) {
                double w = std::exp(lintet.decay_factor * tetnode.distance(mesh.nodes[nbor]));
                w_sum += w;
                vec += efield[nbor] * w;
            }
            if (w_sum > 0) {
                vec *= (1.0 / w_sum);
                efield[i] = vec;
            }
        }
        std::vector<double> e_s(3 * (size_t)n_nodes);
        for (int i = 0; i < n_nodes; ++i) {
            e_s[3 * i] = efield[i].x; e_s[3 * i + 1] = efield[i].y; e_s[3 * i + 2] = efield[i].z;
        }
        put(fo, "nodal_E_smooth", 'd', e_s.size(), e_s.data());
    }

    std::fclose(fo);
    return 0;
}
