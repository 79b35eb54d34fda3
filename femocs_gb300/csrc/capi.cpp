// extern "C" shims over the C++ classes; no exception crosses this boundary. Failures are
// reported through retval = 1 (reference convention) or a NULL / negative return, with the
// message available from femocs_last_error().
#include <chrono>
#include <cstdio>
#include <cstring>
#include <memory>
#include <omp.h>

#include <thread>

#include "batch.h"
#include "bulk.h"
#include "cell_blocks.h"
#include "facade.h"
#include "fem_q2.h"
#include "server.h"
#include "femocs_gb300.h"
#include "mesh_prep.h"
#include "synth.h"

using namespace fgb;

struct FEMOCS {
    std::unique_ptr<FemocsFacade> f;
};
struct FGB_MESH {
    std::shared_ptr<PreparedMesh> pm;
    MeshPrepTiming timing;  // device: kernel and total ms; host: total ms
};
struct FGB_HEAT {
    std::shared_ptr<const PreparedMesh> pm;
    std::unique_ptr<BulkSolver> b;
    SolveStats last;
};
struct FGB_BATCH {
    std::unique_ptr<BatchSolver> b;
};
struct FGB_SERVER {
    std::unique_ptr<FieldServer> s;
};
struct FGB_FIELD {
    ~FGB_FIELD() {
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
    }
    cudaEvent_t ev[8] = {};
    std::unique_ptr<Field> owned;
    Field* f = nullptr;  // owned.get(), or a field borrowed from a FEMOCS handle
    std::shared_ptr<const PreparedMesh> pm;
    const PreparedMesh* mesh = nullptr;
    SolveStats last;
};

namespace {
template <typename F>
int guarded(F&& fn) {
    try {
        return fn();
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return 1;
    } catch (...) {
        set_last_error("unknown error");
        return 1;
    }
}
template <typename F>
void guarded_rv(int* retval, F&& fn) {
    const int rc = guarded(fn);
    if (retval) *retval = rc;
}
NanotipSpec to_spec(const FgbNanotip* s) {
    NanotipSpec n;
    if (!s) return n;
    n.radius = s->radius;
    n.height = s->height;
    n.box_half = s->box_half;
    n.slab = s->slab;
    n.top = s->top;
    n.h = s->h;
    n.growth = s->growth;
    n.margin = s->margin;
    return n;
}
}  // namespace

namespace {
template <typename T>
void fnv(uint64_t& h, const std::vector<T>& v) {
    const unsigned char* p = reinterpret_cast<const unsigned char*>(v.data());
    for (size_t i = 0; i < v.size() * sizeof(T); ++i) h = (h ^ p[i]) * 1099511628211ull;
    h = (h ^ v.size()) * 1099511628211ull;
}
}  // namespace

extern "C" {

const char* femocs_last_error(void) { return last_error(); }
long long fgb_kernel_launches(void) { return g_kernel_launches.load(); }

// ---------------------------------------------------------------- Part 1
FEMOCS* create_femocs(const char* conf_file) {
    FEMOCS* h = new FEMOCS;
    const int rc = guarded([&] {
        h->f.reset(new FemocsFacade(conf_file ? conf_file : ""));
        return 0;
    });
    if (rc) {
        delete h;
        return nullptr;
    }
    return h;
}
void delete_femocs(FEMOCS* h) { delete h; }

void femocs_run(FEMOCS* h, int* retval, int timestep, double time) {
    guarded_rv(retval, [&] { return h->f->run(timestep, time); });
}
void femocs_import_file(FEMOCS* h, int* retval, const char* file_name) {
    guarded_rv(retval, [&] { return h->f->import_file(file_name ? file_name : ""); });
}
void femocs_import_parcas(FEMOCS*, int* retval, int, const double*, const double*, const double*, const int*) {
    set_last_error("PARCAS import is not provided by this library");
    if (retval) *retval = 1;
}
void femocs_import_atoms(FEMOCS* h, int* retval, int n, const double* x, const double* y, const double* z,
                         const int* types) {
    guarded_rv(retval, [&] { return h->f->import_atoms(n, x, y, z, types); });
}
void femocs_import_mesh(FEMOCS* h, int* retval, int n_nodes, const double* xyz, int n_tets, const int* tets,
                        const int* markers) {
    guarded_rv(retval, [&] { return h->f->import_mesh(n_nodes, xyz, n_tets, tets, markers); });
}
void femocs_interpolate_elfield(FEMOCS* h, int* retval, int n, const double* x, const double* y, const double* z,
                                double* Ex, double* Ey, double* Ez, double* En, int* flag) {
    guarded_rv(retval, [&] { return h->f->interpolate_elfield(n, x, y, z, Ex, Ey, Ez, En, flag); });
}
void femocs_interpolate_surface_elfield(FEMOCS* h, int* retval, int n, const double* x, const double* y,
                                        const double* z, double* Ex, double* Ey, double* Ez, double* En, int* flag) {
    guarded_rv(retval, [&] { return h->f->interpolate_surface_elfield(n, x, y, z, Ex, Ey, Ez, En, flag); });
}
void femocs_interpolate_phi(FEMOCS* h, int* retval, int n, const double* x, const double* y, const double* z,
                            double* phi, int* flag) {
    guarded_rv(retval, [&] { return h->f->interpolate_phi(n, x, y, z, phi, flag); });
}
void femocs_export_data(FEMOCS* h, int* retval, double* data, int n, const char* type) {
    guarded_rv(retval, [&] { return h->f->export_data(data, n, type ? type : ""); });
}
void femocs_export_int(FEMOCS* h, int* retval, int* data, int n, const char* type) {
    guarded_rv(retval, [&] { return h->f->export_int(data, n, type ? type : ""); });
}
void femocs_interpolate(FEMOCS* h, int* retval, double* data, int* flag, int n, const char* type, int near_surface,
                        const double* x, const double* y, const double* z) {
    guarded_rv(retval, [&] { return h->f->interpolate(data, flag, n, type ? type : "", near_surface != 0, x, y, z); });
}
void femocs_parse_int(FEMOCS* h, int* retval, const char* cmd, int* arg) {
    guarded_rv(retval, [&] { return h->f->parse(cmd, arg); });
}
void femocs_parse_double(FEMOCS* h, int* retval, const char* cmd, double* arg) {
    guarded_rv(retval, [&] { return h->f->parse(cmd, arg); });
}
void femocs_parse_string(FEMOCS* h, int* retval, const char* cmd, char* arg) {
    guarded_rv(retval, [&] {
        std::string s;
        const int rc = h->f->parse(cmd, s);
        if (!rc) s.copy(arg, s.length());  // like Femocs::parse_command: no terminator appended
        return rc;
    });
}
void femocs_last_solve(FEMOCS* h, int* retval, double* out8) {
    guarded_rv(retval, [&] {
        const SolveStats& s = h->f->last_stats();
        out8[0] = s.iterations;
        out8[1] = s.outer;
        out8[2] = s.status;
        out8[3] = s.rel_residual;
        out8[4] = s.ms;
        out8[5] = h->f->n_dofs();
        out8[6] = s.bnorm;
        out8[7] = s.levels;
        return 0;
    });
}

static void stats13(const SolveStats& s, double* out) {
    const double v[14] = {(double)s.iterations, (double)s.outer, (double)s.status, s.rel_residual, s.bnorm,
                          s.ms, s.kernel_ms, s.setup_ms, (double)s.levels, s.smoother_ms,
                          (double)s.smoother_launches, s.spmv_ms, (double)s.spmv_launches, s.smoother_bytes};
    std::copy(v, v + 14, out);
}
int fgb_femocs_last_stats(FEMOCS* h, double* out14) {
    return guarded([&] { stats13(h->f->last_stats(), out14); return 0; });
}
int fgb_femocs_enhancement(FEMOCS* h, double* ratio) {
    return guarded([&] { *ratio = h->f->last_enhancement(); return 0; });
}

// ---------------------------------------------------------------- Part 2: meshes
namespace {
TetMesh tet_mesh_of(int n_nodes, const double* xyz, int n_tets, const int* tets, const int* markers) {
    FGB_REQUIRE(n_nodes >= 0 && n_tets >= 0 && (xyz || !n_nodes) && ((tets && markers) || !n_tets),
                "invalid mesh arrays");
    TetMesh tm;
    tm.xyz.assign(xyz, xyz + 3 * (size_t)n_nodes);
    tm.tets.assign(tets, tets + 4 * (size_t)n_tets);
    tm.marker.assign(markers, markers + n_tets);
    return tm;
}
// host (prepare_mesh) or device (prepare_mesh_device) preparation, timed
void prepare_into(FGB_MESH* m, TetMesh&& tm, bool device) {
    if (device) {
        cudaStream_t s;
        FGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        try {
            m->pm = std::make_shared<PreparedMesh>(prepare_mesh_device(std::move(tm), s, &m->timing));
        } catch (...) {
            cudaStreamDestroy(s);
            throw;
        }
        cudaStreamDestroy(s);
    } else {
        const auto t0 = std::chrono::steady_clock::now();
        m->pm = std::make_shared<PreparedMesh>(prepare_mesh(std::move(tm)));
        m->timing.kernel_ms = 0;
        m->timing.total_ms =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
}
}  // namespace

FGB_MESH* fgb_mesh_from_arrays(int n_nodes, const double* xyz, int n_tets, const int* tets, const int* markers) {
    FGB_MESH* m = new FGB_MESH;
    const int rc = guarded([&] {
        prepare_into(m, tet_mesh_of(n_nodes, xyz, n_tets, tets, markers), false);
        return 0;
    });
    if (rc) { delete m; return nullptr; }
    return m;
}
FGB_MESH* fgb_mesh_from_arrays_device(int n_nodes, const double* xyz, int n_tets, const int* tets,
                                      const int* markers) {
    FGB_MESH* m = new FGB_MESH;
    const int rc = guarded([&] {
        prepare_into(m, tet_mesh_of(n_nodes, xyz, n_tets, tets, markers), true);
        return 0;
    });
    if (rc) { delete m; return nullptr; }
    return m;
}
int fgb_mesh_set_surface(FGB_MESH* m, int n_tris, const int* tris, const int* tri2tet) {
    return guarded([&] {
        FGB_REQUIRE(n_tris >= 0 && (n_tris == 0 || (tris && tri2tet)), "invalid surface arrays");
        const PreparedMesh& p = *m->pm;
        SurfaceTables st = build_surface_tables(p.tet.xyz.data(), p.tet.n_nodes(), p.tet.n_tets(),
                                                std::vector<int32_t>(tris, tris + 3 * (size_t)n_tris),
                                                std::vector<int32_t>(tri2tet, tri2tet + 2 * (size_t)n_tris));
        // fields created before keep the tables they were built with
        auto pm = std::make_shared<PreparedMesh>(p);
        pm->surf = std::move(st);
        m->pm = std::move(pm);
        return 0;
    });
}
int64_t fgb_mesh_surface_tris(const FGB_MESH* m) { return m && m->pm ? m->pm->surf.n_tris() : -1; }
int fgb_mesh_prep_timing(const FGB_MESH* m, double* out2) {
    return guarded([&] {
        out2[0] = m->timing.kernel_ms;
        out2[1] = m->timing.total_ms;
        return 0;
    });
}
FGB_MESH* fgb_mesh_read_gmsh(const char* path) {
    FGB_MESH* m = new FGB_MESH;
    const int rc = guarded([&] {
        m->pm = std::make_shared<PreparedMesh>(prepare_mesh(read_gmsh(path)));
        return 0;
    });
    if (rc) { delete m; return nullptr; }
    return m;
}
FGB_MESH* fgb_mesh_synthetic(const FgbNanotip* spec) {
    FGB_MESH* m = new FGB_MESH;
    const int rc = guarded([&] {
        prepare_into(m, make_nanotip_mesh(to_spec(spec)), false);
        return 0;
    });
    if (rc) { delete m; return nullptr; }
    return m;
}
FGB_MESH* fgb_mesh_synthetic_device(const FgbNanotip* spec) {
    FGB_MESH* m = new FGB_MESH;
    const int rc = guarded([&] {
        prepare_into(m, make_nanotip_mesh(to_spec(spec)), true);
        return 0;
    });
    if (rc) { delete m; return nullptr; }
    return m;
}
void fgb_mesh_free(FGB_MESH* m) { delete m; }

int fgb_mesh_sizes(const FGB_MESH* m, int64_t* o) {
    return guarded([&] {
        const PreparedMesh& p = *m->pm;
        o[0] = p.hex.n_tetnodes;
        o[1] = p.tet.n_tets();
        o[2] = p.hex.n_nodes();
        o[3] = p.hex.n_hexs();
        o[4] = (int64_t)p.vac.vertex2node.size();
        o[5] = (int64_t)p.vac.cells.size();
        o[6] = (int64_t)p.tt.nbr_idx.size();
        o[7] = (int64_t)p.voro_idx.size();
        for (int k = 8; k < 12; ++k) o[k] = 0;
        return 0;
    });
}

int fgb_mesh_export(const FGB_MESH* m, const char* name, void* out) {
    return guarded([&] {
        const PreparedMesh& p = *m->pm;
        const std::string n = name ? name : "";
        auto cp = [&](const auto& v) {
            std::memcpy(out, v.data(), v.size() * sizeof(v[0]));
            return 0;
        };
        if (n == "tet_nodes") return cp(p.tet.tets);
        if (n == "tet_marker") return cp(p.tet.marker);
        if (n == "tet_nbor") return cp(p.face_nbr);
        if (n == "node_xyz") return cp(p.hex.xyz);
        if (n == "node_marker") {
            std::vector<int32_t> v(p.hex.node_marker.begin(), p.hex.node_marker.end());
            return cp(v);
        }
        if (n == "hex_nodes") return cp(p.hex.hexs);
        if (n == "node_parents") return cp(p.hex.parents);
        if (n == "hex_marker") return cp(p.hex.hex_marker);
        if (n == "tet_det") return cp(p.tt.det);
        if (n == "tet_centroid") return cp(p.tt.centroid);
        if (n == "hex_coeffs") return cp(p.hex_coeffs);
        if (n == "nbr_ptr") return cp(p.tt.nbr_ptr);
        if (n == "nbr_idx") return cp(p.tt.nbr_idx);
        if (n == "quad_nodes") return cp(p.tt.quad_nodes);
        if (n == "voro_ptr") return cp(p.voro_ptr);
        if (n == "voro_idx") return cp(p.voro_idx);
        if (n == "vac_node2vertex") return cp(p.vac.node2vertex);
        if (n == "vac_cells") return cp(p.vac.cells);
        if (n == "surf_tris") return cp(p.surf.tris);
        if (n == "surf_tri2tet") return cp(p.surf.tri2tet);
        if (n == "surf_geo") return cp(p.surf.geo);
        if (n == "surf_nbr_ptr") return cp(p.surf.nbr_ptr);
        if (n == "surf_nbr_idx") return cp(p.surf.nbr_idx);
        if (n == "tet_search") {
            std::vector<int32_t> v(p.tt.search.begin(), p.tt.search.end());
            return cp(v);
        }
        if (n == "edgemax") {
            std::memcpy(out, &p.edgemax, sizeof(double));
            return 0;
        }
        set_last_error("unknown table " + n);
        return 1;
    });
}

int64_t fgb_synth_atoms(const FgbNanotip* spec, double a, double sigma, double cutoff, uint64_t seed, double* xyz,
                        int* type) {
    try {
        AtomSet at = make_nanotip_atoms(to_spec(spec), a, sigma, cutoff, seed);
        const int64_t n = (int64_t)at.type.size();
        if (xyz) std::memcpy(xyz, at.xyz.data(), sizeof(double) * 3 * n);
        if (type) std::memcpy(type, at.type.data(), sizeof(int) * n);
        return n;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return -1;
    }
}

int64_t fgb_synth_probes(const FgbNanotip* spec, int n, uint64_t seed, double* xyz) {
    try {
        std::vector<double> p = make_vacuum_probes(to_spec(spec), n, seed);
        if (xyz) std::memcpy(xyz, p.data(), sizeof(double) * p.size());
        return n;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return -1;
    }
}

// ---------------------------------------------------------------- Part 2: device field
FGB_FIELD* fgb_field_create(const FGB_MESH* m) { return fgb_field_create_order(m, 1); }
FGB_FIELD* fgb_field_create_order(const FGB_MESH* m, int order) {
    FGB_FIELD* f = new FGB_FIELD;
    const int rc = guarded([&] {
        f->pm = m->pm;
        f->owned.reset(new Field(f->pm, nullptr, order));
        f->f = f->owned.get();
        f->mesh = f->pm.get();
        return 0;
    });
    if (rc) { delete f; return nullptr; }
    return f;
}
void fgb_field_free(FGB_FIELD* f) { delete f; }

int fgb_field_sizes(const FGB_FIELD* f, int64_t* o) {
    return guarded([&] {
        const FemStructure& s = f->f->fem().structure();
        o[0] = s.n_dofs;
        o[1] = s.nnz();
        o[2] = s.n_top_faces();
        o[3] = s.slice_ptr.back();
        return 0;
    });
}
int fgb_field_setup(FGB_FIELD* f, double applied_field, double applied_potential) {
    return guarded([&] { f->f->fem().setup(applied_field, applied_potential); return 0; });
}
int fgb_field_assemble(FGB_FIELD* f, int full_run, int anode_dirichlet) {
    return guarded([&] { f->f->fem().assemble(full_run != 0, anode_dirichlet != 0); return 0; });
}
int fgb_field_solve(FGB_FIELD* f, int precision, double rel_tol, double abs_tol, int max_iter, double inner_tol,
                    double* stats6) {
    int rc = 0;
    const int g = guarded([&] {
        SolveOptions o;
        o.precision = precision;
        o.rel_tol = rel_tol;
        o.abs_tol = abs_tol;
        o.max_iter = max_iter;
        if (inner_tol > 0) o.inner_tol = inner_tol;
        else if (precision == 3) o.inner_tol = 1e-3;
        rc = f->f->fem().solve(o, &f->last);
        if (stats6) {
            stats6[0] = f->last.iterations;
            stats6[1] = f->last.outer;
            stats6[2] = f->last.status;
            stats6[3] = f->last.rel_residual;
            stats6[4] = f->last.bnorm;
            stats6[5] = f->last.ms;
            if (stats6[6] == -1.0) stats6[6] = f->last.kernel_ms;  // optional 7th slot on request
        }
        return 0;
    });
    return g ? INT32_MIN : rc;
}
int fgb_field_last_stats(const FGB_FIELD* f, double* out14) {
    return guarded([&] { stats13(f->last, out14); return 0; });
}
int fgb_field_set_outer_spmv(FGB_FIELD* f, int mode) {
    return guarded([&] { f->f->fem().set_outer_spmv(mode); return 0; });
}
int fgb_field_set_cell_blocks(FGB_FIELD* f, int cells_per_block, int max_dofs) {
    return guarded([&] { f->f->fem().set_cell_blocks(cells_per_block, max_dofs); return 0; });
}
double fgb_field_outer_spmv_bytes(const FGB_FIELD* f) {
    double b = -1;
    guarded([&] { b = f->f->fem().outer_spmv_bytes(); return 0; });
    return b;
}
int fgb_field_set_level0_ebe(FGB_FIELD* f, int on) {
    return guarded([&] { f->f->fem().set_level0_ebe(on != 0); return 0; });
}
int fgb_field_set_ke_tensor(FGB_FIELD* f, int on) {
    return guarded([&] { f->f->fem().set_ke_tensor(on != 0); return 0; });
}
long long fgb_field_export_element_matrices(FGB_FIELD* f, double* out) {
    try {
        FemDevice& fem = f->f->fem();
        if (out) fem.export_element_matrices(out);
        return (long long)fem.element_matrix_values();
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return -1;
    }
}
int fgb_field_set_level0_stream(FGB_FIELD* f, int on) {
    return guarded([&] { f->f->fem().set_level0_stream(on != 0); return 0; });
}
int fgb_field_set_level0_operator(FGB_FIELD* f, int kind) {
    int used = -1;
    const int rc = guarded([&] { used = f->f->fem().set_level0_operator(kind); return 0; });
    return rc ? -1 : used;
}
int fgb_field_set_level0_prefetch(FGB_FIELD* f, int cells) {
    return guarded([&] { f->f->fem().set_level0_prefetch(cells); return 0; });
}
int fgb_field_set_coarse_cycles(FGB_FIELD* f, int level, int cycles) {
    return guarded([&] { f->f->fem().set_coarse_cycles(level, cycles); return 0; });
}
int fgb_field_set_lazy_matrix(FGB_FIELD* f, int on) {
    return guarded([&] { f->f->fem().set_lazy_matrix(on != 0); return 0; });
}
int fgb_field_set_level_smoothing(FGB_FIELD* f, int level, int degree, double lo) {
    return guarded([&] { f->f->fem().set_level_smoothing(level, degree, lo); return 0; });
}
int fgb_field_set_smoothing(FGB_FIELD* f, int degree, double lo) {
    return guarded([&] { f->f->fem().set_smoothing(degree, lo); return 0; });
}
int fgb_field_set_profiling(FGB_FIELD* f, int on) {
    return guarded([&] { f->f->fem().set_profiling(on != 0); return 0; });
}
int fgb_field_amg_levels(FGB_FIELD* f, char* buf, int cap) {
    return guarded([&] {
        const std::string d = f->f->fem().amg_levels();
        if (cap > 0) {
            const size_t n = std::min(d.size(), (size_t)cap - 1);
            d.copy(buf, n);
            buf[n] = 0;
        }
        return 0;
    });
}
int fgb_field_export_phi_nodes(FGB_FIELD* f, double* phi) {
    return guarded([&] {
        FemDevice& fem = f->f->fem();
        std::vector<double> x(fem.n_dofs());
        FGB_CUDA(cudaMemcpyAsync(x.data(), fem.d_solution(), sizeof(double) * x.size(), cudaMemcpyDeviceToHost, fem.stream()));
        FGB_CUDA(cudaStreamSynchronize(fem.stream()));
        const FemStructure& s = fem.structure();
        std::fill(phi, phi + f->mesh->hex.n_nodes(), 0.0);
        for (int d = 0; d < s.n_dofs; ++d)
            if (s.dof2node[d] >= 0) phi[s.dof2node[d]] = x[d];  // Q2: only vertex DoFs sit on nodes
        return 0;
    });
}
int fgb_field_space_charge(FGB_FIELD* f, int n, const double* d_xyz, const int* d_hex, double charge_factor,
                           int accumulate, int* n_skipped) {
    return guarded([&] {
        const int sk = f->f->space_charge(n, d_xyz, d_hex, charge_factor, accumulate != 0);
        if (n_skipped) *n_skipped = sk;
        return 0;
    });
}
int fgb_device_sync(void) {
    return guarded([&] { FGB_CUDA(cudaDeviceSynchronize()); return 0; });
}
int fgb_tc_selftest(double* max_err) {
    return guarded([&] { *max_err = tc_selftest(); return 0; });
}
int fgb_device_info(size_t* free_bytes, size_t* total_bytes, char* uuid) {
    return guarded([&] {
        size_t fr = 0, tot = 0;
        FGB_CUDA(cudaMemGetInfo(&fr, &tot));
        if (free_bytes) *free_bytes = fr;
        if (total_bytes) *total_bytes = tot;
        if (uuid) {
            int dev = 0;
            FGB_CUDA(cudaGetDevice(&dev));
            cudaDeviceProp p;
            FGB_CUDA(cudaGetDeviceProperties(&p, dev));
            const unsigned char* b = reinterpret_cast<const unsigned char*>(p.uuid.bytes);
            // the form nvidia-smi prints: GPU-8-4-4-4-12 hex digits
            std::snprintf(uuid, 48, "GPU-%02x%02x%02x%02x-%02x%02x-%02x%02x-%02x%02x-%02x%02x%02x%02x%02x%02x", b[0],
                          b[1], b[2], b[3], b[4], b[5], b[6], b[7], b[8], b[9], b[10], b[11], b[12], b[13], b[14],
                          b[15]);
        }
        return 0;
    });
}
int fgb_field_clear_space_charge(FGB_FIELD* f) {
    return guarded([&] { f->f->fem().clear_space_charge(); return 0; });
}
int fgb_field_export_solution(FGB_FIELD* f, double* x) {
    return guarded([&] {
        FemDevice& fem = f->f->fem();
        FGB_CUDA(cudaMemcpyAsync(x, fem.d_solution(), sizeof(double) * fem.n_dofs(), cudaMemcpyDeviceToHost, fem.stream()));
        FGB_CUDA(cudaStreamSynchronize(fem.stream()));
        return 0;
    });
}
int fgb_field_import_phi_nodes(FGB_FIELD* f, const double* phi) {
    return guarded([&] {
        FemDevice& fem = f->f->fem();
        const FemStructure& s = fem.structure();
        std::vector<double> x(s.n_dofs);
        const PreparedMesh& pm = *f->mesh;
        for (int d = 0; d < s.n_dofs; ++d) {
            if (s.dof2node[d] >= 0) {
                x[d] = phi[s.dof2node[d]];
            } else {
                // Q2 edge/face/interior DoF: the trilinear interpolant of the nodal values,
                // i.e. the mean over the corners of its entity
                int cr[8];
                const int nk = q2_entity_corners(s.dof_local[d], cr);
                const int hex = pm.vac.cells[s.dof_cell[d]];
                double acc = 0.0;
                for (int q = 0; q < nk; ++q) acc += phi[pm.hex.hexs[8 * (size_t)hex + cr[q]]];
                x[d] = acc / nk;
            }
        }
        FGB_CUDA(cudaMemcpyAsync(fem.d_solution(), x.data(), sizeof(double) * x.size(), cudaMemcpyHostToDevice, fem.stream()));
        FGB_CUDA(cudaStreamSynchronize(fem.stream()));
        return 0;
    });
}
int fgb_field_extract(FGB_FIELD* f, int smoothen) {
    return guarded([&] {
        f->f->extract(smoothen != 0);
        FGB_CUDA(cudaStreamSynchronize(f->f->stream()));
        return 0;
    });
}
int fgb_field_get_nodal(FGB_FIELD* f, double* sol5) {
    return guarded([&] { f->f->interp().get_solution(sol5); return 0; });
}
int fgb_field_set_nodal(FGB_FIELD* f, const double* sol5) {
    return guarded([&] {
        f->f->interp().set_solution(sol5);
        FGB_CUDA(cudaStreamSynchronize(f->f->stream()));
        return 0;
    });
}
int fgb_field_interpolate(FGB_FIELD* f, int n, const double* xyz, int rank, int* cells, double* out5, int64_t* st5) {
    return guarded([&] {
        LocateStats ls;
        f->f->interpolate_host(n, xyz, rank, cells, out5, st5 ? &ls : nullptr);
        if (st5) {
            st5[0] = ls.n_points;
            st5[1] = ls.n_walk_failed;
            st5[2] = ls.n_fallback;
            st5[3] = ls.n_dependent;
            st5[4] = ls.longest_run;
        }
        return 0;
    });
}
int fgb_field_interpolate_surface(FGB_FIELD* f, int n, const double* xyz, int rank, int* cells, double* out5) {
    return guarded([&] {
        f->f->interpolate_surface_host(n, xyz, rank, cells, out5);
        return 0;
    });
}
int fgb_field_interpolate_surface_device(FGB_FIELD* f, int n, const double* d_xyz, int rank, int* d_cells,
                                         double* d_out5) {
    return guarded([&] {
        f->f->interp().surface_interpolate(n, d_xyz, rank, d_cells, d_out5);
        return 0;
    });
}
int fgb_field_interpolate_device(FGB_FIELD* f, int n, const double* d_xyz, int rank, int* d_cells, double* d_out5) {
    return guarded([&] {
        f->f->interp().locate_interpolate(n, d_xyz, rank, d_cells, d_out5, nullptr);
        return 0;
    });
}
int fgb_field_interpolate_device_noalloc(FGB_FIELD* f, int n, const double* d_xyz, int rank, int* d_cells,
                                        double* d_out5) {
    return guarded([&] {
        f->f->interp().locate_interpolate_noalloc(n, d_xyz, rank, d_cells, d_out5);
        return 0;
    });
}
int fgb_field_export_system(FGB_FIELD* f, int64_t* rowptr, int* col, double* val, double* rhs, int* dof2node) {
    return guarded([&] {
        FemDevice& fem = f->f->fem();
        const FemStructure& s = fem.structure();
        std::vector<double> v, b;
        fem.download_matrix(v, b);
        std::vector<int64_t> rp;
        std::vector<int32_t> cl;
        if (rowptr || col) fem.download_pattern(rp, cl);
        if (rowptr) std::memcpy(rowptr, rp.data(), sizeof(int64_t) * rp.size());
        if (col) std::memcpy(col, cl.data(), sizeof(int32_t) * cl.size());
        if (val) std::memcpy(val, v.data(), sizeof(double) * v.size());
        if (rhs) std::memcpy(rhs, b.data(), sizeof(double) * b.size());
        if (dof2node) std::memcpy(dof2node, s.dof2node.data(), sizeof(int32_t) * s.dof2node.size());
        return 0;
    });
}
int fgb_field_q2_dofs(FGB_FIELD* f, int* dof_cell, int* dof_local) {
    return guarded([&] {
        const FemStructure& s = f->f->fem().structure();
        FGB_REQUIRE(s.order == 2, "not a Q2 field");
        for (int d = 0; d < s.n_dofs; ++d) {
            if (dof_cell) dof_cell[d] = s.dof_cell[d];
            if (dof_local) dof_local[d] = s.dof_local[d];
        }
        return 0;
    });
}
uint64_t fgb_mesh_structure_digest(const FGB_MESH* m, int order, int region) {
    uint64_t h = 1469598103934665603ull;
    guarded([&] {
        const FemStructure s = order == 2 ? build_q2_structure(*m->pm) : build_fem_structure(*m->pm, region);
        fnv(h, s.dof2node); fnv(h, s.node2dof); fnv(h, s.cell_dofs); fnv(h, s.rowptr); fnv(h, s.col);
        fnv(h, s.r2c_ptr); fnv(h, s.r2c_item); fnv(h, s.top_faces); fnv(h, s.r2f_ptr); fnv(h, s.r2f_item);
        fnv(h, s.bc_kind); fnv(h, s.slice_ptr); fnv(h, s.slice_len); fnv(h, s.csr2sell); fnv(h, s.sell_col);
        fnv(h, s.row_len); fnv(h, s.dof_xyz); fnv(h, s.dof_cell); fnv(h, s.dof_local);
        return 0;
    });
    return h;
}
int fgb_mesh_q1_sizes(const FGB_MESH* m, int64_t* out4) {
    return guarded([&] {
        FemStructure s = build_fem_structure(*m->pm);
        int mx = 0;
        for (int v : s.row_len) mx = std::max(mx, v);
        out4[0] = s.n_dofs;
        out4[1] = s.nnz();
        out4[2] = s.n_top_faces();
        out4[3] = mx;
        return 0;
    });
}
int fgb_mesh_cell_blocks(const FGB_MESH* m, int cells_per_block, int max_dofs, int64_t* out8) {
    return guarded([&] {
        const FemStructure s = build_q2_structure(*m->pm);
        const CellBlocks cb = build_cell_blocks(s, cells_per_block, max_dofs);
        const uint64_t h = validate_cell_blocks(s, cb, cells_per_block, max_dofs);
        out8[0] = cb.n_blocks;
        out8[1] = cb.max_cells;
        out8[2] = cb.max_dofs;
        out8[3] = cb.local_entries();
        out8[4] = cb.n_slots;
        out8[5] = (int64_t)cb.bnd_dofs.size();
        out8[6] = s.n_dofs - (int64_t)cb.bnd_dofs.size();
        std::memcpy(&out8[7], &h, sizeof(h));
        return 0;
    });
}
int fgb_mesh_q2_sizes(const FGB_MESH* m, int64_t* out4) {
    return guarded([&] {
        FemStructure s = build_q2_structure(*m->pm);
        int mx = 0;
        for (int v : s.row_len) mx = std::max(mx, v);
        out4[0] = s.n_dofs;
        out4[1] = s.nnz();
        out4[2] = s.n_top_faces();
        out4[3] = mx;
        return 0;
    });
}
double fgb_field_time_spmv(FGB_FIELD* f, int precision, int reps) {
    double ms = -1;
    guarded([&] { ms = f->f->fem().time_spmv(precision, reps); return 0; });
    return ms;
}
void* fgb_field_stream(FGB_FIELD* f) { return (void*)f->f->stream(); }

int fgb_field_mark(FGB_FIELD* f, int slot) {
    return guarded([&] {
        FGB_REQUIRE(slot >= 0 && slot < 8, "event slot out of range");
        if (!f->ev[slot]) FGB_CUDA(cudaEventCreate(&f->ev[slot]));
        FGB_CUDA(cudaEventRecord(f->ev[slot], f->f->stream()));
        return 0;
    });
}
double fgb_field_elapsed(FGB_FIELD* f, int a, int b) {
    double ms = -1;
    guarded([&] {
        FGB_REQUIRE(a >= 0 && a < 8 && b >= 0 && b < 8 && f->ev[a] && f->ev[b], "unrecorded event slot");
        FGB_CUDA(cudaEventSynchronize(f->ev[b]));
        float m = 0;
        FGB_CUDA(cudaEventElapsedTime(&m, f->ev[a], f->ev[b]));
        ms = m;
        return 0;
    });
    return ms;
}
void* fgb_device_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
        set_last_error("cudaMalloc failed");
        return nullptr;
    }
    return p;
}
void fgb_device_free(void* p) { cudaFree(p); }
int fgb_memcpy_htod(void* dst, const void* src, size_t bytes) {
    return guarded([&] { FGB_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice)); return 0; });
}
int fgb_memcpy_dtoh(void* dst, const void* src, size_t bytes) {
    return guarded([&] { FGB_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost)); return 0; });
}

FGB_FIELD* femocs_field(FEMOCS* h) {
    FGB_FIELD* f = new FGB_FIELD;
    const int rc = guarded([&] {
        Field* fd = h->f->field();
        if (!fd) throw Error("no field yet: call femocs_run first");
        f->f = fd;
        f->mesh = &fd->mesh();
        return 0;
    });
    if (rc) { delete f; return nullptr; }
    return f;
}


// ---------------------------------------------------------------- Part 5: current and heat
FGB_HEAT* fgb_heat_create(const FGB_MESH* m) {
    FGB_HEAT* h = new FGB_HEAT;
    const int rc = guarded([&] {
        h->pm = m->pm;
        h->b.reset(new BulkSolver(h->pm));
        return 0;
    });
    if (rc) { delete h; return nullptr; }
    return h;
}
void fgb_heat_free(FGB_HEAT* h) { delete h; }
int fgb_heat_sizes(FGB_HEAT* h, int64_t* out3) {
    return guarded([&] {
        out3[0] = h->b->n_dofs();
        out3[1] = h->b->nnz();
        out3[2] = h->b->n_faces();
        return 0;
    });
}
int fgb_heat_surface_faces(FGB_HEAT* h, double* centroid3, int* hex_face2) {
    return guarded([&] { h->b->surface_faces(centroid3, hex_face2); return 0; });
}
int fgb_heat_set_resistivity(FGB_HEAT* h, int n, const double* T, const double* rho) {
    return guarded([&] {
        FGB_REQUIRE(n >= 2 && T && rho, "resistivity table needs >= 2 points");
        h->b->set_resistivity(std::vector<double>(T, T + n), std::vector<double>(rho, rho + n));
        return 0;
    });
}
int fgb_heat_setup(FGB_HEAT* h, double t_ambient, double lorentz, double rho_cp) {
    return guarded([&] { h->b->setup(t_ambient, lorentz, rho_cp); return 0; });
}
static int heat_solve(FGB_HEAT* h, bool heat, double dt, const double* vals, int precision, double rel_tol, int max_iter,
                      double* stats14) {
    int rc = 0;
    const int g = guarded([&] {
        SolveOptions o;
        o.precision = precision;
        o.rel_tol = rel_tol;
        o.max_iter = max_iter;
        rc = heat ? h->b->solve_heat(dt, vals, o, &h->last) : h->b->solve_current(vals, o, &h->last);
        if (stats14) stats13(h->last, stats14);
        return 0;
    });
    return g ? INT32_MIN : rc;
}
int fgb_heat_solve_current(FGB_HEAT* h, const double* face_j, int precision, double rel_tol, int max_iter,
                           double* stats14) {
    return heat_solve(h, false, 0.0, face_j, precision, rel_tol, max_iter, stats14);
}
int fgb_heat_solve_heat(FGB_HEAT* h, double delta_time_s, const double* face_q, int precision, double rel_tol,
                        int max_iter, double* stats14) {
    return heat_solve(h, true, delta_time_s, face_q, precision, rel_tol, max_iter, stats14);
}
int fgb_heat_export(FGB_HEAT* h, double* T_node, double* phi_node) {
    return guarded([&] { h->b->export_nodes(T_node, phi_node); return 0; });
}
int fgb_heat_temperature_range(FGB_HEAT* h, double* out2) {
    return guarded([&] { h->b->temperature_range(out2, out2 + 1); return 0; });
}

}  // extern "C"

// ---------------------------------------------------------------- Part 3: batches
FGB_BATCH* fgb_batch_create(int use_graph, int autotune, int grid_ctas) {
    FGB_BATCH* b = new FGB_BATCH;
    const int rc = guarded([&] {
        BatchOptions o;
        o.use_graph = use_graph != 0;
        o.persistent = use_graph == 2;
        o.autotune = autotune != 0;
        o.grid_ctas = grid_ctas;
        b->b.reset(new BatchSolver(o));
        return 0;
    });
    if (rc) { delete b; return nullptr; }
    return b;
}
void fgb_batch_free(FGB_BATCH* b) { delete b; }

int fgb_batch_add_mesh(FGB_BATCH* b, const FGB_MESH* m, double hbm_reserve) {
    int slot = INT32_MIN;
    const int rc = guarded([&] {
        slot = b->b->add_mesh(m->pm, (size_t)std::max(0.0, hbm_reserve));
        return 0;
    });
    return rc ? INT32_MIN : slot;
}

int fgb_batch_add_synthetic(FGB_BATCH* b, int n, const FgbNanotip* specs, int n_threads, double hbm_reserve,
                            int* slots) {
    return guarded([&] {
        const int nt = std::max(1, std::min(n_threads > 0 ? n_threads : (int)std::thread::hardware_concurrency(), n));
        std::vector<std::string> errors(nt);
        std::atomic<int> next{0};
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t)
            pool.emplace_back([&, t] {
                omp_set_num_threads(1);  // the meshes are the parallelism: no nested teams
                try {
                    for (int i = next++; i < n; i = next++) {
                        auto pm = std::make_shared<PreparedMesh>(prepare_mesh(make_nanotip_mesh(to_spec(&specs[i]))));
                        slots[i] = b->b->add_mesh(pm, (size_t)std::max(0.0, hbm_reserve));
                    }
                } catch (const std::exception& e) {
                    errors[t] = e.what();
                }
            });
        for (auto& th : pool) th.join();
        for (auto& e : errors)
            if (!e.empty()) throw Error(e);
        return 0;
    });
}

int fgb_batch_remove_mesh(FGB_BATCH* b, int slot) {
    return guarded([&] { b->b->remove_mesh(slot); return 0; });
}
int fgb_batch_admit(FGB_BATCH* b, int slot, double E0, double rel_tol, int max_iter) {
    return guarded([&] { b->b->admit(slot, E0, rel_tol, max_iter); return 0; });
}
int fgb_batch_step(FGB_BATCH* b, int max_iters) {
    int still = 0;
    const int rc = guarded([&] { still = b->b->step(max_iters); return 0; });
    return rc ? INT32_MIN : still;
}
int fgb_batch_collect(FGB_BATCH* b, int cap, int* slots, double* res4) {
    int n = 0;
    const int rc = guarded([&] {
        auto fin = b->b->collect_finished();
        FGB_REQUIRE((int)fin.size() <= cap, "result arrays too small for the finished solves");
        for (auto& f : fin) {
            slots[n] = f.first;
            res4[4 * n] = f.second.iterations;
            res4[4 * n + 1] = f.second.status;
            res4[4 * n + 2] = f.second.rel_residual;
            res4[4 * n + 3] = f.second.bnorm;
            ++n;
        }
        return 0;
    });
    return rc ? INT32_MIN : n;
}
int fgb_batch_extract(FGB_BATCH* b, int slot, int smoothen) {
    return guarded([&] { b->b->extract(slot, smoothen != 0); return 0; });
}
int fgb_batch_interpolate(FGB_BATCH* b, int slot, int n, const double* d_xyz, int rank, int* d_cells, double* d_out5) {
    return guarded([&] {
        b->b->interp(slot).locate_interpolate(n, d_xyz, rank, d_cells, d_out5, nullptr);
        return 0;
    });
}
int fgb_batch_sync_slot(FGB_BATCH* b, int slot) {
    return guarded([&] { FGB_CUDA(cudaStreamSynchronize(b->b->slot_stream(slot))); return 0; });
}
int fgb_batch_export_phi_nodes(FGB_BATCH* b, int slot, double* phi) {
    return guarded([&] { b->b->export_phi_nodes(slot, phi); return 0; });
}
int fgb_batch_export_nodal(FGB_BATCH* b, int slot, double* sol5) {
    return guarded([&] {
        FGB_CUDA(cudaStreamSynchronize(b->b->slot_stream(slot)));
        b->b->interp(slot).get_solution(sol5);
        return 0;
    });
}
int fgb_batch_reset_solution(FGB_BATCH* b, int slot) {
    return guarded([&] { b->b->reset_solution(slot); return 0; });
}
int fgb_batch_true_residual(FGB_BATCH* b, int slot, double* out) {
    return guarded([&] { *out = b->b->true_residual(slot); return 0; });
}
int fgb_batch_info(FGB_BATCH* b, int slot, int64_t* out4) {
    return guarded([&] {
        out4[0] = b->b->n_dofs(slot);
        out4[1] = b->b->n_nodes(slot);
        out4[2] = b->b->levels(slot);
        out4[3] = 0;
        return 0;
    });
}
int fgb_batch_stats(FGB_BATCH* b, double* out6) {
    return guarded([&] {
        out6[0] = (double)b->b->total_rows();
        out6[1] = (double)b->b->device_bytes();
        out6[2] = b->b->last_iterations();
        out6[3] = b->b->body_kernels();
        out6[4] = (double)b->b->launches();
        out6[5] = b->b->n_slots();
        return 0;
    });
}
int fgb_batch_mark(FGB_BATCH* b, int k) {
    return guarded([&] { b->b->mark(k); return 0; });
}
double fgb_batch_elapsed(FGB_BATCH* b, int k0, int k1) {
    double ms = -1;
    guarded([&] { ms = b->b->elapsed_ms(k0, k1); return 0; });
    return ms;
}
int fgb_batch_tuning(FGB_BATCH* b, char* buf, int cap) {
    return guarded([&] {
        const std::string d = b->b->tuning();
        if (cap > 0) {
            const size_t n = std::min(d.size(), (size_t)cap - 1);
            d.copy(buf, n);
            buf[n] = 0;
        }
        return 0;
    });
}

long long fgb_nanotip_vacuum_hexes(const FgbNanotip* spec) {
    long long n = -1;
    guarded([&] { n = nanotip_vacuum_hexes(to_spec(spec)); return 0; });
    return n;
}
double fgb_nanotip_fit_spacing(const FgbNanotip* spec, double target_hexes) {
    double h = -1;
    guarded([&] { h = fit_nanotip_spacing(to_spec(spec), (long long)target_hexes); return 0; });
    return h;
}

// ---------------------------------------------------------------- Part 4: serving
FGB_SERVER* fgb_server_create(FGB_BATCH* b, double rel_tol, int max_iter, int iters_per_launch, int rank, int smoothen,
                              double hbm_reserve) {
    FGB_SERVER* s = new FGB_SERVER;
    const int rc = guarded([&] {
        ServerOptions o;
        o.rel_tol = rel_tol;
        o.max_iter = max_iter;
        o.iters_per_launch = std::max(1, iters_per_launch);
        o.rank = rank;
        o.smoothen = smoothen != 0;
        o.hbm_reserve = std::max(0.0, hbm_reserve);
        s->s.reset(new FieldServer(*b->b, o));
        return 0;
    });
    if (rc) { delete s; return nullptr; }
    return s;
}
void fgb_server_free(FGB_SERVER* s) { delete s; }
int fgb_server_set_launch_policy(FGB_SERVER* s, int idle_iters, int stop_at_first) {
    return guarded([&] { s->s->set_launch_policy(idle_iters, stop_at_first != 0); return 0; });
}

int fgb_server_add_run(FGB_SERVER* s, const FGB_MESH* m, const double* xyz, int n_atoms, unsigned long long seed) {
    int id = INT32_MIN;
    const int rc = guarded([&] { id = s->s->add_run(m->pm, xyz, n_atoms, seed); return 0; });
    return rc ? INT32_MIN : id;
}

int fgb_server_add_synthetic_runs(FGB_SERVER* s, int n, const FgbNanotip* specs, int n_atoms, unsigned long long seed,
                                  int n_threads) {
    return guarded([&] {
        // meshes and atoms on host threads; atoms = the tip's surface atoms (every k-th when
        // there are more than n_atoms) topped up with random vacuum probes
        const int nt = std::max(1, std::min(n_threads > 0 ? n_threads : (int)std::thread::hardware_concurrency(), n));
        std::vector<std::shared_ptr<PreparedMesh>> pms(n);
        std::vector<std::vector<double>> pts(n);
        std::vector<std::string> err(nt);
        std::atomic<int> next{0};
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t)
            pool.emplace_back([&, t] {
                omp_set_num_threads(1);  // the meshes are the parallelism: no nested teams
                try {
                    for (int i = next++; i < n; i = next++) {
                        const NanotipSpec sp = to_spec(&specs[i]);
                        pms[i] = std::make_shared<PreparedMesh>(prepare_mesh(make_nanotip_mesh(sp)));
                        AtomSet at = make_nanotip_atoms(sp, 3.615, 0.05, 3.1, seed + 7919ull * i);
                        std::vector<double> surf;
                        for (size_t a = 0; a < at.type.size(); ++a)
                            if (at.type[a] == kSurface)
                                surf.insert(surf.end(), &at.xyz[3 * a], &at.xyz[3 * a] + 3);
                        const size_t ns = surf.size() / 3;
                        std::vector<double>& p = pts[i];
                        if (ns >= (size_t)n_atoms) {
                            for (int k = 0; k < n_atoms; ++k) {
                                const size_t a = (size_t)k * ns / n_atoms;
                                p.insert(p.end(), &surf[3 * a], &surf[3 * a] + 3);
                            }
                        } else {
                            p = surf;
                            std::vector<double> pr = make_vacuum_probes(sp, n_atoms - (int)ns, seed + 104729ull * i);
                            p.insert(p.end(), pr.begin(), pr.end());
                        }
                    }
                } catch (const std::exception& e) {
                    err[t] = e.what();
                }
            });
        for (auto& th : pool) th.join();
        for (auto& e : err)
            if (!e.empty()) throw Error(e);
        for (int i = 0; i < n; ++i) s->s->add_run(pms[i], pts[i].data(), (int)(pts[i].size() / 3), seed + 31ull * i);
        s->s->place_pending(n_threads);
        return 0;
    });
}

int fgb_server_place_pending(FGB_SERVER* s, int n_threads) {
    int placed = INT32_MIN;
    const int rc = guarded([&] { placed = s->s->place_pending(n_threads); return 0; });
    return rc ? INT32_MIN : placed;
}
long long fgb_server_submit(FGB_SERVER* s, int run, double E0, double sigma) {
    long long id = -1;
    const int rc = guarded([&] { id = s->s->submit(run, E0, sigma); return 0; });
    return rc ? -1 : id;
}
int fgb_server_start(FGB_SERVER* s) {
    return guarded([&] { s->s->start(); return 0; });
}
int fgb_server_stop(FGB_SERVER* s) {
    return guarded([&] { s->s->stop(); return 0; });
}
int fgb_server_drain(FGB_SERVER* s, double timeout_s) {
    int ok = 0;
    const int rc = guarded([&] { ok = s->s->drain(timeout_s) ? 1 : 0; return 0; });
    return rc ? -1 : (ok ? 0 : 2);
}
int fgb_server_run_poisson(FGB_SERVER* s, double rate, int n, double sigma, unsigned long long seed,
                           const double* base_fields) {
    return guarded([&] {
        std::vector<double> bf(base_fields, base_fields + s->s->n_runs());
        s->s->run_poisson(rate, n, sigma, seed, bf);
        return 0;
    });
}
int fgb_server_records(FGB_SERVER* s, int cap, double* out10) {
    int n = 0;
    const int rc = guarded([&] {
        auto rec = s->s->records();
        for (auto& r : rec) {
            if (n >= cap) break;
            double* o = out10 + 10 * (size_t)n;
            o[0] = (double)r.id; o[1] = r.run; o[2] = r.E0; o[3] = r.iterations; o[4] = r.status;
            o[5] = r.rel_residual; o[6] = r.t_submit; o[7] = r.t_admit; o[8] = r.t_solved; o[9] = r.t_done;
            ++n;
        }
        return 0;
    });
    return rc ? INT32_MIN : n;
}
int fgb_server_clear_records(FGB_SERVER* s) {
    return guarded([&] { s->s->clear_records(); return 0; });
}
int fgb_server_last_result(FGB_SERVER* s, int run, double* out5, int* cells) {
    return guarded([&] { s->s->last_result(run, out5, cells); return 0; });
}
int fgb_server_reset_run(FGB_SERVER* s, int run) {
    return guarded([&] { s->s->reset_run(run); return 0; });
}
int fgb_server_info(FGB_SERVER* s, double* out4) {
    return guarded([&] {
        out4[0] = s->s->n_runs();
        out4[1] = (double)s->s->admitted_launches();
        out4[2] = s->s->max_in_flight();
        out4[3] = 0;
        return 0;
    });
}
int fgb_server_run_info(FGB_SERVER* s, int run, int64_t* out2) {
    return guarded([&] {
        out2[0] = s->s->run_slot(run);
        out2[1] = s->s->n_atoms(run);
        return 0;
    });
}
