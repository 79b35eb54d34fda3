#include "facade.h"
#include "mesh_prep.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <fstream>
#include <sstream>

#include "synth.h"

namespace fgb {

// ------------------------------------------------------------------ configuration script
namespace {
const std::string kComment = "!#%";
const std::string kData = "+-/*_.0123456789abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ()";
std::string lower(std::string s) {
    std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    return s;
}
}  // namespace

void ConfigScript::parse_text(const std::string& text) {
    std::istringstream in(text);
    std::string line;
    while (std::getline(in, line)) {
        line += " ";
        bool started = true;
        while (!line.empty()) {
            // drop everything before the first data or comment symbol
            size_t p = line.find_first_of(kComment + kData);
            if (p == std::string::npos) break;
            line.erase(0, p);
            if (kComment.find(line[0]) != std::string::npos) break;
            size_t i = line.find_first_not_of(kData);
            if (i == std::string::npos) i = line.size();
            if (i == 0) break;
            std::string tok = line.substr(0, i);
            if (started && tok == "femocs_end") return;
            if (started) {
                data_.push_back({lower(tok)});
            } else {
                data_.back().push_back(tok);
            }
            line = line.substr(i);
            started = false;
        }
    }
}

void ConfigScript::parse_file(const std::string& path) {
    std::ifstream f(path);
    FGB_REQUIRE(f.is_open(), "configuration file not found: " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    data_.clear();
    parse_text(ss.str());
}

bool ConfigScript::get(const std::string& key, std::string& v) const {
    const std::string k = lower(key);
    for (const auto& c : data_)
        if (c.size() >= 2 && c[0] == k) { v = c[1]; return true; }
    return false;
}
bool ConfigScript::get(const std::string& key, double& v) const {
    std::string s;
    if (!get(key, s)) return false;
    std::istringstream is(s);
    double r;
    if (is >> r) { v = r; return true; }
    return false;
}
bool ConfigScript::get(const std::string& key, int& v) const {
    std::string s;
    if (!get(key, s)) return false;
    std::istringstream is(s);
    int r;
    if (is >> r) { v = r; return true; }
    return false;
}
bool ConfigScript::get(const std::string& key, bool& v) const {
    std::string s;
    if (!get(key, s)) return false;
    std::string l = lower(s);
    if (l == "true") { v = true; return true; }
    if (l == "false") { v = false; return true; }
    std::istringstream is(s);
    int r;
    if (is >> r) { v = r != 0; return true; }
    return false;
}
int ConfigScript::get_args(const std::string& key, std::vector<double>& args) const {
    const std::string k = lower(key);
    int n = 0;
    for (const auto& c : data_)
        if (c.size() >= 2 && c[0] == k)
            for (size_t i = 0; i < args.size() && i + 1 < c.size(); ++i) {
                std::istringstream is(c[i + 1]);
                double r;
                if (is >> r) { args[i] = r; ++n; }
            }
    return n;
}

void ConfigScript::set(const std::string& key, const std::string& v) {
    const std::string k = lower(key);
    for (auto& c : data_)
        if (!c.empty() && c[0] == k) { c = {k, v}; return; }
    data_.push_back({k, v});
}

// ------------------------------------------------------------------ facade
FemocsFacade::FemocsFacade(const std::string& conf_file) {
    if (!conf_file.empty()) conf_.parse_file(conf_file);
    read_params();
}

void FemocsFacade::read_params() {
    conf_.get("elfield", E0_);
    conf_.get("vappl", V0_);
    conf_.get("field_cgtol", cg_tol_abs_);
    conf_.get("field_ssor", ssor_);
    conf_.get("field_ncg", n_cg_);
    conf_.get("interpolation_rank", rank_);
    conf_.get("smoothen_field", smoothen_);
    std::string abc = "neumann";
    conf_.get("anode_bc", abc);
    anode_dirichlet_ = abc == "dirichlet";
    conf_.get("radius", radius_);
    // GPU-specific keys
    conf_.get("gpu_rel_tol", rel_tol_);
    std::string prec = "amg";
    conf_.get("gpu_precision", prec);
    precision_ = prec == "fp64" ? 0 : (prec == "mixed" ? 1 : (prec == "amg_mixed" ? 3 : 2));
    inner_tol_ = precision_ == 3 ? 1e-3 : 0.1;
    conf_.get("gpu_inner_tol", inner_tol_);
    conf_.get("gpu_use_abs_tol", use_abs_tol_);
    conf_.get("gpu_element_order", element_order_);
    std::string prep = "device";
    conf_.get("gpu_mesh_prep", prep);
    FGB_REQUIRE(prep == "device" || prep == "host", "gpu_mesh_prep must be device or host");
    mesh_prep_device_ = prep == "device";
    FGB_REQUIRE(element_order_ == 1 || element_order_ == 2, "gpu_element_order must be 1 or 2");
    // field_tolerance: one value t gives [1-t, 1+t], two give [min, max] (src/Config.cpp:285-292)
    std::vector<double> lim = {0.0, 0.0};
    const int n_lim = conf_.get_args("field_tolerance", lim);
    if (n_lim == 1) {
        field_min_ = 1.0 - lim[0];
        field_max_ = 1.0 + lim[0];
    } else if (n_lim == 2) {
        field_min_ = lim[0];
        field_max_ = lim[1];
    }
}

std::shared_ptr<const PreparedMesh> FemocsFacade::prepare(TetMesh&& tm) {
    if (mesh_prep_device_) return std::make_shared<PreparedMesh>(prepare_mesh_device(std::move(tm), 0));
    return std::make_shared<PreparedMesh>(prepare_mesh(std::move(tm)));
}

int FemocsFacade::ensure_mesh() {
    if (field_) return 0;
    if (!mesh_) {
        std::string mf;
        if (!conf_.get("mesh_file", mf) || mf.empty()) {
            set_last_error("no mesh: give mesh_file in the configuration or call femocs_import_mesh "
                           "(mesh generation from atoms is outside this library)");
            return 1;
        }
        if (mf == "synthetic") {
            NanotipSpec s;
            conf_.get("radius", s.radius);
            conf_.get("tip_height", s.height);
            conf_.get("gpu_box_half", s.box_half);
            conf_.get("gpu_slab", s.slab);
            conf_.get("gpu_top", s.top);
            conf_.get("gpu_h", s.h);
            conf_.get("gpu_growth", s.growth);
            conf_.get("gpu_margin", s.margin);
            mesh_ = prepare(make_nanotip_mesh(s));
        } else {
            mesh_ = prepare(read_gmsh(mf));
        }
    }
    field_.reset(new Field(mesh_, nullptr, element_order_));
    return 0;
}

int FemocsFacade::import_mesh(int n_nodes, const double* xyz, int n_tets, const int* tets, const int* markers) {
    TetMesh tm;
    tm.xyz.assign(xyz, xyz + 3 * (size_t)n_nodes);
    tm.tets.assign(tets, tets + 4 * (size_t)n_tets);
    tm.marker.assign(markers, markers + n_tets);
    mesh_ = prepare(std::move(tm));
    field_.reset();
    solved_ = false;
    return 0;
}

int FemocsFacade::import_atoms(int n, const double* x, const double* y, const double* z, const int* types) {
    atoms_.resize(3 * (size_t)std::max(0, n));
    types_.resize(std::max(0, n));
    surf_ids_.clear();
    for (int i = 0; i < n; ++i) {
        atoms_[3 * (size_t)i] = x[i];
        atoms_[3 * (size_t)i + 1] = y[i];
        atoms_[3 * (size_t)i + 2] = z[i];
        types_[i] = types ? types[i] : kSurface;
        // Femocs::import_atoms with known types: the dense surface is the SURFACE type
        if (types_[i] == kSurface) surf_ids_.push_back(i);
    }
    surf_interp_.clear();
    surf_cells_.clear();
    return 0;
}

int FemocsFacade::import_file(const std::string& path) {
    std::ifstream in(path);
    if (!in.is_open()) { set_last_error("cannot open " + path); return 1; }
    int n = 0;
    std::string line;
    std::getline(in, line);
    n = std::atoi(line.c_str());
    std::getline(in, line);
    std::vector<double> x, y, z;
    std::vector<int> t;
    for (int i = 0; i < n && std::getline(in, line); ++i) {
        std::istringstream ls(line);
        std::string a;
        double px, py, pz;
        ls >> a >> px >> py >> pz;
        char* end = nullptr;
        long tv = std::strtol(a.c_str(), &end, 10);
        x.push_back(px);
        y.push_back(py);
        z.push_back(pz);
        t.push_back(end && *end == '\0' ? (int)tv : kSurface);
    }
    return import_atoms((int)x.size(), x.data(), y.data(), z.data(), t.data());
}

int FemocsFacade::run(int timestep, double time) {
    (void)timestep;
    (void)time;
    read_params();
    if (ensure_mesh()) return 1;
    SolveOptions opt;
    opt.precision = precision_;
    opt.rel_tol = rel_tol_;
    opt.abs_tol = use_abs_tol_ ? cg_tol_abs_ : 0.0;
    opt.max_iter = n_cg_;
    opt.inner_tol = inner_tol_;
    const int rc = field_->solve_laplace(E0_, V0_, anode_dirichlet_, opt, smoothen_, &last_);
    if (rc < 0) {
        set_last_error("field solver did not complete normally, #CG=" + std::to_string(-rc));
        return 1;
    }
    // FieldReader::check_limits over the nodal solutions (src/SolutionReader.cpp:538-556, called
    // from src/ProjectRunaway.cpp:444) with the parameters of set_check_params (:568-588):
    // tip height = z extent of the surface triangles, box height = z extent of the mesh nodes
    // (src/ProjectRunaway.cpp:354); a Dirichlet anode gives E0 = V0 / box height
    last_enhancement_ = 0.0;
    const double e0_check = anode_dirichlet_ ? V0_ / (mesh_->bbox_max[2] - mesh_->bbox_min[2]) : E0_;
    if (radius_ > 0 && field_min_ != field_max_ && e0_check != 0) {
        const double emax = field_->interp().max_field_norm();
        const double tip_h = surface_z_extent();
        double r1 = radius_, r2 = radius_;
        if (tip_h > radius_) { r2 = tip_h; r1 = std::sqrt(tip_h * radius_); }
        double g2 = 3.0;
        if (r2 > r1) {
            const double nu = r2 / r1, zeta = std::sqrt(nu * nu - 1);
            g2 = std::pow(zeta, 3.0) / (nu * std::log(zeta + nu) - zeta);
        }
        const double beta = std::fabs(std::fabs(emax / e0_check) / g2);
        last_enhancement_ = beta;
        if (beta < field_min_ || beta > field_max_) {
            set_last_error("field enhancement is out of limits, M/A=" + std::to_string(beta));
            return 1;
        }
    }
    solved_ = true;
    // ProjectRunaway::prepare_export: interpolate E and phi onto the dense surface atoms
    if (!surf_ids_.empty()) {
        std::vector<double> p(3 * surf_ids_.size());
        for (size_t k = 0; k < surf_ids_.size(); ++k)
            for (int c = 0; c < 3; ++c) p[3 * k + c] = atoms_[3 * (size_t)surf_ids_[k] + c];
        surf_cells_.resize(surf_ids_.size());
        surf_interp_.resize(5 * surf_ids_.size());
        field_->interpolate_host((int)surf_ids_.size(), p.data(), rank_, surf_cells_.data(), surf_interp_.data(), nullptr);
    }
    return 0;
}

double FemocsFacade::surface_z_extent() const {
    const std::vector<int32_t>& tris = mesh_->surf.tris;
    if (tris.empty()) return 0.0;
    double lo = 1e300, hi = -1e300;
    for (int32_t v : tris) {
        const double z = mesh_->tet.xyz[3 * (size_t)v + 2];
        lo = std::min(lo, z);
        hi = std::max(hi, z);
    }
    return hi - lo;
}

int FemocsFacade::interp_points(int n, const double* x, const double* y, const double* z, std::vector<int32_t>& cells,
                                std::vector<double>& out, bool surface) {
    if (!field_ || !solved_) { set_last_error("no solution to interpolate"); return 1; }
    std::vector<double> p(3 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        p[3 * (size_t)i] = x[i];
        p[3 * (size_t)i + 1] = y[i];
        p[3 * (size_t)i + 2] = z[i];
    }
    cells.resize(n);
    out.resize(5 * (size_t)n);
    if (surface) field_->interpolate_surface_host(n, p.data(), rank_, cells.data(), out.data());
    else field_->interpolate_host(n, p.data(), rank_, cells.data(), out.data(), nullptr);
    return 0;
}

int FemocsFacade::interpolate_surface_elfield(int n, const double* x, const double* y, const double* z, double* Ex,
                                              double* Ey, double* Ez, double* En, int* flag) {
    if (n <= 0) return 0;
    std::vector<int32_t> cells;
    std::vector<double> out;
    if (interp_points(n, x, y, z, cells, out, true)) return 1;
    for (int i = 0; i < n; ++i) {
        const double* o = &out[5 * (size_t)i];
        Ex[i] = o[0];
        Ey[i] = o[1];
        Ez[i] = o[2];
        En[i] = std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
        flag[i] = cells[i] < 0 ? 1 : 0;
    }
    return 0;
}

int FemocsFacade::interpolate_elfield(int n, const double* x, const double* y, const double* z, double* Ex, double* Ey,
                                      double* Ez, double* En, int* flag) {
    if (n <= 0) return 0;
    std::vector<int32_t> cells;
    std::vector<double> out;
    if (interp_points(n, x, y, z, cells, out)) return 1;
    for (int i = 0; i < n; ++i) {
        const double* o = &out[5 * (size_t)i];
        Ex[i] = o[0];
        Ey[i] = o[1];
        Ez[i] = o[2];
        En[i] = std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
        flag[i] = cells[i] < 0 ? 1 : 0;
    }
    return 0;
}

int FemocsFacade::interpolate_phi(int n, const double* x, const double* y, const double* z, double* phi, int* flag) {
    if (n <= 0) return 0;
    std::vector<int32_t> cells;
    std::vector<double> out;
    if (interp_points(n, x, y, z, cells, out)) return 1;
    for (int i = 0; i < n; ++i) {
        phi[i] = out[5 * (size_t)i + 4];
        flag[i] = cells[i] < 0 ? 1 : 0;
    }
    return 0;
}

namespace {
// SolutionReader::contains for the field reader labels (src/SolutionReader.cpp:269-284):
// exact label -> append (+=), upper-case variant -> overwrite; 1 vec, 2 norm, 3 scalar1, 4 scalar2
int label_kind(const std::string& label) {
    static const char* names[4] = {"elfield", "elfield_norm", "charge_density", "potential"};
    for (int k = 0; k < 4; ++k)
        if (label == names[k]) return k + 1;
    const std::string l = lower(label);
    for (int k = 0; k < 4; ++k)
        if (l == names[k]) return -(k + 1);
    return 0;
}
void export_by_label(int kind, int n, const std::vector<int32_t>& ids, const std::vector<double>& interp, double* data) {
    const bool append = kind > 0;
    const int k = std::abs(kind);
    if (!append) std::fill(data, data + (k == 1 ? 3 : 1) * (size_t)n, 0.0);
    for (size_t i = 0; i < ids.size(); ++i) {
        const int id = ids[i];
        if (id < 0 || id >= n) continue;
        const double* s = &interp[5 * i];
        if (k == 1) {
            for (int c = 0; c < 3; ++c) data[3 * (size_t)id + c] = append ? data[3 * (size_t)id + c] + s[c] : s[c];
        } else {
            double v = k == 2 ? std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]) : (k == 3 ? s[3] : s[4]);
            data[id] = append ? data[id] + v : v;
        }
    }
}
}  // namespace

int FemocsFacade::interpolate(double* data, int* flag, int n, const std::string& label, bool near_surface,
                              const double* x, const double* y, const double* z) {
    if (n <= 0) return 0;
    const int kind = label_kind(label);
    if (!kind) { set_last_error("unimplemented type of interpolation data: " + label); return 1; }
    std::vector<int32_t> cells;
    std::vector<double> out;
    if (interp_points(n, x, y, z, cells, out, near_surface)) return 1;
    std::vector<int32_t> ids(n);
    for (int i = 0; i < n; ++i) ids[i] = i;
    export_by_label(kind, n, ids, out, data);
    for (int i = 0; i < n; ++i) flag[i] = cells[i] < 0 ? 1 : 0;
    return 0;
}

int FemocsFacade::export_data(double* data, int n, const std::string& label) {
    if (n <= 0) return 0;
    const int kind = label_kind(label);
    if (!kind) { set_last_error("unimplemented type of export data: " + label); return 1; }
    if (surf_interp_.empty()) { set_last_error("no " + label + " to export"); return 1; }
    export_by_label(kind, n, surf_ids_, surf_interp_, data);
    return 0;
}

int FemocsFacade::export_int(int* data, int n, const std::string& label) {
    const std::string l = lower(label);
    if (l != "atom_type") { set_last_error("unimplemented type of export data: " + label); return 1; }
    if (label != "atom_type")
        for (int i = 0; i < n; ++i) data[i] = 0;
    return 0;
}

}  // namespace fgb
