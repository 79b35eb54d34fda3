// Host facade mirroring the reference's Femocs class (include/Femocs.h:19-193) for the
// field-solve path: configuration script, atom import, run (field solve + interpolation onto
// the surface atoms), interpolation at arbitrary points and export by label.
#pragma once

#include <map>
#include <memory>

#include "field.h"

namespace fgb {

// Key/value configuration script with the reference's parsing rules (src/Config.cpp:314-447):
// commands are lower-cased, '!', '#', '%' start comments, "femocs_end" stops reading.
class ConfigScript {
public:
    void parse_file(const std::string& path);
    void parse_text(const std::string& text);
    bool get(const std::string& key, std::string& v) const;
    bool get(const std::string& key, double& v) const;
    bool get(const std::string& key, int& v) const;
    bool get(const std::string& key, bool& v) const;
    // the numeric arguments of a command (Config::read_command with a vector,
    // src/Config.cpp:434-447): how many were read, at most args.size()
    int get_args(const std::string& key, std::vector<double>& args) const;
    void set(const std::string& key, const std::string& v);

private:
    std::vector<std::vector<std::string>> data_;
};

class FemocsFacade {
public:
    explicit FemocsFacade(const std::string& conf_file);

    int run(int timestep, double time);
    int import_atoms(int n, const double* x, const double* y, const double* z, const int* types);
    int import_file(const std::string& path);
    int import_mesh(int n_nodes, const double* xyz, int n_tets, const int* tets, const int* markers);
    int interpolate_elfield(int n, const double* x, const double* y, const double* z, double* Ex, double* Ey, double* Ez,
                            double* En, int* flag);
    int interpolate_phi(int n, const double* x, const double* y, const double* z, double* phi, int* flag);
    // Femocs::interpolate_surface_elfield (src/Femocs.cpp:198-214): E on the surface triangles
    int interpolate_surface_elfield(int n, const double* x, const double* y, const double* z, double* Ex, double* Ey,
                                    double* Ez, double* En, int* flag);
    int interpolate(double* data, int* flag, int n, const std::string& label, bool near_surface, const double* x,
                    const double* y, const double* z);
    int export_data(double* data, int n, const std::string& label);
    int export_int(int* data, int n, const std::string& label);
    int parse(const std::string& cmd, int* v) { return conf_.get(cmd, *v) ? 0 : 1; }
    int parse(const std::string& cmd, double* v) { return conf_.get(cmd, *v) ? 0 : 1; }
    int parse(const std::string& cmd, std::string& v) { return conf_.get(cmd, v) ? 0 : 1; }
    const SolveStats& last_stats() const { return last_; }
    // M/A of the last femocs_run's field-enhancement check; 0 when the check did not run
    double last_enhancement() const { return last_enhancement_; }
    int n_dofs() const { return field_ ? field_->fem().n_dofs() : 0; }
    Field* field() { return field_.get(); }

private:
    int ensure_mesh();
    // tet mesh -> prepared tables, by kernels (gpu_mesh_prep = device, default) or on the host
    std::shared_ptr<const PreparedMesh> prepare(TetMesh&& tm);
    void read_params();
    // z extent of the surface triangles' nodes (TetgenFaces stat.zbox); 0 without a surface
    double surface_z_extent() const;
    int interp_points(int n, const double* x, const double* y, const double* z, std::vector<int32_t>& cells,
                      std::vector<double>& out, bool surface = false);

    ConfigScript conf_;
    std::shared_ptr<const PreparedMesh> mesh_;
    std::unique_ptr<Field> field_;
    bool mesh_prep_device_ = true;
    bool solved_ = false;
    // atoms and the surface (dense) subset that run() interpolates onto
    std::vector<double> atoms_;
    std::vector<int32_t> types_;
    std::vector<int32_t> surf_ids_;
    std::vector<double> surf_interp_;  // 5 per surface atom
    std::vector<int32_t> surf_cells_;
    SolveStats last_;
    double last_enhancement_ = 0.0;  // M/A of the last enhancement check (0: not checked)
    // parameters (reference defaults, src/Config.cpp:17-118)
    double E0_ = 0, V0_ = 0, cg_tol_abs_ = 1e-9, ssor_ = 1.2, rel_tol_ = 1e-9, inner_tol_ = 0.1;
    int n_cg_ = 10000, rank_ = 1, precision_ = 2, element_order_ = 1;
    bool smoothen_ = true, anode_dirichlet_ = false, use_abs_tol_ = false;
    double radius_ = 0, field_min_ = 0.1, field_max_ = 5.0;
};

}  // namespace fgb
