"""The reference-facing C ABI (create_femocs / femocs_run / femocs_interpolate_* /
femocs_export_data) end to end on the GPU."""
import numpy as np
import pytest

import femocs_gb300 as fg
import oracle as orc
from oracle import pipeline

pytestmark = pytest.mark.gpu
TIP = dict(radius=10.0, height=30.0, box_half=40.0, slab=10.0, top=120.0, h=5.0, growth=1.4, margin=6.0)


def write_conf(path, extra=""):
    path.write_text(f"""mesh_file synthetic
radius {TIP['radius']}
tip_height {TIP['height']}
gpu_box_half {TIP['box_half']}
gpu_slab {TIP['slab']}
gpu_top {TIP['top']}
gpu_h {TIP['h']}
gpu_growth {TIP['growth']}
gpu_margin {TIP['margin']}
elfield -0.1
interpolation_rank 3
gpu_rel_tol 1e-12
{extra}
""")


def test_run_interpolate_export(tmp_path):
    """femocs_run + femocs_interpolate_elfield/phi + femocs_export_data through the C ABI
    against the oracle: the reference's FP64 SSOR-CG solve (to 1e-13), nodal field, smoothing
    and sequential rank-3 location/interpolation. Cells and flags bit-exact; phi and E within
    the error of a solve at the configured 1e-12 relative residual."""
    conf = tmp_path / "in.conf"
    write_conf(conf)
    fem = fg.Femocs(str(conf))
    atoms, types = fg.synth_atoms(TIP, seed=1)
    assert fem.import_atoms(atoms[:, 0], atoms[:, 1], atoms[:, 2], types) == 0
    assert fem.run() == 0
    st = fem.last_solve()
    assert st["status"] == 1 and st["rel_residual"] <= 1.05e-12
    m = fg.Mesh.synthetic(**TIP)
    sol, _ = pipeline.reference_solution(m, 0.1, rel_tol=1e-13)
    tab = pipeline.tables(m, sol)
    phi_tol = 50 * 1e-12 * np.abs(sol[:, 4]).max()
    e_tol = 500 * 1e-12 * np.linalg.norm(sol[:, :3], axis=1).max()
    pts = fg.synth_probes(TIP, 500, seed=2)
    rv, Ex, Ey, Ez, En, flag = fem.interpolate_elfield(pts[:, 0], pts[:, 1], pts[:, 2])
    assert rv == 0
    rv, phi, flag2 = fem.interpolate_phi(pts[:, 0], pts[:, 1], pts[:, 2])
    assert rv == 0 and np.array_equal(flag, flag2)
    ref_cells, ref = orc.locate_interpolate(tab, 3, pts)
    np.testing.assert_array_equal(flag, (ref_cells < 0).astype(np.int32))
    np.testing.assert_allclose(np.c_[Ex, Ey, Ez], ref[:, :3], rtol=0, atol=e_tol)
    np.testing.assert_allclose(phi, ref[:, 4], rtol=0, atol=phi_tol)
    np.testing.assert_allclose(En, np.linalg.norm(np.c_[Ex, Ey, Ez], axis=1), rtol=1e-15, atol=0)
    # export by atom id: surface atoms only, others stay zero (overwrite mode, capital label)
    rv, e = fem.export_data(len(types), "Elfield")
    assert rv == 0
    e = e.reshape(-1, 3)
    surf = types == 2
    # (a surface atom whose fallback cell is a bulk tet gets the empty value 0, as in the reference)
    assert np.all(e[~surf] == 0) and np.mean(np.linalg.norm(e[surf], axis=1) > 0) > 0.5
    sc, so = orc.locate_interpolate(tab, 3, atoms[surf])
    np.testing.assert_allclose(e[surf], so[:, :3], rtol=0, atol=e_tol)
    # append mode with the exact label adds to the caller's data
    rv, pot = fem.export_data(len(types), "potential")
    assert rv == 0
    np.testing.assert_allclose(pot[surf], so[:, 4], rtol=0, atol=phi_tol)


def test_errors_are_return_codes(tmp_path):
    conf = tmp_path / "in.conf"
    conf.write_text("elfield -0.1\n")
    fem = fg.Femocs(str(conf))
    assert fem.run() == 1  # no mesh
    assert "mesh" in fg.last_error()
    rv, *_ = fem.interpolate_elfield(np.zeros(3), np.zeros(3), np.zeros(3))
    assert rv == 1


def test_fp64_mode_and_import_mesh(tmp_path):
    conf = tmp_path / "in.conf"
    conf.write_text("elfield -0.1\ngpu_precision fp64\ngpu_rel_tol 1e-10\ninterpolation_rank 1\n")
    fem = fg.Femocs(str(conf))
    m = fg.Mesh.synthetic(**TIP)
    s = m.sizes()
    assert fem.import_mesh(m.export("node_xyz").reshape(-1, 3)[: s["n_tetnodes"]], m.export("tet_nodes"),
                           m.export("tet_marker")) == 0
    assert fem.run() == 0
    st = fem.last_solve()
    assert st["outer"] == 0 and st["status"] == 1


def analytic_enhancement(radius, tip_height):
    """FieldReader::get_analyt_enhancement (src/SolutionReader.cpp:526-536) with the radii of
    set_check_params (:579-586)."""
    r1 = r2 = radius
    if tip_height > radius:
        r2, r1 = tip_height, np.sqrt(tip_height * radius)
    if r2 <= r1:
        return 3.0
    nu = r2 / r1
    zeta = np.sqrt(nu * nu - 1)
    return zeta ** 3 / (nu * np.log(zeta + nu) - zeta)


@pytest.mark.parametrize("anode", ["neumann", "dirichlet"])
def test_field_enhancement_check(tmp_path, anode):
    """femocs_run fails (retval 1) exactly when M/A leaves the field_tolerance window
    (FieldReader::check_limits, src/SolutionReader.cpp:538-556). E0 is `elfield` for a Neumann
    anode and Vappl / box height for a Dirichlet one (set_check_params, :568-588); the tip
    height is the z extent of the surface triangles (src/ProjectRunaway.cpp:354)."""
    m = fg.Mesh.synthetic(**TIP)
    xyz = m.export("node_xyz").reshape(-1, 3)
    tris, _, _ = m.surface()
    zs = xyz[np.asarray(tris).reshape(-1), 2]
    n_tet_nodes = m.sizes()["n_tetnodes"]
    box_h = xyz[:n_tet_nodes, 2].max() - xyz[:n_tet_nodes, 2].min()
    V0 = 25.0
    bc = f"anode_bc {anode}\nVappl {V0}\nradius {TIP['radius']}\n"

    def run(tol_line):
        conf = tmp_path / f"{anode}_{abs(hash(tol_line))}.conf"
        write_conf(conf, bc + tol_line)
        fem = fg.Femocs(str(conf))
        return fem, fem.run()

    fem, rv = run("field_tolerance 1e-6 1e6")
    assert rv == 0
    beta = fem.enhancement()
    # the same ratio from the nodal field this run recovered
    f = fem.field(m.sizes())
    e_max = np.linalg.norm(f.nodal()[:, :3], axis=1).max()
    e0 = V0 / box_h if anode == "dirichlet" else -0.1
    expect = abs(e_max / e0) / analytic_enhancement(TIP["radius"], zs.max() - zs.min())
    assert beta > 0 and abs(beta - expect) <= 1e-12 * expect, (beta, expect)
    # inside the window: success; on either side of it: failure with the reference's message
    assert run(f"field_tolerance {0.99 * beta} {1.01 * beta}")[1] == 0
    for window in (f"{1.01 * beta} {2 * beta}", f"{0.5 * beta} {0.99 * beta}"):
        fem, rv = run("field_tolerance " + window)
        assert rv == 1 and "enhancement" in fg.last_error()
    # one argument t gives the window [1 - t, 1 + t] (src/Config.cpp:285-292)
    t = abs(beta - 1.0)
    assert run(f"field_tolerance {t * 1.01}")[1] == 0
    assert run(f"field_tolerance {t * 0.99}")[1] == 1
