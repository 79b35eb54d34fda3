"""The reference-facing C ABI (create_femocs / femocs_run / femocs_interpolate_* /
femocs_export_data) end to end on the GPU."""
import numpy as np
import pytest

import femocs_gb300 as fg
import oracle as orc
from util import oracle_tables

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
    conf = tmp_path / "in.conf"
    write_conf(conf)
    fem = fg.Femocs(str(conf))
    atoms, types = fg.synth_atoms(TIP, seed=1)
    assert fem.import_atoms(atoms[:, 0], atoms[:, 1], atoms[:, 2], types) == 0
    assert fem.run() == 0
    st = fem.last_solve()
    assert st["status"] == 1 and st["rel_residual"] <= 1.05e-12
    # interpolation at arbitrary points equals a direct field evaluation of the same mesh
    pts = fg.synth_probes(TIP, 500, seed=2)
    rv, Ex, Ey, Ez, En, flag = fem.interpolate_elfield(pts[:, 0], pts[:, 1], pts[:, 2])
    assert rv == 0
    rv, phi, flag2 = fem.interpolate_phi(pts[:, 0], pts[:, 1], pts[:, 2])
    assert rv == 0 and np.array_equal(flag, flag2)
    m = fg.Mesh.synthetic(**TIP)
    f = fg.Field(m)
    f.setup(0.1)
    f.assemble(True, False)
    f.solve(precision=1, rel_tol=1e-12)
    f.extract(True)
    cells, out = f.interpolate(pts, rank=3)
    np.testing.assert_array_equal(flag, (cells < 0).astype(np.int32))
    np.testing.assert_allclose(np.c_[Ex, Ey, Ez], out[:, :3], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(phi, out[:, 4], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(En, np.linalg.norm(out[:, :3], axis=1), rtol=1e-9, atol=1e-12)
    # export by atom id: surface atoms only, others stay zero (overwrite mode, capital label)
    rv, e = fem.export_data(len(types), "Elfield")
    assert rv == 0
    e = e.reshape(-1, 3)
    surf = types == 2
    # (a surface atom whose fallback cell is a bulk tet gets the empty value 0, as in the reference)
    assert np.all(e[~surf] == 0) and np.mean(np.linalg.norm(e[surf], axis=1) > 0) > 0.5
    sc, so = f.interpolate(atoms[surf], rank=3)
    np.testing.assert_allclose(e[surf], so[:, :3], rtol=1e-9, atol=1e-12)
    # append mode with the exact label adds to the caller's data
    rv, pot = fem.export_data(len(types), "potential")
    assert rv == 0
    np.testing.assert_allclose(pot[surf], so[:, 4], rtol=1e-9, atol=1e-12)


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
