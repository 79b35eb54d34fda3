"""Surface (2-D) location and interpolation on the GPU: against the reference's golden vectors
(LinearTriangles / QuadraticTriangles / LinearQuadrangles with TetGen's triangle/tet pairs,
bit-exact cells and values) and against the oracle's restatement on larger point sets."""
import numpy as np
import pytest

import femocs_gb300 as fg
import oracle as orc
from util import bits_equal, load_surface, oracle_tables, surface_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=surface_cases())
def case(request):
    g = load_surface(request.param)
    m = fg.Mesh.synthetic(**g["spec_kw"])
    m.set_surface(g["tri_nodes"], g["tri2tet"])
    f = fg.Field(m)
    f.set_nodal(orc.test_solution(m.export("node_xyz")))
    return g, m, f


@pytest.mark.parametrize("rank", [1, 2, 3])
def test_gpu_surface_interpolation_matches_reference_bit_exact(case, rank):
    g, m, f = case
    cells, out = f.interpolate_surface(g["pts"], rank=rank)
    np.testing.assert_array_equal(cells, g[f"cells_s{rank}"])
    assert bits_equal(out, g[f"interp_s{rank}"])
    # the fixture reaches the nearest-centroid fallback and points held by several triangles
    assert (cells < 0).any() and (cells > 0).any()


@pytest.mark.parametrize("rank", [1, 2, 3])
def test_gpu_surface_large_point_sets_match_oracle(rank):
    m = fg.Mesh.synthetic(**fg.CONFIG1)
    f = fg.Field(m)
    xyz = m.export("node_xyz")
    sol = orc.test_solution(xyz)
    f.set_nodal(sol)
    tris, t2t, geo = m.surface()
    rng = np.random.default_rng(7)
    atoms, types = fg.synth_atoms(fg.CONFIG1, seed=5)
    k = rng.integers(0, len(tris), 4000)
    off = geo[k, 16:19] + geo[k, 12:15] * (rng.uniform(-1.2, 1.2, len(k)) * geo[k, 15])[:, None]
    pts = np.ascontiguousarray(np.r_[atoms[types == 2], off, xyz.reshape(-1, 3)[tris[k[:500], 0]]])
    cells, out = f.interpolate_surface(pts, rank=rank)
    oc, oo = orc.surface_interpolate(oracle_tables(m, sol), tris, t2t, xyz, rank, pts)
    np.testing.assert_array_equal(cells, oc)
    assert bits_equal(out, oo)


def test_surface_elfield_through_the_reference_api(tmp_path):
    """femocs_interpolate_surface_elfield: E at the surface atoms from the rank-1 surface path,
    |E| and the flag (1 = no triangle holds the point) as for the volume call."""
    spec = dict(radius=10.0, height=30.0, box_half=40.0, slab=10.0, top=120.0, h=5.0, growth=1.4, margin=6.0)
    conf = tmp_path / "s.in"
    conf.write_text("mesh_file synthetic\nradius %r\ntip_height %r\ngpu_box_half %r\ngpu_slab %r\ngpu_top %r\n"
                    "gpu_h %r\ngpu_growth %r\ngpu_margin %r\nelfield -0.1\nanode_bc neumann\n"
                    "interpolation_rank 1\nsmoothen_field true\n" % (spec["radius"], spec["height"], spec["box_half"],
                                                                      spec["slab"], spec["top"], spec["h"],
                                                                      spec["growth"], spec["margin"]))
    fem = fg.Femocs(str(conf))
    assert fem.run() == 0
    atoms, types = fg.synth_atoms(spec, seed=9)
    p = atoms[types == 2][:2000]
    rv, Ex, Ey, Ez, En, flag = fem.interpolate_surface_elfield(p[:, 0], p[:, 1], p[:, 2])
    assert rv == 0
    field = fem.field({"n_nodes": 0})
    cells, out = field.interpolate_surface(p, rank=1)
    assert bits_equal(np.c_[Ex, Ey, Ez], out[:, :3])
    np.testing.assert_allclose(En, np.linalg.norm(out[:, :3], axis=1), rtol=1e-15)
    np.testing.assert_array_equal(flag, (cells < 0).astype(np.int32))
    # field enhancement at the apex: E points away from the surface and is stronger than E0
    apex = np.argmax(p[:, 2])
    assert En[apex] > 0.1
