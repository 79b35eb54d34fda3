"""Device mesh preparation (tet -> hex split, grouping and interpolation tables built by kernels)
against the reference's golden vectors and the host builder: every table equal bit for bit."""
import hashlib

import numpy as np
import pytest

import femocs_gb300 as fg
from util import golden_cases, load_golden

pytestmark = pytest.mark.gpu

TABLES = ["tet_nodes", "tet_marker", "tet_nbor", "node_xyz", "node_marker", "hex_nodes", "hex_marker", "tet_det",
          "tet_centroid", "hex_coeffs", "nbr_ptr", "nbr_idx", "quad_nodes", "voro_ptr", "voro_idx", "vac_node2vertex",
          "vac_cells", "tet_search", "edgemax", "node_parents", "surf_tris", "surf_tri2tet", "surf_geo", "surf_nbr_ptr",
          "surf_nbr_idx"]
SMALL = dict(radius=5.0, height=14.0, box_half=18.0, slab=4.0, top=40.0, h=4.0, growth=1.6, margin=3.0)


def bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


def assert_same_tables(mh, md):
    assert mh.sizes() == md.sizes()
    for n in TABLES:
        a, b = mh.export(n), md.export(n)
        assert a.dtype == b.dtype and np.array_equal(bits(a), bits(b)), n


@pytest.mark.parametrize("case", golden_cases())
def test_device_split_matches_reference_golden(case):
    g = load_golden(case)
    md = fg.Mesh.synthetic(device=True, **g["spec_kw"])
    s = md.sizes()
    assert [s["n_tetnodes"], s["n_tets"], s["n_nodes"], s["n_hexs"]] == g["sizes"].tolist()
    for name in ("tet_nodes", "tet_nbor", "tet_marker", "hex_nodes", "hex_marker", "node_marker", "node_xyz"):
        assert hashlib.sha256(np.ascontiguousarray(md.export(name)).tobytes()).hexdigest() == str(g["sha_" + name]), name
    assert md.export("edgemax")[0] == g["edgemax"][0]
    assert md.prep_timing()["kernel_ms"] > 0
    assert_same_tables(fg.Mesh.synthetic(**g["spec_kw"]), md)


@pytest.mark.parametrize("cfg", [SMALL, fg.CONFIG1], ids=["small", "config1"])
def test_device_tables_equal_host(cfg):
    assert_same_tables(fg.Mesh.synthetic(**cfg), fg.Mesh.synthetic(device=True, **cfg))


def test_device_prep_of_renumbered_mesh():
    """The same geometry with vertices, tets and the vertex order inside each tet shuffled:
    other edge and face orders, other hex orientations, same agreement."""
    m = fg.Mesh.synthetic(**SMALL)
    s = m.sizes()
    xyz = m.export("node_xyz").reshape(-1, 3)[: s["n_tetnodes"]]
    tets = m.export("tet_nodes").reshape(-1, 4)
    mk = m.export("tet_marker")
    rng = np.random.default_rng(11)
    pn = rng.permutation(len(xyz))
    inv = np.empty_like(pn)
    inv[pn] = np.arange(len(pn))
    pt = rng.permutation(len(tets))
    t2 = inv[tets[pt]]
    t2 = np.take_along_axis(t2, np.argsort(rng.random(t2.shape), axis=1), axis=1)
    args = (xyz[pn], t2.astype(np.int32), mk[pt])
    assert_same_tables(fg.Mesh.from_arrays(*args), fg.Mesh.from_arrays(*args, device=True))


def test_device_prep_single_tet_and_invalid_meshes():
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1], [-1, -1, -1]], dtype=float)
    one = (xyz[:4], np.array([[0, 1, 2, 3]], dtype=np.int32), np.array([3], dtype=np.int32))
    assert_same_tables(fg.Mesh.from_arrays(*one), fg.Mesh.from_arrays(*one, device=True))
    bad = [
        (xyz[:4], np.array([[0, 1, 2, 2]]), np.array([3])),                                  # degenerate tet
        (xyz, np.array([[0, 1, 2, 3], [0, 1, 2, 4], [0, 1, 2, 5]]), np.array([3, 3, 3])),      # non-manifold face
        (xyz[:4], np.array([[0, 1, 2, 7]]), np.array([3])),                                   # node out of range
    ]
    for a in bad:
        with pytest.raises(RuntimeError):
            fg.Mesh.from_arrays(*a)
        with pytest.raises(RuntimeError):
            fg.Mesh.from_arrays(*a, device=True)


def test_field_on_device_prepared_mesh_solves_the_same():
    phi = []
    for device in (False, True):
        m = fg.Mesh.synthetic(device=device, **SMALL)
        f = fg.Field(m)
        f.setup(-0.1)
        f.assemble(True, False)
        rc, st = f.solve(precision=2, rel_tol=1e-10)
        assert rc > 0
        phi.append(f.phi_nodes())
    assert np.array_equal(bits(phi[0]), bits(phi[1]))
