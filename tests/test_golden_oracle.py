"""The oracle and the host-side mesh preparation against the reference's golden vectors.

Golden vectors come from the reference's own compiled sources (tests/golden/make_golden.py):
tet->hex split, neighbour lists, located cells and interpolated values for ranks 1-3, nodal
field recovery and smoothing."""
import hashlib

import numpy as np
import pytest

import femocs_gb300 as fg
import oracle as orc
from util import bits_equal, golden_cases, load_golden, load_surface, oracle_tables, surface_cases

CASES = golden_cases()


@pytest.fixture(scope="module", params=CASES)
def case(request):
    g = load_golden(request.param)
    m = fg.Mesh.synthetic(**g["spec_kw"])
    return g, m


def test_fixtures_present():
    assert len(CASES) >= 2


def test_host_split_matches_reference(case):
    g, m = case
    s = m.sizes()
    assert [s["n_tetnodes"], s["n_tets"], s["n_nodes"], s["n_hexs"]] == g["sizes"].tolist()
    for name in ("tet_nodes", "tet_nbor", "tet_marker", "hex_nodes", "hex_marker", "node_marker", "node_xyz"):
        assert hashlib.sha256(np.ascontiguousarray(m.export(name)).tobytes()).hexdigest() == str(g["sha_" + name]), name
    assert m.export("edgemax")[0] == g["edgemax"][0]


def test_det_tables_product_equals_oracle(case):
    _, m = case
    s = m.sizes()
    det, ctr = orc.tet_tables(m.export("tet_nodes"), m.export("node_xyz")[: 3 * s["n_tetnodes"]])
    assert bits_equal(det, m.export("tet_det"))
    assert bits_equal(ctr, m.export("tet_centroid"))


@pytest.mark.parametrize("rank", [1, 2, 3])
def test_oracle_locate_interpolate_bit_exact(case, rank):
    g, m = case
    sol = orc.test_solution(m.export("node_xyz"))
    cells, out = orc.locate_interpolate(oracle_tables(m, sol), rank, g["pts"])
    np.testing.assert_array_equal(cells, g[f"cells_r{rank}"])
    assert bits_equal(out, g[f"interp_r{rank}"])


def test_oracle_nodal_field_bit_exact(case):
    g, m = case
    xyz = m.export("node_xyz")
    phi = orc.test_solution(xyz)[:, 4]
    is_vac = (m.export("vac_node2vertex") >= 0).astype(np.int8)
    E = orc.nodal_field(xyz, m.export("hex_nodes"), m.export("hex_marker"), is_vac, phi)
    assert hashlib.sha256(E.tobytes()).hexdigest() == str(g["e_raw_sha"])
    s = m.sizes()
    Es = orc.smooth_field(s["n_tetnodes"], xyz, m.export("voro_ptr"), m.export("voro_idx"), float(g["decay"][0]), E)
    assert bits_equal(Es.reshape(-1, 3)[g["e_nodes"]], g["e_smooth"])


def test_neighbour_lists_cover_reference_lists(case):
    # the product's candidate lists are the reference's (face neighbours first, then
    # vertex-sharing tets) with repeats removed: same first match for every query
    _, m = case
    s = m.sizes()
    rptr, ridx = orc.neighbour_lists(s["n_tetnodes"], m.export("tet_nodes"), m.export("tet_nbor"))
    pptr, pidx = m.export("nbr_ptr"), m.export("nbr_idx")
    for t in range(0, s["n_tets"], max(1, s["n_tets"] // 500)):
        ref = ridx[rptr[t]:rptr[t + 1]]
        seen, dedup = set(), []
        for u in ref:
            if u not in seen:
                seen.add(u)
                dedup.append(u)
        assert list(pidx[pptr[t]:pptr[t + 1]]) == dedup


@pytest.mark.parametrize("name", surface_cases())
def test_surface_fixture_matches_product_surface(name):
    """The reference (with TetGen recomputing the triangle/tet pairs) keeps the product's
    interface triangles, their vertex order and their tet pairs."""
    g = load_surface(name)
    m = fg.Mesh.synthetic(**g["spec_kw"])
    tris, t2t, geo = m.surface()
    np.testing.assert_array_equal(tris, g["tri_nodes"])
    np.testing.assert_array_equal(t2t, g["tri2tet"])
    assert bits_equal(geo[:, 12:15], g["tri_norm"])


@pytest.mark.parametrize("name", surface_cases())
@pytest.mark.parametrize("rank", [1, 2, 3])
def test_oracle_surface_interpolation_bit_exact(name, rank):
    g = load_surface(name)
    m = fg.Mesh.synthetic(**g["spec_kw"])
    xyz = m.export("node_xyz")
    sol = orc.test_solution(xyz)
    cells, out = orc.surface_interpolate(oracle_tables(m, sol), g["tri_nodes"], g["tri2tet"], xyz, rank, g["pts"])
    np.testing.assert_array_equal(cells, g[f"cells_s{rank}"])
    assert bits_equal(out, g[f"interp_s{rank}"])
