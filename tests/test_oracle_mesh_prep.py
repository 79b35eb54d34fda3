"""The oracle's numpy tet -> hex split and interpolator tables (oracle/mesh_prep.py) against
the product's host builder, table by table and bit for bit, on meshes built by the oracle's
own workload generator (the golden tests pin the product's split to the reference's)."""
import numpy as np
import pytest

import femocs_gb300 as fg
from oracle import mesh_prep, workload
from util import load_golden

SMALL = dict(radius=6.0, height=24.0, box_half=24.0, slab=6.0, top=60.0, h=3.0, growth=1.5, margin=4.0)
TABLES = ["node_xyz", "node_marker", "hex_nodes", "hex_marker", "tet_nbor", "tet_search", "hex_coeffs", "quad_nodes",
          "vac_node2vertex", "vac_cells", "voro_ptr", "voro_idx", "edgemax"]


@pytest.mark.parametrize("spec", [SMALL, fg.CONFIG1], ids=["small", "config1"])
def test_oracle_mesh_tables_equal_product(spec):
    om = mesh_prep.OracleMesh(*workload.tet_mesh(spec))
    m = fg.Mesh.synthetic(**spec)
    s = m.sizes()
    for k, v in om.sizes().items():
        assert s[k] == v, k
    for name in TABLES:
        a = np.ascontiguousarray(om.export(name))
        b = np.ascontiguousarray(m.export(name))
        assert a.shape == b.shape, name
        if a.dtype.kind == "f":
            assert np.array_equal(a.view(np.int64), b.view(np.int64)), name
        else:
            np.testing.assert_array_equal(a, b, err_msg=name)


def test_oracle_split_of_golden_mesh_equals_product():
    g = load_golden("tip_b")
    xyz, tets, marker = workload.tet_mesh(g["spec_kw"])
    om = mesh_prep.OracleMesh(xyz, tets, marker)
    m = fg.Mesh.synthetic(**g["spec_kw"])
    np.testing.assert_array_equal(om.export("hex_nodes"), m.export("hex_nodes"))
