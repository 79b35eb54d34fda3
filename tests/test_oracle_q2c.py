"""The C Q2 assembler of the oracle (oracle/q2_oracle.c, used for the benchmark-size CPU
reference) against the numpy Q2 restatement (oracle/q2_oracle.py): same DoF numbering, the
same matrix and rhs within 1e-12 relative, both anode modes, independent of the thread count."""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle as orc
from oracle import mesh_prep, workload
from oracle.q2_oracle import Q2System

TIP = dict(radius=6.0, height=18.0, box_half=18.0, slab=4.0, top=40.0, h=4.0, growth=1.5, margin=3.0)


@pytest.fixture(scope="module")
def mesh():
    return mesh_prep.OracleMesh(*workload.tet_mesh(TIP))


@pytest.mark.parametrize("anode", [False, True])
def test_q2_c_equals_numpy(mesh, anode):
    xyz = mesh.export("node_xyz").reshape(-1, 3)
    hexes = mesh.export("hex_nodes").reshape(-1, 8)
    vc = mesh.export("vac_cells")
    ref = Q2System(xyz, hexes, vc, 0.1, anode, 2.5)
    got = orc.Q2CSystem(xyz, hexes[vc], 0.1, anode, 2.5, n_threads=3)
    np.testing.assert_array_equal(got.cell_dofs, ref.cell_dofs)
    assert got.n == ref.n
    A = sp.csr_matrix((got.val, got.col, got.rowptr), shape=(got.n, got.n))
    R = ref.A.tocsr()
    R.eliminate_zeros()
    B = A.copy()
    B.eliminate_zeros()
    assert abs(B - R).max() <= 1e-12 * abs(R).max()
    np.testing.assert_allclose(got.rhs, ref.rhs, rtol=0, atol=1e-12 * np.abs(ref.rhs).max())
    np.testing.assert_array_equal(got.constrained.astype(bool), ref.fixed)
    # vertex DoFs carry the mesh node they sit on
    for (node,), d in ((k, v) for k, v in ref.keys.items() if isinstance(k, tuple) and len(k) == 1):
        assert got.dof_node[d] == node


def test_q2_c_does_not_depend_on_threads(mesh):
    xyz = mesh.export("node_xyz").reshape(-1, 3)
    cells = mesh.export("hex_nodes").reshape(-1, 8)[mesh.export("vac_cells")]
    a = orc.Q2CSystem(xyz, cells, 0.1, n_threads=1)
    b = orc.Q2CSystem(xyz, cells, 0.1, n_threads=4)
    for x, y in ((a.rowptr, b.rowptr), (a.col, b.col)):
        np.testing.assert_array_equal(x, y)
    assert np.array_equal(a.val.view(np.int64), b.val.view(np.int64))
    assert np.array_equal(a.rhs.view(np.int64), b.rhs.view(np.int64))
