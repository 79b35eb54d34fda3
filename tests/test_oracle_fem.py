"""The oracle's restatement of the reference FEM (deal.II Q1 assembly, boundary conditions,
SSOR-PCG). Parity with the reference's solve is unpinned (deal.II is absent); these known-answer
tests pin the restatement to the mathematics instead."""
import numpy as np

import femocs_gb300 as fg
import oracle as orc
from util import vacuum_system_inputs

FLAT = dict(radius=0.0, height=0.0, box_half=30.0, slab=6.0, top=60.0, h=6.0, growth=1.3, margin=0.0)
TIP = dict(radius=8.0, height=25.0, box_half=30.0, slab=6.0, top=80.0, h=4.0, growth=1.4, margin=4.0)


def test_flat_surface_linear_potential_is_exact():
    # phi = 0 on the metal (z=0), d(phi)/dz = bc on the top: the exact solution bc*z is
    # linear, so Q1 reproduces it to solver precision (applied field 0.1 V/A)
    m = fg.Mesh.synthetic(**FLAT)
    xyz, cells, _ = vacuum_system_inputs(m)
    bc = 0.1
    sysm = orc.System(xyz, cells, bc)
    it, x = sysm.ssor_cg(1.2, 1e-12, 5000)
    assert it > 0
    assert np.abs(x - bc * xyz[:, 2]).max() < 1e-8
    # nodal field recovery of a linear potential is exact: E = -grad(phi) = (0, 0, -bc)
    phi_nodes = np.zeros(m.sizes()["n_nodes"])
    n2v = m.export("vac_node2vertex")
    phi_nodes[n2v >= 0] = x[n2v[n2v >= 0]]
    is_vac = (n2v >= 0).astype(np.int8)
    E = orc.nodal_field(m.export("node_xyz"), m.export("hex_nodes"), m.export("hex_marker"), is_vac, phi_nodes)
    E = E.reshape(-1, 3)[n2v >= 0]
    assert np.abs(E[:, 2] + bc).max() < 1e-7 and np.abs(E[:, :2]).max() < 1e-7


def test_system_symmetric_and_constrained_rows():
    m = fg.Mesh.synthetic(**TIP)
    xyz, cells, _ = vacuum_system_inputs(m)
    s = orc.System(xyz, cells, 0.1)
    import scipy.sparse as sp
    A = sp.csr_matrix((s.val, s.col, s.rowptr), shape=(s.n, s.n))
    assert abs(A - A.T).max() < 1e-12 * abs(A).max()
    c = np.flatnonzero(s.constrained)
    assert len(c) > 0
    # constrained rows and columns keep only their diagonal
    Ac = A[c].tocoo()
    assert np.all((Ac.data == 0) | (c[Ac.row] == Ac.col))
    Act = A[:, c].tocoo()
    assert np.all((Act.data == 0) | (c[Act.col] == Act.row))
    assert np.all(s.rhs[c] == 0) and np.all(s.x0[c] == 0)
    # row sums of the unconstrained stiffness vanish (constant functions are in the kernel)
    free = np.flatnonzero(s.constrained == 0)
    assert np.all(A.diagonal()[free] > 0)


def test_ssor_and_jacobi_cg_agree():
    m = fg.Mesh.synthetic(**TIP)
    xyz, cells, _ = vacuum_system_inputs(m)
    s = orc.System(xyz, cells, 0.1)
    b = np.linalg.norm(s.rhs)
    it1, x1 = s.ssor_cg(1.2, 1e-12 * b, 20000)
    it2, x2 = s.jacobi_cg(1e-12 * b, 200000)
    assert it1 > 0 and it2 > 0 and it1 < it2
    assert np.abs(x1 - x2).max() < 1e-8 * np.abs(x1).max()
    assert np.linalg.norm(s.spmv(x1) - s.rhs) <= 1e-12 * b * 1.0001


def test_field_enhancement_above_flat():
    # the tip enhances the field: max |E| at the apex region exceeds the applied field
    m = fg.Mesh.synthetic(**TIP)
    xyz, cells, v2n = vacuum_system_inputs(m)
    s = orc.System(xyz, cells, 0.1)
    it, x = s.ssor_cg(1.2, 1e-10, 20000)
    phi = np.zeros(m.sizes()["n_nodes"])
    phi[v2n] = x
    n2v = m.export("vac_node2vertex")
    E = orc.nodal_field(m.export("node_xyz"), m.export("hex_nodes"), m.export("hex_marker"),
                        (n2v >= 0).astype(np.int8), phi).reshape(-1, 3)
    assert np.linalg.norm(E, axis=1).max() > 0.2
