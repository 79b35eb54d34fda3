"""PIC-mode solves: particle space charge scattered on the device (rank-3 location, trilinear
or Q2 shape functions at the particle), the matrix reused (assemble(full_run=false), as
ProjectRunaway::make_pic_step), warm-started multigrid solve.

Tolerances: the space-charge rhs against the numpy restatement (oracle/pic_oracle.py) within
1e-13 of its largest entry (FP64 atomics order the particle sums differently); the solve as
the other solver tests (2e3 x tol x max|phi|)."""
import numpy as np
import pytest
import scipy.sparse as sp

import femocs_gb300 as fg
import oracle as orc
from oracle.pic_oracle import space_charge_q1, space_charge_q2
from oracle.q2_oracle import Q2System, gpu_dof_keys
from util import oracle_tables

pytestmark = pytest.mark.gpu
TIP = dict(radius=8.0, height=25.0, box_half=30.0, slab=6.0, top=80.0, h=4.0, growth=1.4, margin=4.0)
SMALL = dict(radius=5.0, height=14.0, box_half=18.0, slab=4.0, top=40.0, h=4.0, growth=1.6, margin=3.0)
E0, CF = 0.1, 2e-3


def located_hexes(m, pts):
    tables = oracle_tables(m, np.zeros((m.sizes()["n_nodes"], 5)))
    cells, _ = orc.locate_interpolate(tables, 3, pts)
    return np.where(cells >= 0, cells, -1)


def rhs_of(f):
    rowptr, col, val, rhs, d2n = f.system()
    return rowptr, col, val, rhs, d2n


def test_space_charge_q1_matches_oracle_and_solves():
    m = fg.Mesh.synthetic(**TIP)
    f = fg.Field(m)
    pts = fg.synth_probes(TIP, 4000, seed=21)
    f.setup(-E0)
    f.assemble(True, False)
    _, _, _, rhs0, d2n = rhs_of(f)
    skipped = f.space_charge(pts, CF)  # located on the device
    f.assemble(False, False)           # PIC step: matrix reused, rhs rebuilt with the charge
    rowptr, col, val, rhs1, _ = rhs_of(f)
    hexes = located_hexes(m, pts)
    assert skipped == int((hexes < 0).sum())
    n2d = np.full(m.sizes()["n_nodes"], -1)
    n2d[d2n] = np.arange(len(d2n))
    ref = space_charge_q1(m.export("hex_coeffs"), m.export("hex_nodes"), n2d, len(d2n), pts, hexes, CF)
    # Dirichlet rows keep only their diagonal after the elimination and take the boundary
    # value, not the charge
    A = sp.csr_matrix((val, col, rowptr), shape=(len(d2n), len(d2n)))
    fixed = np.asarray((A != 0).sum(axis=1)).ravel() == 1
    dif = (rhs1 - rhs0)[~fixed]
    assert np.abs(dif - ref[~fixed]).max() <= 1e-13 * np.abs(ref).max()
    # with the hexes given (the reference keeps particle.cell) the rhs is the same
    f.space_charge(pts, CF, hex_cells=hexes)
    f.assemble(False, False)
    np.testing.assert_allclose(rhs_of(f)[3], rhs1, rtol=0, atol=1e-13 * np.abs(ref).max())
    # warm-started PIC solve against the oracle solve of the same system
    rc, st = f.solve(precision=2, rel_tol=1e-11)
    assert rc > 0 and st["status"] == 1
    so = orc.System(csr=(rowptr, col, val, rhs1))
    it, x = so.ssor_cg(1.2, 1e-13 * np.linalg.norm(rhs1), 50000)
    assert np.abs(f.solution() - x).max() <= 2e3 * 1e-11 * np.abs(x).max()
    # the charge changes the solution; clearing it restores the Laplace solve
    f.clear_space_charge()
    f.assemble(False, False)
    np.testing.assert_array_equal(rhs_of(f)[3], rhs0)


def test_space_charge_q2_matches_oracle():
    m = fg.Mesh.synthetic(**SMALL)
    f = fg.Field(m, order=2)
    pts = fg.synth_probes(SMALL, 1500, seed=5)
    f.setup(-E0)
    f.assemble(True, False)
    _, _, _, rhs0, _ = rhs_of(f)
    f.space_charge(pts, CF)
    f.assemble(False, False)
    _, _, _, rhs1, _ = rhs_of(f)
    hexes = located_hexes(m, pts)
    s = Q2System(m.export("node_xyz"), m.export("hex_nodes"), m.export("vac_cells"), -E0)
    dc, dl = f.q2_dofs()
    g2o = np.array([s.keys[k] for k in gpu_dof_keys(m, dc, dl)])
    vac = m.export("vac_cells")
    cell_of_hex = {int(h): c for c, h in enumerate(vac)}
    ref_o = space_charge_q2(m.export("hex_coeffs"), cell_of_hex, s.cell_dofs, s.n, pts, hexes, CF)
    ref = ref_o[g2o]  # oracle numbering -> GPU DoFs
    free = ~s.fixed[g2o]
    assert np.abs((rhs1 - rhs0)[free] - ref[free]).max() <= 1e-13 * np.abs(ref).max()
    # partition of unity: every particle inside deposits exactly CF over its hex
    assert abs(ref.sum() - CF * int((hexes >= 0).sum())) <= 1e-10 * CF * len(pts)
