"""Q2 (27-node hexahedra) assembly and solves on the device against the independent numpy
restatement (oracle/q2_oracle.py) and the C oracle's SSOR-CG on that system.

Tolerances: matrix and rhs within 1e-12 relative (FP64 summation order differs); solutions
within 2e3 x tol x max|phi| of the oracle's converged solution at relative residual tol; the
flat-surface known answer (phi = E z is in the Q2 space) to 1e-8."""
import numpy as np
import pytest
import scipy.sparse as sp

import femocs_gb300 as fg
import oracle as orc
from oracle.q2_oracle import Q2System, gpu_dof_keys

pytestmark = pytest.mark.gpu
SMALL = dict(radius=5.0, height=14.0, box_half=18.0, slab=4.0, top=40.0, h=4.0, growth=1.6, margin=3.0)
FLAT = dict(radius=0.0, height=0.0, box_half=20.0, slab=4.0, top=40.0, h=6.0, growth=1.4, margin=0.0)
E0 = 0.1


@pytest.fixture(scope="module")
def q2():
    m = fg.Mesh.synthetic(**SMALL)
    f = fg.Field(m, order=2)
    dc, dl = f.q2_dofs()
    keys = gpu_dof_keys(m, dc, dl)
    return m, f, keys


_cache = {}


def oracle_system(m, anode=False, v0=0.0):
    key = (id(m), anode, v0)
    if key not in _cache:
        _cache[key] = Q2System(m.export("node_xyz"), m.export("hex_nodes"), m.export("vac_cells"), -E0, anode, v0)
    return _cache[key]


def gpu_to_oracle(keys, s):
    return np.array([s.keys[k] for k in keys])


def test_q2_structure_sizes(q2):
    m, f, keys = q2
    s = oracle_system(m)
    assert f.n_dofs == s.n and f.nnz == s.nnz_pattern
    assert len(set(keys)) == f.n_dofs
    assert m.q2_sizes()["n_dofs"] == f.n_dofs


@pytest.mark.parametrize("anode", [False, True])
def test_q2_system_matches_oracle(q2, anode):
    m, f, keys = q2
    f.setup(-E0, 2.0)
    f.assemble(True, anode)
    rowptr, col, val, rhs, d2n = f.system()
    s = oracle_system(m, anode, 2.0)
    g2o = gpu_to_oracle(keys, s)
    A = sp.csr_matrix((val, col, rowptr), shape=(f.n_dofs, f.n_dofs)).tocoo()
    P = sp.csr_matrix((A.data, (g2o[A.row], g2o[A.col])), shape=A.shape)
    R = s.A.tocsr()
    assert abs(P - R).max() <= 1e-12 * abs(R).max()
    b = np.zeros(f.n_dofs)
    b[g2o] = rhs
    np.testing.assert_allclose(b, s.rhs, rtol=0, atol=1e-12 * np.abs(s.rhs).max())
    # vertex DoFs sit on the mesh nodes
    node_of_vertex = {d: n for d, n in enumerate(d2n) if n >= 0}
    for d, n in list(node_of_vertex.items())[:200]:
        assert keys[d] == (n,)


@pytest.mark.parametrize("precision", [0, 1, 2, 3])
def test_q2_solve_matches_oracle(q2, precision):
    m, f, keys = q2
    tol = 1e-10
    f.setup(-E0)
    f.assemble(True, False)
    rc, st = f.solve(precision=precision, rel_tol=tol, max_iter=50000)
    assert rc > 0 and st["status"] == 1
    assert st["rel_residual"] <= tol * (1.05 if precision in (1, 3) else 2.0)
    if precision == 3:
        assert st["outer"] >= 2  # FP64 refinements around the FP32 multigrid CG
    s = oracle_system(m)
    R = s.A.tocsr()
    so = orc.System(csr=(R.indptr.astype(np.int64), R.indices.astype(np.int32), R.data, s.rhs))
    it, x = so.ssor_cg(1.2, 1e-13 * np.linalg.norm(s.rhs), 100000)
    assert it > 0
    g2o = gpu_to_oracle(keys, s)
    rowptr, col, val, rhs, d2n = f.system()
    phi_dof = np.zeros(f.n_dofs)
    phi_nodes = f.phi_nodes()
    vert = d2n >= 0
    phi_dof[vert] = phi_nodes[d2n[vert]]
    assert np.abs(phi_dof[vert] - x[g2o[vert]]).max() <= 2e3 * tol * np.abs(x).max()
    if precision == 2:
        assert st["iterations"] <= 80 and st["levels"] >= 3


def test_q2_flat_known_answer():
    m = fg.Mesh.synthetic(**FLAT)
    f = fg.Field(m, order=2)
    f.setup(0.1)
    f.assemble(True, False)
    rc, st = f.solve(precision=2, rel_tol=1e-12)
    assert rc > 0
    xyz = m.export("node_xyz").reshape(-1, 3)
    n2v = m.export("vac_node2vertex")
    phi = f.phi_nodes()
    vac = n2v >= 0
    assert np.abs(phi[vac] - 0.1 * xyz[vac, 2]).max() < 1e-8
    f.extract(smoothen=True)
    E = f.nodal()[vac, :3]
    assert np.abs(E[:, 2] + 0.1).max() < 1e-7 and np.abs(E[:, :2]).max() < 1e-7


def test_q2_pipeline_against_q1(q2):
    """Location does not depend on the element; phi at the vertices differs from the Q1
    solution only by the discretisation error."""
    m, f2, _ = q2
    f1 = fg.Field(m, order=1)
    for f in (f1, f2):
        f.setup(-E0)
        f.assemble(True, False)
        rc, st = f.solve(precision=2, rel_tol=1e-10)
        assert rc > 0
        f.extract(smoothen=True)
    atoms, types = fg.synth_atoms(SMALL, seed=4)
    pts = np.ascontiguousarray(np.r_[atoms[types == 2], fg.synth_probes(SMALL, 1000, seed=2)])
    c1, o1 = f1.interpolate(pts, rank=1)
    c2, o2 = f2.interpolate(pts, rank=1)
    np.testing.assert_array_equal(c1, c2)
    scale = np.abs(o1[:, 4]).max()
    d = np.abs(o2[:, 4] - o1[:, 4]).max()
    assert 0 < d < 0.05 * scale


def test_q2_level0_element_by_element_matches_sell(q2):
    """The finest multigrid level applied element by element (cell blocks, the default) is the
    same operator as the assembled SELL matrix (FP32 rounding aside): same convergence, same
    solution."""
    m, f, keys = q2
    out = {}
    for ebe in (True, False):
        f.set_level0_ebe(ebe)
        f.setup(-E0)
        f.assemble(True, False)
        rc, st = f.solve(precision=2, rel_tol=1e-10)
        assert rc > 0 and st["status"] == 1
        out[ebe] = (st["iterations"], f.solution())
    f.set_level0_ebe(True)
    assert abs(out[True][0] - out[False][0]) <= 2
    x = out[False][1]
    assert np.abs(out[True][1] - x).max() <= 2e3 * 1e-10 * np.abs(x).max()


@pytest.mark.parametrize("anode", [False, True])
def test_q2_cell_block_limits_give_the_same_solve(anode):
    """The cell-block level 0 and outer SpMV equal the assembled SELL operators for any block
    limits: single-hex blocks (every DoF but the interior ones split over blocks, all partial
    sums through the slots), small blocks halved for their DoF limit, the default blocks —
    same PCG iterations (within 2), same solution within the tolerance; with the anode as a
    Dirichlet boundary too."""
    m = fg.Mesh.synthetic(**SMALL)
    f = fg.Field(m, order=2)
    f.set_level0_ebe(False)
    f.set_outer_spmv(0)
    f.setup(-E0, 3.0)
    f.assemble(True, anode)
    rc, st = f.solve(precision=2, rel_tol=1e-10)
    assert rc > 0 and st["status"] == 1
    it_ref, x_ref = st["iterations"], f.solution()
    f.set_level0_ebe(True)
    f.set_outer_spmv(2)
    for cells, max_dofs in ((1, 27), (16, 300), (256, 4096)):
        f.set_cell_blocks(cells, max_dofs)
        f.setup(-E0, 3.0)
        f.assemble(True, anode)
        rc, st = f.solve(precision=2, rel_tol=1e-10)
        assert rc > 0 and st["status"] == 1 and st["rel_residual"] <= 1e-10, (cells, st)
        assert abs(st["iterations"] - it_ref) <= 2, (cells, st["iterations"], it_ref)
        assert np.abs(f.solution() - x_ref).max() <= 2e3 * 1e-10 * np.abs(x_ref).max(), cells


@pytest.mark.parametrize("cells,max_dofs", [(1, 27), (5, 150), (256, 4096)])
def test_q2_streamed_element_matrices_are_bit_identical(cells, max_dofs):
    """The level-0 element matrices streamed through the bulk-copy ring and loaded by the
    applying warps give bit-identical solves: the same products in the same order. Block
    limits cover one-cell blocks (every chunk partial, copies starting 8 bytes past a
    16-byte boundary for odd cells, the array's last bytes loaded plainly), blocks of five
    cells (odd chunk sizes) and the default blocks (full chunks, rings reused)."""
    m = fg.Mesh.synthetic(**SMALL)
    f = fg.Field(m, order=2)
    f.set_cell_blocks(cells, max_dofs)
    assert f.set_level0_operator(0) == 0
    out = {}
    for stream in (False, True):
        f.set_level0_stream(stream)
        f.setup(-E0)
        f.assemble(True, False)
        rc, st = f.solve(precision=2, rel_tol=1e-10)
        assert rc > 0 and st["status"] == 1, st
        out[stream] = (st["iterations"], f.solution())
    assert out[True][0] == out[False][0]
    assert np.array_equal(out[True][1].view(np.int64), out[False][1].view(np.int64))


@pytest.mark.gpu
@pytest.mark.parametrize("cells,max_dofs", [(1, 27), (5, 150), (256, 4096)])
def test_q2_matrix_free_level0_matches_element_matrices(cells, max_dofs):
    """The level-0 smoother applied matrix-free from the geometric factors (sum factorisation
    over the hexes' pencils, three hexes per warp; FP32 and FP16 factors, with and without L2
    prefetch) preconditions as well as the element matrices: the same iteration count within
    one, the same true residual bound, and the same solution within the solve tolerance.
    Block limits cover one-hex blocks (every three-hex group partial), five-hex blocks (a
    partial last group) and the default blocks."""
    m = fg.Mesh.synthetic(**SMALL)
    f = fg.Field(m, order=2)
    f.set_cell_blocks(cells, max_dofs)
    res = {}
    for kind, pf in ((0, 0), (1, 0), (2, 0), (2, 2)):
        assert f.set_level0_operator(kind) == kind
        f.set_level0_prefetch(pf)
        f.setup(-E0)
        f.assemble(True, False)
        rc, st = f.solve(precision=2, rel_tol=1e-10)
        assert rc > 0 and st["status"] == 1 and st["rel_residual"] <= 1e-10, (kind, st)
        res[(kind, pf)] = (st["iterations"], f.solution())
    it0, x0 = res[(0, 0)]
    for key, (it, x) in res.items():
        assert abs(it - it0) <= 1, (key, it, it0)
        assert np.abs(x - x0).max() <= 2e3 * 1e-10 * np.abs(x0).max(), key


@pytest.mark.gpu
def test_q2_fp16_factors_fall_back_to_fp32_beyond_range():
    """Geometric factors scale with the element size (w |det J| |J^-1|^2 ~ h / 3): on the small
    tip scaled by 1e5 they exceed the FP16 range, so asking for FP16 factors gives the FP32
    ones (the kind returned), and the solve matches the element-matrix smoother's."""
    big = {k: (v if k == "growth" else v * 1e5) for k, v in SMALL.items()}
    m = fg.Mesh.synthetic(**big)
    f = fg.Field(m, order=2)
    assert f.set_level0_operator(2) == 1
    res = {}
    for kind in (2, 0):
        f.set_level0_operator(kind)
        f.setup(-E0 * 1e-5)
        f.assemble(True, False)
        rc, st = f.solve(precision=2, rel_tol=1e-10)
        assert rc > 0 and st["status"] == 1, (kind, st)
        res[kind] = (st["iterations"], f.solution())
    assert abs(res[2][0] - res[0][0]) <= 1, res
    assert np.abs(res[2][1] - res[0][1]).max() <= 2e3 * 1e-10 * np.abs(res[0][1]).max()


@pytest.mark.gpu
def test_q2_level_smoothing_override_and_restore():
    """Per-level Chebyshev settings change only the polynomial: the Q1 level and the
    aggregation levels at other degrees still converge to the same solution, and restoring
    the defaults gives the default solve bit for bit (no rebuild in between)."""
    m = fg.Mesh.synthetic(**SMALL)
    f = fg.Field(m, order=2)
    tol = 1e-10

    def solve():
        f.setup(-E0)
        f.assemble(True, False)
        rc, st = f.solve(precision=2, rel_tol=tol)
        assert rc > 0 and st["status"] == 1, st
        assert st["rel_residual"] <= 2 * tol
        return st["iterations"], f.solution().copy()

    it0, x0 = solve()
    f.set_level_smoothing(1, 2, 0.1)
    for lvl in range(2, 6):
        f.set_level_smoothing(lvl, 3)
    it1, x1 = solve()
    assert np.abs(x1 - x0).max() <= 2e3 * tol * np.abs(x0).max()
    for lvl in range(1, 6):
        f.set_level_smoothing(lvl)
    it2, x2 = solve()
    assert it2 == it0 and np.array_equal(x2, x0)
    with pytest.raises(RuntimeError):
        f.set_level_smoothing(0, 2)


@pytest.mark.gpu
@pytest.mark.parametrize("anode,v0", [(False, 0.0), (True, 2.5)])
def test_q2_lazy_matrix_matches_eager(anode, v0):
    """The default Q2 assembly forms the assembled matrix only when it is read: the multigrid
    solve takes D^-1 from the element matrices and its true residual over the cell blocks.
    Against the eager assembly: the exported system is bit for bit the same, the solve takes
    the same iterations to the same solution (a nonzero Dirichlet value takes the assembled
    path in both)."""
    m = fg.Mesh.synthetic(**SMALL)
    res = {}
    for lazy in (True, False):
        f = fg.Field(m, order=2)
        f.set_lazy_matrix(lazy)
        f.setup(-E0, v0)
        f.assemble(True, anode)
        rc, st = f.solve(precision=2, rel_tol=1e-10)
        assert rc > 0 and st["status"] == 1, st
        assert st["rel_residual"] <= 2e-10
        x = f.solution().copy()
        _, _, val, rhs, _ = f.system()
        res[lazy] = (st["iterations"], x, val, rhs)
    (it1, x1, val1, b1), (it0, x0, val0, b0) = res[True], res[False]
    assert np.array_equal(val1, val0) and np.array_equal(b1, b0)
    assert it1 == it0
    assert np.abs(x1 - x0).max() <= 1e-12 * np.abs(x0).max()
