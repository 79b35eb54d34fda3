"""Batched solves of several resident meshes (block-diagonal multigrid PCG, one graph launch
per step) against single-mesh solves and the oracle.

Tolerances: every batched solve stops at the stated relative residual; phi then agrees with
the oracle's converged solution within 2e3 x tol x max|phi| (the same bound as the
single-mesh tests). With the autotuner off the per-mesh reductions make a mesh's result
independent of the other meshes in the launch, so "alone" and "in the mix" agree bit for
bit; with it on, the chosen threads-per-row (and so the FP32 summation order inside the
preconditioner) may differ, and the results agree within the solve tolerance."""
import numpy as np
import pytest

import femocs_gb300 as fg
import oracle as orc
from util import oracle_tables, vacuum_system_inputs

pytestmark = pytest.mark.gpu
SPECS = [
    dict(radius=8.0, height=25.0, box_half=30.0, slab=6.0, top=80.0, h=4.0, growth=1.4, margin=4.0),
    dict(radius=10.0, height=35.0, box_half=40.0, slab=8.0, top=120.0, h=4.0, growth=1.35, margin=5.0),
    dict(radius=6.0, height=30.0, box_half=25.0, slab=5.0, top=70.0, h=3.5, growth=1.45, margin=4.0),
]
FIELDS = [0.1, 0.25, 0.05]


@pytest.fixture(scope="module")
def meshes():
    return [fg.Mesh.synthetic(**s) for s in SPECS]


@pytest.fixture(scope="module")
def oracle_phi(meshes):
    out = []
    for m, E0 in zip(meshes, FIELDS):
        xyz, cells, v2n = vacuum_system_inputs(m)
        s = orc.System(xyz, cells, -E0)  # Neumann value -E0, as PoissonSolver::setup(-E0)
        it, x = s.ssor_cg(1.2, 1e-13 * np.linalg.norm(s.rhs), 50000)
        phi = np.zeros(m.sizes()["n_nodes"])
        phi[v2n] = x
        out.append(phi)
    return out


def batch_of(meshes, **kw):
    b = fg.Batch(**kw)
    slots = [b.add_mesh(m) for m in meshes]
    assert slots == list(range(len(meshes)))
    return b, slots


@pytest.mark.parametrize("use_graph", [True, False])
@pytest.mark.parametrize("tol", [1e-9, 1e-12])
def test_batch_matches_oracle(meshes, oracle_phi, use_graph, tol):
    b, slots = batch_of(meshes, use_graph=use_graph)
    res = b.solve_all(dict(zip(slots, FIELDS)), rel_tol=tol, max_iter=500)
    assert sorted(res) == slots
    for s, m, phi in zip(slots, meshes, oracle_phi):
        r = res[s]
        assert r["status"] == 1 and 0 < r["iterations"] <= 80
        assert b.true_residual(s) <= 2 * tol
        got = b.phi_nodes(s)
        assert np.abs(got - phi).max() <= 2e3 * tol * np.abs(phi).max()


def test_alone_and_in_the_mix_bit_identical(meshes):
    # alone: only mesh 1 admitted
    b, slots = batch_of(meshes, autotune=False)
    r_alone = b.solve_all({1: FIELDS[1]}, rel_tol=1e-10)[1]
    phi_alone = b.phi_nodes(1)
    # in the mix: all three admitted together, mesh 1 from the same (zero) start
    b.reset_solution(1)
    r_mix = b.solve_all(dict(zip(slots, FIELDS)), rel_tol=1e-10)
    assert r_mix[1]["iterations"] == r_alone["iterations"]
    np.testing.assert_array_equal(b.phi_nodes(1), phi_alone)
    # admitted while another mesh is already mid-solve (continuous batching)
    for s in slots:
        b.reset_solution(s)
    b.admit(0, FIELDS[0], 1e-10)
    b.step(3)
    b.admit(1, FIELDS[1], 1e-10)
    b.admit(2, FIELDS[2], 1e-10)
    got = {}
    while True:
        still = b.step(4)
        got.update(b.collect())
        if still == 0:
            break
    assert got[1]["iterations"] == r_alone["iterations"]
    np.testing.assert_array_equal(b.phi_nodes(1), phi_alone)


def test_alone_and_in_the_mix_autotuned(meshes):
    b, slots = batch_of(meshes, autotune=True)
    r_alone = b.solve_all({2: FIELDS[2]}, rel_tol=1e-10)[2]
    phi_alone = b.phi_nodes(2)
    b.reset_solution(2)
    b.solve_all(dict(zip(slots, FIELDS)), rel_tol=1e-10)
    phi_mix = b.phi_nodes(2)
    assert np.abs(phi_mix - phi_alone).max() <= 2e3 * 1e-10 * np.abs(phi_alone).max()
    assert "L1:A" in b.tuning()


def test_graph_and_host_loop_agree(meshes):
    ref = None
    for use_graph in (True, False):
        b, slots = batch_of(meshes, use_graph=use_graph, autotune=False)
        res = b.solve_all(dict(zip(slots, FIELDS)), rel_tol=1e-10)
        phis = [b.phi_nodes(s) for s in slots]
        its = [res[s]["iterations"] for s in slots]
        if ref is None:
            ref = (its, phis)
        else:
            assert its == ref[0]
            for a, c in zip(phis, ref[1]):
                np.testing.assert_array_equal(a, c)
    st = b.stats()
    assert st["total_dofs"] == sum(b.info(s)["n_dofs"] for s in slots)
    assert st["kernels_per_iteration"] > 10


def test_persistent_kernel_and_graph_bit_identical(meshes):
    """One persistent cooperative kernel per step (grid-wide barriers between the phases of
    the iteration) runs the same phase bodies in the same order as the graph-captured
    launches, and every reduction is per 256-row block and per mesh in block order: the same
    iterations and solutions bit for bit, cold and warm-started (threads per row fixed: the
    autotuner's timed choice may differ between two batches). A step capped at 3 iterations
    stops there and the solve then continues to the same result."""
    ref = None
    for persistent in (False, True):
        b, slots = batch_of(meshes, persistent=persistent, autotune=False)
        res = b.solve_all(dict(zip(slots, FIELDS)), rel_tol=1e-10)
        res2 = b.solve_all({s: 1.1 * f for s, f in zip(slots, FIELDS)}, rel_tol=1e-10)
        out = ([res[s]["iterations"] for s in slots], [res2[s]["iterations"] for s in slots],
               [b.phi_nodes(s) for s in slots])
        for s in slots:
            assert res[s]["status"] == 1 and res2[s]["status"] == 1
        if ref is None:
            ref = out
        else:
            assert out[0] == ref[0] and out[1] == ref[1]
            for x, y in zip(out[2], ref[2]):
                np.testing.assert_array_equal(x, y)
    b1, slots = batch_of(meshes, persistent=True, autotune=False)
    it_full = b1.solve_all({slots[0]: FIELDS[0]}, rel_tol=1e-10)[slots[0]]["iterations"]
    b2, slots = batch_of(meshes, persistent=True, autotune=False)
    b2.admit(slots[0], FIELDS[0], rel_tol=1e-10)
    assert b2.step(3) == 1 and b2.stats()["last_iterations"] == 3
    while b2.step(8):
        pass
    fin = b2.collect()
    assert fin[slots[0]]["status"] == 1 and fin[slots[0]]["iterations"] == it_full


def test_warm_start_iteration_cap_and_slot_reuse(meshes, oracle_phi):
    b, slots = batch_of(meshes)
    b.solve_all({0: FIELDS[0]}, rel_tol=1e-11)
    # same field again: the warm start already meets the tolerance
    r = b.solve_all({0: FIELDS[0]}, rel_tol=1e-11)[0]
    assert r["iterations"] == 0 and r["status"] == 1
    # an iteration cap reports failure and leaves the slot usable
    b.reset_solution(1)
    r = b.solve_all({1: FIELDS[1]}, rel_tol=1e-14, max_iter=2)[1]
    assert r["status"] == -1 and r["iterations"] == 2
    # remove a mesh, add another into the freed ranges, solve everything again
    b.remove_mesh(1)
    s3 = b.add_mesh(meshes[1])
    assert s3 == 1
    res = b.solve_all({0: FIELDS[0], 1: FIELDS[1], 2: FIELDS[2]}, rel_tol=1e-11)
    for s in (0, 1, 2):
        assert res[s]["status"] == 1
        phi = oracle_phi[s]
        assert np.abs(b.phi_nodes(s) - phi).max() <= 2e3 * 1e-11 * np.abs(phi).max()


def test_admission_by_free_memory(meshes):
    b = fg.Batch()
    assert b.add_mesh(meshes[0], hbm_reserve=1e15) == -1
    assert b.add_mesh(meshes[0]) == 0


def test_batch_pipeline_cells_and_fields(meshes):
    """Nodal field + interpolation from a batched solve against the single-mesh pipeline:
    identical cells, phi/E within the solve tolerance."""
    m, spec, E0 = meshes[1], SPECS[1], FIELDS[1]
    b, slots = batch_of([m])
    b.solve_all({0: E0}, rel_tol=1e-12)
    b.extract(0, smoothen=True)
    atoms, types = fg.synth_atoms(spec, seed=3)
    pts = np.ascontiguousarray(np.r_[atoms[types == 2], fg.synth_probes(spec, 2000, seed=9)])
    n = len(pts)
    d_pts, d_cells, d_out = fg.DeviceBuffer(24 * n), fg.DeviceBuffer(4 * n), fg.DeviceBuffer(40 * n)
    d_pts.upload(pts)
    b.interpolate_device(0, n, d_pts.ptr, 1, d_cells.ptr, d_out.ptr)
    b.sync(0)
    cells = d_cells.download(np.zeros(n, dtype=np.int32))
    out = d_out.download(np.zeros(5 * n)).reshape(-1, 5)
    f = fg.Field(m)
    f.setup(-E0)
    f.assemble(True, False)
    f.solve(precision=2, rel_tol=1e-12)
    f.extract(smoothen=True)
    cells_f, out_f = f.interpolate(pts, rank=1)
    np.testing.assert_array_equal(cells, cells_f)
    assert np.abs(out[:, 4] - out_f[:, 4]).max() <= 4e3 * 1e-12 * np.abs(out_f[:, 4]).max()
    e = np.linalg.norm(out_f[:, :3], axis=1).max()
    assert np.linalg.norm(out[:, :3] - out_f[:, :3], axis=1).max() <= 4e3 * 1e-12 * e
