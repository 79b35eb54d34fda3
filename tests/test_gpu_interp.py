"""CUDA location / interpolation / nodal-field kernels against the reference's golden vectors
(bit-exact cells and values) and against the oracle on larger random point sets."""
import hashlib

import numpy as np
import pytest

import femocs_gb300 as fg
import oracle as orc
from util import bits_equal, golden_cases, load_golden, oracle_tables

pytestmark = pytest.mark.gpu
CASES = golden_cases()


@pytest.fixture(scope="module", params=CASES)
def case(request):
    g = load_golden(request.param)
    m = fg.Mesh.synthetic(**g["spec_kw"])
    f = fg.Field(m)
    return g, m, f


@pytest.mark.parametrize("rank", [1, 2, 3])
def test_gpu_locate_interpolate_matches_reference_bit_exact(case, rank):
    g, m, f = case
    f.set_nodal(orc.test_solution(m.export("node_xyz")))
    cells, out, st = f.interpolate(g["pts"], rank=rank, stats=True)
    np.testing.assert_array_equal(cells, g[f"cells_r{rank}"])
    assert bits_equal(out, g[f"interp_r{rank}"])
    # the golden points exercise every branch of the reference's chained search
    assert st["fallback"] > 0 and st["dependent"] > 0


def test_gpu_nodal_field_matches_reference(case):
    g, m, f = case
    f.set_phi_nodes(orc.test_solution(m.export("node_xyz"))[:, 4])
    f.extract(smoothen=False)
    E = np.ascontiguousarray(f.nodal()[:, :3]).reshape(-1)
    assert hashlib.sha256(E.tobytes()).hexdigest() == str(g["e_raw_sha"])
    f.extract(smoothen=True)
    Es = f.nodal()[:, :3][g["e_nodes"]]
    # the smoothing weights use exp(); CUDA's and the host libm's may differ in the last bit
    np.testing.assert_allclose(Es, g["e_smooth"], rtol=1e-13, atol=1e-15 * float(g["e_smooth_absmax"][0]))


@pytest.mark.parametrize("rank", [1, 3])
def test_gpu_random_points_match_oracle(case, rank):
    g, m, f = case
    spec = g["spec_kw"]
    rng = np.random.default_rng(42)
    b, top, slab = spec["box_half"], spec["top"], spec["slab"]
    n = 6000
    pts = np.c_[rng.uniform(-1.1 * b, 1.1 * b, n), rng.uniform(-1.1 * b, 1.1 * b, n), rng.uniform(-slab - 3, top + 3, n)]
    # add a sorted sweep (long runs of neighbouring points, like atoms)
    sweep = np.c_[np.linspace(-b, b, 2000), np.zeros(2000), np.full(2000, 0.3 * spec["height"])]
    pts = np.r_[pts, sweep]
    sol = orc.test_solution(m.export("node_xyz"))
    f.set_nodal(sol)
    cells, out = f.interpolate(pts, rank=rank)
    rc, ro = orc.locate_interpolate(oracle_tables(m, sol), rank, pts)
    np.testing.assert_array_equal(cells, rc)
    assert bits_equal(out, ro)


def test_gpu_bulk_only_chain(case):
    # points inside the metal: no searchable tet contains them, the result of each depends on
    # the previous one (long dependent runs)
    g, m, f = case
    atoms, types = fg.synth_atoms(g["spec_kw"], seed=9)
    pts = atoms[types == 1][:3000]
    sol = orc.test_solution(m.export("node_xyz"))
    f.set_nodal(sol)
    cells, out, st = f.interpolate(pts, rank=1, stats=True)
    rc, ro = orc.locate_interpolate(oracle_tables(m, sol), 1, pts)
    np.testing.assert_array_equal(cells, rc)
    assert bits_equal(out, ro)


def test_empty_and_single_point(case):
    g, m, f = case
    f.set_nodal(orc.test_solution(m.export("node_xyz")))
    c, o = f.interpolate(np.zeros((0, 3)), rank=3)
    assert len(c) == 0 and len(o) == 0
    c1, o1 = f.interpolate(g["pts"][:1], rank=3)
    assert c1[0] == g["cells_r3"][0] and bits_equal(o1, g["interp_r3"][:1])
