"""Current and heat on the bulk hexahedra on the GPU (CurrentHeatSolver verbs) against the
oracle's restatement and known answers. Tolerances: potentials and temperature rises within
1e-8 of the oracle's direct solve (GPU solves to 1e-12 relative residual)."""
import numpy as np
import pytest

import femocs_gb300 as fg
from oracle.heat_oracle import BulkSystem

pytestmark = pytest.mark.gpu
FLAT = dict(radius=0.0, height=0.0, box_half=20.0, slab=8.0, top=40.0, h=4.0, growth=1.4, margin=0.0)
SMALL = dict(radius=5.0, height=14.0, box_half=18.0, slab=4.0, top=40.0, h=4.0, growth=1.6, margin=3.0)
TAB_T = np.array([200.0, 400.0, 800.0, 1600.0])
TAB_RHO = np.array([1.0e-8, 1.7e-8, 3.5e-8, 7.0e-8])


@pytest.fixture(scope="module")
def small():
    m = fg.Mesh.synthetic(**SMALL)
    b = BulkSystem(m.export("node_xyz"), m.export("hex_nodes"), m.export("hex_marker"))
    h = fg.Heat(m)
    h.set_resistivity(TAB_T, TAB_RHO)
    h.setup(300.0, 2.44e-8, 3.4496e-24)
    return m, b, h


def test_surface_faces_match_oracle_order(small):
    m, b, h = small
    c, hf = h.surface_faces()
    assert h.n_faces == len(b.surface) and h.n_dofs == b.n
    np.testing.assert_allclose(c, b.surface_centroids, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(hf[:, 0], b.cells_hex[[cf[0] for cf in b.surface]])


@pytest.mark.parametrize("precision", [0, 2])
def test_current_and_heat_match_oracle(small, precision):
    m, b, h = small
    h.setup(300.0, 2.44e-8, 3.4496e-24)
    c, _ = h.surface_faces()
    j = 2e-3 * (1.0 + c[:, 2] / SMALL["height"])          # stronger emission towards the apex
    q = 1e-9 * (1.0 + 0.5 * c[:, 0] / SMALL["box_half"])
    rc, st = h.solve_current(j, precision=precision, rel_tol=1e-12)
    assert rc > 0 and st["status"] == 1
    T_node, phi_node = h.nodes()
    phi_o = b.current(j)
    v2n = b.vertex2node
    assert np.abs(phi_node[v2n] - phi_o).max() <= 1e-8 * np.abs(phi_o).max()
    dt = 1e-13
    rc, st = h.solve_heat(dt, q, precision=precision, rel_tol=1e-12)
    assert rc > 0 and st["status"] == 1
    T_node, _ = h.nodes()
    T_o = b.heat(np.full(b.n, 300.0), phi_o, dt, q, TAB_T, TAB_RHO, 2.44e-8, 3.4496e-24, 300.0)
    rise = T_o - 300.0
    assert np.abs(rise).max() > 1e-6
    assert np.abs((T_node[v2n] - 300.0) - rise).max() <= 1e-7 * np.abs(rise).max()
    tmin, tmax = h.temperature_range()
    assert tmin == pytest.approx(T_node[v2n].min()) and tmax == pytest.approx(T_node[v2n].max())
    # outside the bulk nothing is exported
    assert np.isnan(T_node[np.setdiff1d(np.arange(len(T_node)), v2n)]).all()


def test_flat_slab_known_answers():
    m = fg.Mesh.synthetic(**FLAT)
    h = fg.Heat(m)
    h.set_resistivity(TAB_T, TAB_RHO)
    h.setup(300.0, 2.44e-8, 3.4496e-24)
    j = 0.01
    rc, _ = h.solve_current(np.full(h.n_faces, j), rel_tol=1e-13)
    assert rc > 0
    T, phi = h.nodes()
    xyz = m.export("node_xyz").reshape(-1, 3)
    bulk = ~np.isnan(phi)
    z = xyz[bulk, 2]
    np.testing.assert_allclose(phi[bulk], j * (z - z.min()), rtol=0, atol=1e-9)
    # no current, no flux: the temperature stays at ambient
    h.setup(300.0, 2.44e-8, 3.4496e-24)
    h.solve_current(np.zeros(h.n_faces))
    rc, _ = h.solve_heat(1e-12, np.zeros(h.n_faces), rel_tol=1e-12)
    T, _ = h.nodes()
    np.testing.assert_allclose(T[bulk], 300.0, rtol=1e-12)


def test_consecutive_heat_steps_match_oracle(small):
    """Two implicit-Euler steps: the second assembles a new matrix (kappa(T) of the first
    step's temperatures) under the kept multigrid hierarchy; both match the oracle's chain."""
    m, b, h = small
    h.setup(300.0, 2.44e-8, 3.4496e-24)
    c, _ = h.surface_faces()
    j = 2e-3 * (1.0 + c[:, 2] / SMALL["height"])
    q = 1e-9 * (1.0 + 0.5 * c[:, 0] / SMALL["box_half"])
    rc, _ = h.solve_current(j, precision=2, rel_tol=1e-12)
    assert rc > 0
    phi_o = b.current(j)
    dt = 1e-13
    T_o = np.full(b.n, 300.0)
    v2n = b.vertex2node
    for step in range(2):
        rc, st = h.solve_heat(dt, q, precision=2, rel_tol=1e-12)
        assert rc > 0 and st["status"] == 1, (step, st)
        T_o = b.heat(T_o, phi_o, dt, q, TAB_T, TAB_RHO, 2.44e-8, 3.4496e-24, 300.0)
        T_node, _ = h.nodes()
        rise = T_o - 300.0
        assert np.abs((T_node[v2n] - 300.0) - rise).max() <= 1e-7 * np.abs(rise).max(), step
