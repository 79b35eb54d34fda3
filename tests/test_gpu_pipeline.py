"""End-to-end parity of the field path: GPU (assemble, mixed-precision solve, nodal field,
smoothing, location, interpolation) against the oracle (SSOR-CG, nodal field, smoothing,
the reference's sequential location), on synthetic nanotips with their surface atoms and
random vacuum probes. Cells must match bit-exactly; phi and E agree within the solver
tolerance."""
import numpy as np
import pytest

import femocs_gb300 as fg
import oracle as orc
from util import oracle_tables, vacuum_system_inputs

pytestmark = pytest.mark.gpu
TIP = dict(radius=10.0, height=35.0, box_half=40.0, slab=8.0, top=120.0, h=4.0, growth=1.35, margin=5.0)


@pytest.fixture(scope="module")
def setup():
    m = fg.Mesh.synthetic(**TIP)
    f = fg.Field(m)
    atoms, types = fg.synth_atoms(TIP, seed=12345)
    pts = np.r_[atoms[types == 2], fg.synth_probes(TIP, 3000, seed=5)]
    # oracle reference solution
    xyz, cells, v2n = vacuum_system_inputs(m)
    s = orc.System(xyz, cells, 0.1)
    it, x = s.ssor_cg(1.2, 1e-13 * np.linalg.norm(s.rhs), 50000)
    assert it > 0
    n = m.sizes()
    phi = np.zeros(n["n_nodes"])
    phi[v2n] = x
    n2v = m.export("vac_node2vertex")
    E = orc.nodal_field(m.export("node_xyz"), m.export("hex_nodes"), m.export("hex_marker"),
                        (n2v >= 0).astype(np.int8), phi)
    E = orc.smooth_field(n["n_tetnodes"], m.export("node_xyz"), m.export("voro_ptr"), m.export("voro_idx"),
                         -1.0 / m.export("edgemax")[0], E)
    sol = np.zeros((n["n_nodes"], 5))
    sol[:, :3] = E.reshape(-1, 3)
    sol[:, 4] = phi
    return m, f, pts, sol


@pytest.mark.parametrize("rank", [1, 2, 3])
@pytest.mark.parametrize("precision,tol", [(2, 1e-9), (2, 1e-12), (1, 1e-9), (1, 1e-12), (0, 1e-12)])
def test_pipeline_parity(setup, rank, precision, tol):
    m, f, pts, sol = setup
    f.setup(0.1)
    f.assemble(True, False)
    rc, st = f.solve(precision=precision, rel_tol=tol)
    # the mixed solver stops on the FP64 true residual; plain CG, like deal.II's SolverCG,
    # stops on its recursive residual, which drifts slightly from the true one at 1e-12
    assert rc > 0 and st["rel_residual"] <= tol * (1.05 if precision == 1 else 2.0)
    f.extract(smoothen=True)
    cells, out = f.interpolate(pts, rank=rank)
    rc_, ro = orc.locate_interpolate(oracle_tables(m, sol), rank, pts)
    np.testing.assert_array_equal(cells, rc_)
    phi_scale = np.abs(sol[:, 4]).max()
    e_scale = np.linalg.norm(sol[:, :3], axis=1).max()
    dphi = np.abs(out[:, 4] - ro[:, 4]).max()
    dE = np.linalg.norm(out[:, :3] - ro[:, :3], axis=1).max()
    assert dphi <= 2e3 * tol * phi_scale, dphi
    assert dE <= 2e4 * tol * e_scale, dE
