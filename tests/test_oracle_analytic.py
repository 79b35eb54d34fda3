"""The oracle's restatement of the reference FEM solve (Q1 assembly, boundary marking, Neumann
top, Dirichlet elimination, SSOR-CG, nodal field) against the reference's own analytic answer
for a hemisphere on a plane (FieldReader::get_analyt_potential / get_analyt_field,
src/SolutionReader.cpp:501-524), on the boundary-fitted meshes of tests/analytic.py at two
refinements: the potential at the vacuum nodes with 1.2 R < r < 4 R converges at rate >= 1.6,
the recovered field (before smoothing) at the tet vertices with 1.5 R < r < 4 R (beyond the
first radial layer of the coarsest mesh) at rate >= 0.8. This pins the oracle's FEM path,
which the GPU solves are compared with, to a result the reference itself defines."""
import numpy as np

from analytic import analytic_field, analytic_phi, hemisphere_mesh
from oracle import mesh_prep, pipeline

R, BOX, E0 = 10.0, 200.0, -0.1


def errors(n):
    om = mesh_prep.OracleMesh(*hemisphere_mesh(n, R, BOX))
    sol, info = pipeline.reference_solution(om, -E0, rel_tol=1e-11, smoothen=False)
    X = om.export("node_xyz").reshape(-1, 3)
    r = np.linalg.norm(X, axis=1)
    sel = (om.export("vac_node2vertex") >= 0) & (r > 1.2 * R) & (r < 4 * R)
    tv = (om.export("vac_node2vertex") >= 0) & (r > 1.5 * R) & (r < 4 * R) & (om.export("node_marker") == 1)
    e_phi = np.abs(sol[sel, 4] - analytic_phi(X[sel], E0, R)).max()
    e_E = np.linalg.norm(sol[tv, :3] - analytic_field(X[tv], E0, R), axis=1).max()
    return e_phi, e_E


def test_oracle_fem_converges_to_reference_formula():
    (p4, e4), (p8, e8) = errors(4), errors(8)
    assert np.log2(p4 / p8) >= 1.6, (p4, p8)
    assert np.log2(e4 / e8) >= 0.8, (e4, e8)
