"""The oracle's restatement of the reference FEM solve (Q1 assembly, boundary marking, Neumann
top, Dirichlet elimination, SSOR-CG, nodal field) against the reference's own analytic answer
for a hemisphere on a plane (FieldReader::get_analyt_potential / get_analyt_field,
src/SolutionReader.cpp:501-524), on the boundary-fitted meshes of tests/analytic.py at two
refinements: the potential at the vacuum nodes with 1.2 R < r < 4 R converges at rate >= 1.6
(max norm), the recovered field (before smoothing) with 1.5 R < r < 4 R (beyond the first radial
layer of the coarsest mesh) at rate >= 1.2 at the tet vertices and >= 0.8 over all nodes (RMS). This pins the oracle's FEM path,
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
    band = (om.export("vac_node2vertex") >= 0) & (r > 1.5 * R) & (r < 4 * R)
    tv = band & (om.export("node_marker") == 1)
    e_phi = np.abs(sol[sel, 4] - analytic_phi(X[sel], E0, R)).max()
    rms = lambda m: np.sqrt((np.linalg.norm(sol[m, :3] - analytic_field(X[m], E0, R), axis=1) ** 2).mean())
    return e_phi, rms(tv), rms(band)


def test_oracle_fem_converges_to_reference_formula():
    (p4, t4, a4), (p8, t8, a8) = errors(4), errors(8)
    assert np.log2(p4 / p8) >= 1.6, (p4, p8)
    assert np.log2(t4 / t8) >= 1.2, (t4, t8)
    assert np.log2(a4 / a8) >= 0.8, (a4, a8)
