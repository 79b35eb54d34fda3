"""The solve against the reference's own analytic answer: a conducting hemisphere on a grounded
plane in a uniform field, FieldReader::get_analyt_potential / get_analyt_field
(src/SolutionReader.cpp:501-524), on boundary-fitted meshes refined three times (tests/analytic.py).

Measured at the mesh nodes with 1.2 R < r < 4 R (away from the hemisphere, where the polyhedral
surface differs from the sphere, and from the box, where the exact solution is not quite the
box's boundary data):

* phi at every vacuum node: the error falls at rate ~2 per halving of h for Q1 and Q2 (Q2 is
  held to second order by the straight-faced approximation of the sphere); required >= 1.6
  between consecutive levels and a finest error below 0.5 % of max |phi| there;
* the recovered nodal E (src/Interpolator.cpp:125-140, before the smoothing step, whose
  weighted neighbourhood average adds an O(h) bias and is checked bit for bit against the
  reference elsewhere) with 1.5 R < r < 4 R (beyond the first radial layer of the coarsest
  mesh), in the RMS norm: at the tet vertices (rate ~2 measured; >= 1.2 required) and over
  every node of the hexahedra (rate ~1, the first order of the reference's three-neighbour
  gradient shortcut, src/InterpolatorCells.cpp:1462-1505, at face and tet-centroid nodes;
  Q2 measured 0.72 on the coarsest step, then 0.96: >= 0.6 on every step and >= 0.85 on the
  finest required). The max norm at single nodes is reported, not asserted: on the
  non-orthogonal corners of the split hexahedra it has a pre-asymptotic plateau;
* the M/A field-enhancement ratio of the reference's check (src/SolutionReader.cpp:526-556)
  with the hemisphere's analytic enhancement 3 approaches 1.
"""
import json
import os

import numpy as np
import pytest

import femocs_gb300 as fg
from analytic import analytic_field, analytic_phi, hemisphere_mesh

pytestmark = pytest.mark.gpu
R, BOX, E0 = 10.0, 200.0, -0.1
LEVELS = (4, 8, 16)


@pytest.fixture(scope="module")
def meshes():
    return {n: fg.Mesh.from_arrays(*hemisphere_mesh(n, R, BOX)) for n in LEVELS}


def node_errors(m, f):
    X = m.export("node_xyz").reshape(-1, 3)
    r = np.linalg.norm(X, axis=1)
    vac = m.export("vac_node2vertex") >= 0
    sel = vac & (r > 1.2 * R) & (r < 4 * R)
    band = vac & (r > 1.5 * R) & (r < 4 * R)
    tv = band & (m.export("node_marker") == 1)
    phi = f.phi_nodes()
    f.extract(smoothen=False)
    E = f.nodal()[:, :3]
    e_phi = np.abs(phi[sel] - analytic_phi(X[sel], E0, R)).max()
    phi_scale = np.abs(analytic_phi(X[sel], E0, R)).max()
    d_tv = np.linalg.norm(E[tv] - analytic_field(X[tv], E0, R), axis=1)
    d_all = np.linalg.norm(E[band] - analytic_field(X[band], E0, R), axis=1)
    e_E = {"rms_tet_vertices": float(np.sqrt((d_tv ** 2).mean())), "rms_all_nodes": float(np.sqrt((d_all ** 2).mean())),
           "max_tet_vertices": float(d_tv.max())}
    # the enhancement check reads the smoothed nodal field, as the reference's does
    f.extract(smoothen=True)
    m_over_a = np.linalg.norm(f.nodal()[vac, :3], axis=1).max() / abs(E0) / 3.0
    return float(e_phi), float(phi_scale), e_E, float(m_over_a)


@pytest.mark.parametrize("order", [1, 2])
def test_hemisphere_converges_to_reference_formula(meshes, order):
    rows = []
    for n in LEVELS:
        m = meshes[n]
        f = fg.Field(m, order=order)
        f.setup(-E0)
        f.assemble(True, False)
        rc, st = f.solve(precision=2, rel_tol=1e-11, max_iter=20000)
        assert rc > 0, st
        e_phi, scale, e_E, ma = node_errors(m, f)
        rows.append({"n": n, "dofs": f.n_dofs, "max_dphi": e_phi, "max_phi": scale, **e_E,
                     "M_over_A": ma, "iterations": st["iterations"]})
    for a, b in zip(rows, rows[1:]):
        b["rate_phi"] = float(np.log2(a["max_dphi"] / b["max_dphi"]))
        b["rate_E_tet_vertices"] = float(np.log2(a["rms_tet_vertices"] / b["rms_tet_vertices"]))
        b["rate_E_all_nodes"] = float(np.log2(a["rms_all_nodes"] / b["rms_all_nodes"]))
    print(json.dumps({"order": order, "levels": rows}))
    out_dir = os.environ.get("FGB_PARITY_OUT")
    if out_dir:
        with open(os.path.join(out_dir, f"analytic_hemisphere_q{order}.json"), "w") as fh:
            json.dump({"order": order, "levels": rows}, fh)
    for b in rows[1:]:
        assert b["rate_phi"] >= 1.6, rows
        assert b["rate_E_tet_vertices"] >= 1.2, rows
        assert b["rate_E_all_nodes"] >= 0.6, rows
    assert rows[-1]["rate_E_all_nodes"] >= 0.85, rows
    assert rows[-1]["max_dphi"] <= 5e-3 * rows[-1]["max_phi"], rows
    # M/A moves toward 1 with refinement and ends within 10 %
    assert abs(rows[-1]["M_over_A"] - 1) <= abs(rows[0]["M_over_A"] - 1) and abs(rows[-1]["M_over_A"] - 1) < 0.1, rows
