"""The reference's field path end to end on the CPU -- TEST INFRASTRUCTURE ONLY.

Chains the oracle's restatements the way `ProjectRunaway::solve_laplace` and
`Femocs::interpolate_elfield` chain the reference's steps (src/ProjectRunaway.cpp:422-447,
src/Femocs.cpp:216-238):

* vacuum system in the reference's vertex numbering (src/DealSolver.cpp:192-208), assembled
  with the Neumann top and the copper Dirichlet rows (src/PoissonSolver.cpp:170-263);
* deal.II SolverCG + PreconditionSSOR(1.2) (src/DealSolver.cpp:443-459) run far below the
  product's tolerance, so its answer stands for the exact FP64 solution;
* phi by mesh node (src/DealSolver.cpp:270-279), nodal E (src/Interpolator.cpp:125-140) and
  its smoothing (src/Interpolator.cpp:142-170);
* the reference's sequential location + interpolation (src/SolutionReader.cpp:136-165).

Meshes are duck-typed: anything with `sizes()` (a dict with n_nodes, n_tetnodes) and
`export(name)` (the arrays named below), whether the product's Mesh handle or a mesh the
oracle built itself. Only tests/, the smoke test and bench.py's parity and CPU legs use this.
"""
from __future__ import annotations

import numpy as np

from . import oracle_lib as orc

__all__ = ["tables", "vacuum_inputs", "reference_solution", "point_parity", "surface_atoms_parity"]


def tables(mesh, sol):
    """Interpolator tables of the vacuum (src/InterpolatorCells.cpp:523-629, 1205-1267) with the
    nodal solution `sol` (5 doubles per node: E, scalar1, phi)."""
    s = mesh.sizes()
    tets = mesh.export("tet_nodes")
    xyz = mesh.export("node_xyz")
    det, ctr = orc.tet_tables(tets, xyz[: 3 * s["n_tetnodes"]])
    nptr, nidx = orc.neighbour_lists(s["n_tetnodes"], tets, mesh.export("tet_nbor"))
    return dict(tets=tets, search=mesh.export("tet_search"), det=det, centroid=ctr, nbr_ptr=nptr, nbr_idx=nidx,
                hexs=mesh.export("hex_nodes"), hexf=mesh.export("hex_coeffs"), quad_nodes=mesh.export("quad_nodes"),
                sol=sol)


def vacuum_inputs(mesh):
    """Vertex coordinates and vacuum cells in the reference's vertex numbering (ascending mesh
    node ids of the vacuum hexes, src/DealSolver.cpp:192-208) and the vertex -> node map."""
    n2v = mesh.export("vac_node2vertex")
    xyz = mesh.export("node_xyz").reshape(-1, 3)
    v2n = np.flatnonzero(n2v >= 0)
    cells = mesh.export("hex_nodes").reshape(-1, 8)[mesh.export("vac_cells")]
    return xyz[v2n], n2v[cells], v2n


def reference_solution(mesh, applied_field, rel_tol=1e-13, anode_dirichlet=False, applied_potential=0.0,
                       smoothen=True, max_it=200000):
    """FP64 SSOR(1.2)-CG solution to a TRUE residual ||b - A x|| <= rel_tol ||b||, or as close to
    it as FP64 gets, and the nodal solution the reference's interpolator would hold. Returns
    (sol (n_nodes, 5), info dict with the true relative residual reached)."""
    xyz, cells, v2n = vacuum_inputs(mesh)
    s = orc.System(xyz, cells, applied_field, anode_dirichlet, applied_potential)
    bnorm = float(np.linalg.norm(s.rhs))
    # CG's recursive residual drifts from the true one near 1e-12 (the FP64 rounding floor of
    # b - A x, ~1e-12 of |b| on the nanotip meshes); like a repeated DealSolver::solve_cg call
    # (warm start from the current solution), restart until the true residual, evaluated
    # compensated, meets the tolerance or stops falling
    x, it, restarts, r_prev = None, 0, 0, np.inf
    for restarts in range(12):
        k, x = s.ssor_cg(1.2, rel_tol * bnorm, max_it, x=x)
        if k <= 0 and restarts == 0:
            raise RuntimeError(f"oracle SSOR-CG did not reach {rel_tol} in {max_it} iterations")
        it += abs(k)
        r_true, _ = s.residual(x)
        if r_true <= rel_tol * bnorm or r_true > 0.5 * r_prev:
            break
        r_prev = r_true
    n = mesh.sizes()
    phi = np.zeros(n["n_nodes"])
    phi[v2n] = x
    n2v = mesh.export("vac_node2vertex")
    E = orc.nodal_field(mesh.export("node_xyz"), mesh.export("hex_nodes"), mesh.export("hex_marker"),
                        (n2v >= 0).astype(np.int8), phi)
    if smoothen:
        E = orc.smooth_field(n["n_tetnodes"], mesh.export("node_xyz"), mesh.export("voro_ptr"),
                             mesh.export("voro_idx"), -1.0 / mesh.export("edgemax")[0], E)
    sol = np.zeros((n["n_nodes"], 5))
    sol[:, :3] = E.reshape(-1, 3)
    sol[:, 4] = phi
    r, floor = s.residual(x)
    return sol, {"ssor_iterations": int(it), "restarts": int(restarts), "rel_residual": r / bnorm,
                 "rel_floor": floor / bnorm,
                 "n_dofs": int(s.n), "system": s, "vertex2node": v2n}


def point_parity(cells, out, ref_cells, ref_out, field_floor=1e-3):
    """Per-result error of interpolated phi and E against the oracle's: cells bit-exact, max
    |dphi|, max relative |dE| over points whose oracle |E| is above field_floor x the largest
    (points in metal carry the empty value 0), and the normwise max |dE| / max |E|."""
    cells = np.asarray(cells)
    ref_cells = np.asarray(ref_cells)
    out = np.asarray(out).reshape(-1, 5)
    ref_out = np.asarray(ref_out).reshape(-1, 5)
    en = np.linalg.norm(ref_out[:, :3], axis=1)
    de = np.linalg.norm(out[:, :3] - ref_out[:, :3], axis=1)
    scale = float(en.max()) if len(en) else 0.0
    sel = en > field_floor * scale
    return {"points": int(len(cells)), "cells_bit_exact": bool(np.array_equal(cells, ref_cells)),
            "cells_differing": int((cells != ref_cells).sum()),
            "max_abs_dphi": float(np.abs(out[:, 4] - ref_out[:, 4]).max()) if len(cells) else 0.0,
            "max_abs_phi": float(np.abs(ref_out[:, 4]).max()) if len(cells) else 0.0,
            "max_rel_dE": float((de[sel] / en[sel]).max()) if sel.any() else 0.0,
            "max_dE_over_max_E": float(de.max() / scale) if scale > 0 else 0.0,
            "rel_dE_points": int(sel.sum())}


def surface_atoms_parity(mesh, sol_ref, pts, rank, cells, out):
    """point_parity of the product's results at `pts` against the oracle's location and
    interpolation of the same points with the oracle's own nodal solution."""
    ref_cells, ref_out = orc.locate_interpolate(tables(mesh, sol_ref), rank, pts)
    return point_parity(cells, out, ref_cells, ref_out)
