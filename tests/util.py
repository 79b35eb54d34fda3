"""Shared helpers of the test suite (golden loading, oracle tables from a product mesh)."""
import os

import numpy as np

import femocs_gb300 as fg
import oracle as orc

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SPEC_KEYS = ("radius", "height", "box_half", "slab", "top", "h", "growth", "margin")


def golden_cases():
    return sorted(f[len("golden_"):-4] for f in os.listdir(GOLDEN_DIR) if f.startswith("golden_") and f.endswith(".npz"))


def load_golden(name):
    g = dict(np.load(os.path.join(GOLDEN_DIR, f"golden_{name}.npz")))
    g["spec_kw"] = dict(zip(SPEC_KEYS, [float(v) for v in g["spec"]]))
    return g


def surface_cases():
    return sorted(f[len("surface_"):-4] for f in os.listdir(GOLDEN_DIR) if f.startswith("surface_") and f.endswith(".npz"))


def load_surface(name):
    g = dict(np.load(os.path.join(GOLDEN_DIR, f"surface_{name}.npz")))
    g["spec_kw"] = dict(zip(SPEC_KEYS, [float(v) for v in g["spec"]]))
    return g


def oracle_tables(mesh, sol):
    s = mesh.sizes()
    tets = mesh.export("tet_nodes")
    xyz = mesh.export("node_xyz")
    det, ctr = orc.tet_tables(tets, xyz[: 3 * s["n_tetnodes"]])
    nptr, nidx = orc.neighbour_lists(s["n_tetnodes"], tets, mesh.export("tet_nbor"))
    return dict(tets=tets, search=mesh.export("tet_search"), det=det, centroid=ctr, nbr_ptr=nptr, nbr_idx=nidx,
                hexs=mesh.export("hex_nodes"), hexf=mesh.export("hex_coeffs"), quad_nodes=mesh.export("quad_nodes"),
                sol=sol)


def vacuum_system_inputs(mesh):
    """Vertex coordinates and vacuum cells in the reference's vertex numbering
    (ascending mesh node ids of the vacuum hexes, src/DealSolver.cpp:192-208)."""
    n2v = mesh.export("vac_node2vertex")
    xyz = mesh.export("node_xyz").reshape(-1, 3)
    v2n = np.flatnonzero(n2v >= 0)
    cells = mesh.export("hex_nodes").reshape(-1, 8)[mesh.export("vac_cells")]
    return xyz[v2n], n2v[cells], v2n


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return a.shape == b.shape and bool((a.view(np.int64) == b.view(np.int64)).all())
