"""Generate the golden vectors in tests/golden/ from the reference's own compiled sources.

    python tests/golden/make_golden.py            (needs the mounted FEMOCS sources)
    python tests/golden/make_golden.py --surface  (only the surface-interpolation fixtures)

The tetrahedral input meshes are synthetic nanotip meshes (femocs_gb300's seeded generator),
written as Gmsh files and read back by the reference exactly the way it reads `mesh_file`
(oracle/ref_driver.cpp). The reference then splits the tets into hexes, precomputes its
interpolator, locates and interpolates a mix of query points for ranks 1-3, recovers and
smooths the nodal field. Everything it produces is stored here as .npz (mesh arrays as
SHA-256 digests, per-point results in full).

Query points per mesh: uniform points in and slightly outside the box, tet vertices,
face centroids and edge midpoints (points shared by several tets, where the reference's
chained guess decides), the surface atoms of the tip (many lie in bulk tets, which exercises
the nearest-centroid fallback) and points inside the metal.
"""
from __future__ import annotations

import hashlib
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import femocs_gb300 as fg  # noqa: E402
from oracle import read_records, test_solution, write_msh  # noqa: E402

REF = os.environ.get("FEMOCS_REF", "/root/reference")
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")

CASES = {
    "tip_a": dict(radius=10.0, height=30.0, box_half=40.0, slab=10.0, top=120.0, h=5.0, growth=1.4, margin=6.0),
    "tip_b": dict(radius=6.0, height=24.0, box_half=24.0, slab=6.0, top=60.0, h=3.0, growth=1.5, margin=4.0),
}
MESH_ARRAYS = ["tet_nodes", "tet_nbor", "tet_marker", "hex_nodes", "hex_marker", "node_marker", "node_xyz"]


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def query_points(mesh: fg.Mesh, spec: dict, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    s = mesh.sizes()
    X = mesh.export("node_xyz").reshape(-1, 3)
    T = mesh.export("tet_nodes").reshape(-1, 4)
    b, top, slab = spec["box_half"], spec["top"], spec["slab"]
    uni = np.c_[rng.uniform(-b, b, 1200), rng.uniform(-b, b, 1200), rng.uniform(-slab, top, 1200)]
    out = np.c_[rng.uniform(-1.05 * b, 1.05 * b, 60), rng.uniform(-1.05 * b, 1.05 * b, 60),
                rng.uniform(-slab - 5, top + 5, 60)]
    verts = X[rng.integers(0, s["n_tetnodes"], 200)]
    tt = T[rng.integers(0, len(T), 150)]
    faces = (X[tt[:, 0]] + X[tt[:, 1]] + X[tt[:, 2]]) / 3.0
    edges = (X[tt[:, 0]] + X[tt[:, 3]]) / 2.0
    atoms, types = fg.synth_atoms(spec, seed=seed)
    surf = atoms[types == 2][:1500]
    bulk = atoms[types == 1][:: max(1, int((types == 1).sum() // 200))][:200]
    return np.ascontiguousarray(np.r_[uni, out, verts, faces, edges, surf, bulk], dtype=np.float64)


def make_case(name: str, spec: dict, seed: int) -> dict:
    mesh = fg.Mesh.synthetic(**spec)
    s = mesh.sizes()
    pts = query_points(mesh, spec, seed)
    with tempfile.TemporaryDirectory() as td:
        msh, pbin, obin = (os.path.join(td, f) for f in ("m.msh", "p.bin", "o.bin"))
        write_msh(msh, mesh.export("node_xyz").reshape(-1, 3)[: s["n_tetnodes"]], mesh.export("tet_nodes"),
                  mesh.export("tet_marker"))
        with open(pbin, "wb") as f:
            f.write(struct.pack("<i", len(pts)) + pts.astype("<f8").tobytes())
        subprocess.run([DRIVER, msh, pbin, obin], check=True)
        r = read_records(obin)
    rng = np.random.default_rng(seed + 1)
    sub = np.sort(rng.choice(s["n_nodes"], size=min(3000, s["n_nodes"]), replace=False)).astype(np.int32)
    e_raw = r["nodal_E_raw"].reshape(-1, 3)
    e_s = r["nodal_E_smooth"].reshape(-1, 3)
    g = dict(
        spec=np.array([spec[k] for k in ("radius", "height", "box_half", "slab", "top", "h", "growth", "margin")]),
        pts=pts,
        sizes=np.array([s["n_tetnodes"], s["n_tets"], s["n_nodes"], s["n_hexs"]], dtype=np.int64),
        edgemax=r["tet_edgemax"], decay=r["decay_factor"],
        e_nodes=sub, e_raw=e_raw[sub], e_smooth=e_s[sub], e_raw_sha=np.array(digest(r["nodal_E_raw"])),
        e_smooth_absmax=np.array([np.abs(e_s).max()]),
    )
    for a in MESH_ARRAYS:
        g["sha_" + a] = np.array(digest(r[a]))
    for rank in (1, 2, 3):
        g[f"cells_r{rank}"] = r[f"cells_r{rank}"]
        g[f"interp_r{rank}"] = r[f"interp_r{rank}"].reshape(-1, 5)
    # sanity: the test field is the one the tests will rebuild
    sol = test_solution(r["node_xyz"])
    assert sol.shape[0] == s["n_nodes"]
    return g


def surface_points(mesh: fg.Mesh, spec: dict, seed: int) -> np.ndarray:
    """Queries for surface (2-D) interpolation: surface atoms, points off triangle centroids
    along the normal, triangle vertices and edge midpoints (held by several triangles, where
    the chained guess decides), points exactly on triangles, and points far from the surface
    (nearest-centroid fallback)."""
    rng = np.random.default_rng(seed)
    tris, _, geo = mesh.surface()
    X = mesh.export("node_xyz").reshape(-1, 3)
    atoms, types = fg.synth_atoms(spec, seed=seed)
    surf = atoms[types == 2][:1200]
    pick = rng.integers(0, len(tris), 300)
    off = geo[pick, 16:19] + geo[pick, 12:15] * (rng.uniform(-0.8, 0.8, 300) * geo[pick, 15])[:, None]
    on = geo[pick[:100], 16:19]
    verts = X[tris[rng.integers(0, len(tris), 120)][:, 0]]
    tt = tris[rng.integers(0, len(tris), 120)]
    edges = (X[tt[:, 0]] + X[tt[:, 1]]) / 2.0
    b, top, slab = spec["box_half"], spec["top"], spec["slab"]
    far = np.c_[rng.uniform(-b, b, 80), rng.uniform(-b, b, 80), rng.uniform(0.5 * top, top, 80)]
    return np.ascontiguousarray(np.r_[surf, off, on, verts, edges, far], dtype=np.float64)


def make_surface_case(name: str, spec: dict, seed: int) -> dict:
    """The reference reads the mesh together with its vacuum/metal surface triangles (TetGen
    recomputes their tet pairs) and interpolates on the surface for ranks 1-3."""
    mesh = fg.Mesh.synthetic(**spec)
    s = mesh.sizes()
    tris, t2t, _ = mesh.surface()
    pts = surface_points(mesh, spec, seed)
    with tempfile.TemporaryDirectory() as td:
        msh, pbin, obin = (os.path.join(td, f) for f in ("m.msh", "p.bin", "o.bin"))
        write_msh(msh, mesh.export("node_xyz").reshape(-1, 3)[: s["n_tetnodes"]], mesh.export("tet_nodes"),
                  mesh.export("tet_marker"), tris)
        with open(pbin, "wb") as f:
            f.write(struct.pack("<i", len(pts)) + pts.astype("<f8").tobytes())
        subprocess.run([DRIVER, msh, pbin, obin], check=True)
        r = read_records(obin)
    assert digest(r["hex_nodes"]) == digest(mesh.export("hex_nodes")), "the triangles changed the hex split"
    g = dict(
        spec=np.array([spec[k] for k in ("radius", "height", "box_half", "slab", "top", "h", "growth", "margin")]),
        pts=pts, tri_nodes=r["tri_nodes"].reshape(-1, 3), tri2tet=r["tri2tet"].reshape(-1, 2),
        tri_norm=r["tri_norm"].reshape(-1, 3),
    )
    for rank in (1, 2, 3):
        g[f"cells_s{rank}"] = r[f"cells_s{rank}"]
        g[f"interp_s{rank}"] = r[f"interp_s{rank}"].reshape(-1, 5)
    return g


def main():
    if not os.path.exists(DRIVER):
        subprocess.run(["make", "-f", os.path.join(ROOT, "oracle", "Makefile.ref"), f"REF={REF}", "-j8"], cwd=ROOT,
                       check=True)
    fg.load()
    from femocs_gb300.build import build
    build()
    only_surface = "--surface" in sys.argv
    for i, (name, spec) in enumerate(CASES.items()):
        if not only_surface:
            g = make_case(name, spec, seed=100 + i)
            path = os.path.join(HERE, f"golden_{name}.npz")
            np.savez_compressed(path, **g)
            print(path, os.path.getsize(path), "bytes,", len(g["pts"]), "points, neg cells r3:",
                  int((g["cells_r3"] < 0).sum()))
        g = make_surface_case(name, spec, seed=200 + i)
        path = os.path.join(HERE, f"surface_{name}.npz")
        np.savez_compressed(path, **g)
        print(path, os.path.getsize(path), "bytes,", len(g["pts"]), "points,", len(g["tri_nodes"]),
              "triangles, neg cells s1:", int((g["cells_s1"] < 0).sum()))


if __name__ == "__main__":
    main()
