"""Boundary-fitted test meshes of a hemisphere on a plane, and the reference's analytic field
for it (test infrastructure).

FieldReader::get_analyt_potential / get_analyt_field (src/SolutionReader.cpp:501-524) give,
for a conducting hemisphere of radius R on a grounded plane in a uniform applied field E0
along z,

    phi = -E0 z (1 - (R/r)^3),   E = (3 E0 R^3 x z / r^5, 3 E0 R^3 y z / r^5,
                                      E0 (1 - R^3 (x^2 + y^2 - 2 z^2) / r^5)),

which is also the reference's field-enhancement known answer (M/A = 1 with A = 3).

The mesh covers the quarter x, y >= 0 of the vacuum between the hemisphere and the box
[0, L]^3: the octant of directions is covered by the three faces x = 1, y = 1, z = 1 of the
unit cube (n x n cells each), and every direction is blended radially from the sphere to the
box, position = (1 - s) R p/|p| + s L p, with s graded geometrically so cells stay roughly
isotropic. The planes x = 0 and y = 0 are symmetry planes of the exact solution (zero normal
derivative), which is what the reference's boundary marking makes of the x/y extremes; the
plane z = 0 and the hemisphere are copper (phi = 0); z = L is the Neumann top (-E0 there up to
(R/L)^3). Each structured cell is split into 12 tetrahedra through its centre, each face by
the diagonal through its vertex of smallest global id, so neighbouring cells agree.
"""
from __future__ import annotations

import numpy as np

VACUUM = 3


def hemisphere_mesh(n, radius=10.0, box=200.0, layers=None):
    """(xyz (N, 3), tets (M, 4) int32, markers (M,) int32) with n x n cells per cube face and
    `layers` radial cells (default 2n)"""
    m = layers or 2 * n
    kappa = np.log(box / radius)
    t = np.arange(m + 1) / m
    s = np.expm1(kappa * t) / np.expm1(kappa)
    u = np.arange(n + 1) / n
    U, V = np.meshgrid(u, u, indexing="ij")
    one = np.ones_like(U)
    faces = [np.stack([one, U, V], -1), np.stack([U, one, V], -1), np.stack([U, V, one], -1)]
    # nodes: unique directions (merge the shared patch edges by exact cube-surface coordinates)
    pts = np.concatenate([f.reshape(-1, 3) for f in faces])
    key = np.round(pts * n).astype(np.int64)
    _, first, inv = np.unique(key[:, 0] * (n + 1) ** 2 + key[:, 1] * (n + 1) + key[:, 2], return_index=True,
                              return_inverse=True)
    P = pts[first]
    D = P / np.linalg.norm(P, axis=1, keepdims=True)
    nd = len(P)
    xyz = ((1.0 - s)[:, None, None] * radius * D[None] + s[:, None, None] * box * P[None]).reshape(-1, 3)
    # exact planes: x = 0, y = 0, z = 0 where the direction has a zero component; box faces
    xyz[np.tile(P[:, 0] == 0, m + 1), 0] = 0.0
    xyz[np.tile(P[:, 1] == 0, m + 1), 1] = 0.0
    xyz[np.tile(P[:, 2] == 0, m + 1), 2] = 0.0
    dir_id = inv.reshape(3, n + 1, n + 1)
    cells = []
    for f in range(3):
        g = dir_id[f]
        for k in range(m):
            for i in range(n):
                for j in range(n):
                    q = [g[i, j], g[i + 1, j], g[i + 1, j + 1], g[i, j + 1]]
                    cells.append([k * nd + a for a in q] + [(k + 1) * nd + a for a in q])
    cells = np.array(cells, dtype=np.int64)  # (c, 8): bottom quad, top quad
    # 12 tets per cell through a centre node
    n0 = len(xyz)
    ctr = xyz[cells].mean(axis=1)
    xyz = np.r_[xyz, ctr]
    quads = [(0, 1, 2, 3), (4, 5, 6, 7), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7)]
    tets = []
    for c, cv in enumerate(cells):
        cn = n0 + c
        for qd in quads:
            v = [cv[a] for a in qd]
            a = int(np.argmin(v))
            v = v[a:] + v[:a]  # start at the smallest id: diagonal v0-v2
            tets.append([v[0], v[1], v[2], cn])
            tets.append([v[0], v[2], v[3], cn])
    tets = np.array(tets, dtype=np.int64)
    # positive orientation
    p = xyz[tets]
    vol = np.einsum("ij,ij->i", np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), p[:, 3] - p[:, 0])
    tets[vol < 0] = tets[vol < 0][:, [0, 2, 1, 3]]
    return xyz, tets.astype(np.int32), np.full(len(tets), VACUUM, dtype=np.int32)


def analytic_phi(xyz, E0, radius):
    """FieldReader::get_analyt_potential (src/SolutionReader.cpp:501-508), origin at the centre"""
    p = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    r = np.linalg.norm(p, axis=1)
    return -E0 * p[:, 2] * (1 - (radius / r) ** 3)


def analytic_field(xyz, E0, radius):
    """FieldReader::get_analyt_field (src/SolutionReader.cpp:510-524)"""
    p = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    r5 = (x * x + y * y + z * z) ** 2.5
    r3 = radius ** 3
    f = x * x + y * y - 2.0 * z * z
    return np.stack([3 * E0 * r3 * x * z / r5, 3 * E0 * r3 * y * z / r5, E0 * (1.0 - r3 * f / r5)], axis=1)
