"""Tet -> hex split and interpolator tables of the reference, restated in numpy -- TEST
INFRASTRUCTURE ONLY.

Follows the reference's mesh preparation for the vacuum interpolator:

* nodes: tet vertices, then one node per edge (edges numbered by ascending (larger, smaller)
  vertex id), per face (numbered in the order the reference's incidence walk first meets
  them: tets in order, their local edges (i, j) with v[i] > v[j], i outer, and the two
  vertices opposite each edge) and per tet; coordinates are the IEEE mean of the parents in
  that order (src/Tethex.cpp:965-1035, 1244-1342);
* hex 4t+k is the corner of tet t around its vertex k, vertices {v_k, e0, f01, e1, e2, f02,
  tet centroid, f12}, front and back swapped when the trilinear Jacobian at the centre is
  negative (src/Tethex.cpp:1037-1102, 1565), marker +-(1 + v_k) for vacuum / bulk
  (src/TetgenMesh.cpp:353-385);
* face neighbours (TetGen's neighbour lists), searchable vacuum tets and the quadratic-tet
  mid-edge nodes (src/InterpolatorCells.cpp:523-629, 720-742, 1151-1174);
* trilinear map coefficients f0..f7 per hex (src/InterpolatorCells.cpp:1205-1245);
* the vacuum vertex compaction in ascending node order (src/DealSolver.cpp:192-208) and the
  pseudo-Voronoi smoothing stencils (src/TetgenMesh.cpp:819-837);
* the longest tet edge (decay length of the smoothing weights).

`OracleMesh` answers `sizes()` and `export(name)` like the product's mesh handle, so the
oracle pipeline runs on it without the product's library; tests/test_oracle_mesh_prep.py
checks every table against the product's bit for bit, and the golden hashes of the
reference's own split pin both.
"""
from __future__ import annotations

import numpy as np

TET_NODE, EDGE_CENTROID, FACE_CENTROID, TET_CENTROID = 1, 2, 3, 4
VACUUM = 3

# position of femocs hex vertex i in deal.II's lexicographic order
_TO_DEAL = np.array([0, 1, 5, 4, 2, 3, 7, 6])


def _local_edges(tets):
    """per tet the 6 local edges (a, b) with v[a] > v[b], a outer, b inner: (m, 6) each"""
    ii, jj = np.meshgrid(np.arange(4), np.arange(4), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()
    mask = tets[:, ii] > tets[:, jj]  # (m, 16), exactly 6 per row
    rows, cols = np.nonzero(mask)
    return ii[cols].reshape(-1, 6), jj[cols].reshape(-1, 6)


def _lex_groups(keys):
    """sort rows of `keys` (n, k) lexicographically; returns (order, group start flags)"""
    order = np.lexsort(keys.T[::-1])
    s = keys[order]
    new = np.ones(len(s), dtype=bool)
    new[1:] = np.any(s[1:] != s[:-1], axis=1)
    return order, new


def tethex_split(xyz, tets, marker):
    """(node_xyz (n, 3), node_marker, hexs (4m, 8), hex_marker, n_edges, n_faces)"""
    xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    T = np.asarray(tets, dtype=np.int64).reshape(-1, 4)
    m = len(T)
    n_old = len(xyz)
    # edges
    a, b = _local_edges(T)
    t_idx = np.arange(m)[:, None]
    hi = T[t_idx, a]
    lo = T[t_idx, b]
    ekeys = np.unique((hi << 32) | lo)
    n_edges = len(ekeys)

    def edge_id(x, y):
        k = (np.maximum(x, y) << 32) | np.minimum(x, y)
        return np.searchsorted(ekeys, k)

    # faces in first-encounter order: per tet, its local edges in order, the two other
    # vertices ascending -> 12 records (slot 0..11)
    ks = np.empty((m, 6, 2), dtype=np.int64)
    for e in range(6):
        ks[:, e, :] = _others(a[:, e], b[:, e])
    A = np.repeat(a, 2, axis=1)
    B = np.repeat(b, 2, axis=1)
    K = ks.reshape(m, 12)
    f = np.sort(np.stack([T[t_idx, A], T[t_idx, B], T[t_idx, K]], axis=2), axis=2).reshape(-1, 3)
    opp = (6 - A - B - K).reshape(-1)
    rec_tet = np.repeat(np.arange(m), 12)
    order_key = np.arange(12 * m)  # t * 12 + slot
    srt, _ = _lex_groups(np.c_[f, order_key])
    # groups by face triple (records of a group sorted by encounter order)
    fs = f[srt]
    gnew = np.ones(len(fs), dtype=bool)
    gnew[1:] = np.any(fs[1:] != fs[:-1], axis=1)
    gid = np.cumsum(gnew) - 1
    first_order = order_key[srt][gnew]  # first encounter of each group (records sorted by order inside)
    rank = np.empty(len(first_order), dtype=np.int64)
    rank[np.argsort(first_order, kind="stable")] = np.arange(len(first_order))
    n_faces = len(first_order)
    face_of_rec = np.empty(len(f), dtype=np.int64)
    face_of_rec[srt] = rank[gid]
    face_verts = np.empty((n_faces, 3), dtype=np.int64)
    face_verts[rank] = fs[gnew]
    tet_face = np.full(4 * m, -1, dtype=np.int64)
    tet_face[4 * rec_tet + opp] = face_of_rec

    # node coordinates: IEEE means of the parents in order
    X = xyz
    n_nodes = n_old + n_edges + n_faces + m
    nx = np.empty((n_nodes, 3))
    nx[:n_old] = X
    ehi, elo = ekeys >> 32, ekeys & 0xFFFFFFFF
    nx[n_old:n_old + n_edges] = ((0.0 + X[elo]) + X[ehi]) / 2
    fv = face_verts
    nx[n_old + n_edges:n_old + n_edges + n_faces] = (((0.0 + X[fv[:, 0]]) + X[fv[:, 1]]) + X[fv[:, 2]]) / 3
    nx[n_old + n_edges + n_faces:] = ((((0.0 + X[T[:, 0]]) + X[T[:, 1]]) + X[T[:, 2]]) + X[T[:, 3]]) / 4
    node_marker = np.r_[np.full(n_old, TET_NODE), np.full(n_edges, EDGE_CENTROID), np.full(n_faces, FACE_CENTROID),
                        np.full(m, TET_CENTROID)].astype(np.int8)

    # hexahedra, four per tet
    hexs = np.empty((m, 4, 8), dtype=np.int64)
    for ver in range(4):
        # the three local edges at `ver` in local-edge order and their other ends
        inc = (a == ver) | (b == ver)
        cols = np.nonzero(inc)[1].reshape(m, 3)
        ea, eb = a[t_idx, cols], b[t_idx, cols]
        other = np.where(ea == ver, eb, ea)  # (m, 3)
        vv = T[:, ver]

        def edge_node(k):
            return n_old + edge_id(vv, T[np.arange(m), other[:, k]])

        def face_node(k1, k2):
            o = 6 - ver - other[:, k1] - other[:, k2]
            return n_old + n_edges + tet_face[4 * np.arange(m) + o]

        h = np.stack([vv, edge_node(0), face_node(0, 1), edge_node(1), edge_node(2), face_node(0, 2),
                      n_old + n_edges + n_faces + np.arange(m), face_node(1, 2)], axis=1)
        d = np.empty((m, 8, 3))
        d[:, _TO_DEAL, :] = nx[h]
        neg = _orientation(d) < 0
        h[neg] = np.c_[h[neg, 4:], h[neg, :4]]
        hexs[:, ver, :] = h
    hexs = hexs.reshape(-1, 8)
    vac = np.asarray(marker).reshape(-1) == VACUUM
    vt = T.reshape(-1)
    hex_marker = np.where(np.repeat(vac, 4), 1 + vt, -1 - vt)
    return nx, node_marker, hexs.astype(np.int32), hex_marker.astype(np.int32), n_edges, n_faces


def _others(a, b):
    """the two local vertices of a tet that are not a or b, ascending"""
    allv = np.arange(4)[None, :]
    keep = (allv != a[:, None]) & (allv != b[:, None])
    return np.broadcast_to(allv, keep.shape)[keep].reshape(-1, 2)


def _orientation(d):
    """sign-bearing triple product of the centre Jacobian, deal.II vertex order d (m, 8, 3)"""
    ex = (((d[:, 1] - d[:, 0]) + (d[:, 3] - d[:, 2])) + (d[:, 5] - d[:, 4])) + (d[:, 7] - d[:, 6])
    ey = (((d[:, 2] - d[:, 0]) + (d[:, 3] - d[:, 1])) + (d[:, 6] - d[:, 4])) + (d[:, 7] - d[:, 5])
    ez = (((d[:, 4] - d[:, 0]) + (d[:, 5] - d[:, 1])) + (d[:, 6] - d[:, 2])) + (d[:, 7] - d[:, 3])
    return ((ex[:, 0] * (ey[:, 1] * ez[:, 2] - ey[:, 2] * ez[:, 1]) - ex[:, 1] * (ey[:, 0] * ez[:, 2] - ey[:, 2] * ez[:, 0]))
            + ex[:, 2] * (ey[:, 0] * ez[:, 1] - ey[:, 1] * ez[:, 0]))


def face_neighbours(tets):
    """entry 4t+j = the tet across the face opposite to vertex j, or -1"""
    T = np.asarray(tets, dtype=np.int64).reshape(-1, 4)
    m = len(T)
    faces = np.stack([np.sort(np.delete(T, j, axis=1), axis=1) for j in range(4)], axis=1).reshape(-1, 3)
    slot = np.arange(4 * m)
    order, _ = _lex_groups(np.c_[faces, slot])
    fs = faces[order]
    same = np.all(fs[1:] == fs[:-1], axis=1)
    if np.any(same[1:] & same[:-1]):
        raise ValueError("non-manifold face shared by more than two tets")
    i = np.nonzero(same)[0]
    nb = np.full(4 * m, -1, dtype=np.int32)
    nb[order[i]] = order[i + 1] // 4
    nb[order[i + 1]] = order[i] // 4
    return nb


def hex_coefficients(node_xyz, hexs):
    """trilinear coefficients f0..f7 (3 each): signed left-to-right sums from node 0, then / 8"""
    P = np.asarray(node_xyz).reshape(-1, 3)[np.asarray(hexs).reshape(-1, 8)]  # (n, 8, 3)
    k = np.arange(8)
    hx = np.where((k ^ (k >> 1)) & 1, 1, -1)
    hy = np.where(k & 2, 1, -1)
    hz = np.where(k & 4, 1, -1)
    signs = [np.ones(8, dtype=int), hx, hy, hz, hx * hy, hx * hz, hy * hz, hx * hy * hz]
    f = np.empty((len(P), 8, 3))
    for r in range(8):
        sg = signs[r]
        s = P[:, 0, :] * float(sg[0])
        for q in range(1, 8):
            s = s + P[:, q, :] if sg[q] > 0 else s - P[:, q, :]
        f[:, r, :] = s / 8.0
    return f.reshape(-1)


class OracleMesh:
    """A tet mesh prepared by the oracle; `sizes()` and `export(name)` as the product's handle."""

    def __init__(self, xyz, tets, marker):
        self.tet_xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        self.tets = np.ascontiguousarray(tets, dtype=np.int32).reshape(-1, 4)
        self.marker = np.ascontiguousarray(marker, dtype=np.int32).reshape(-1)
        nx, nm, hexs, hm, self.n_edges, self.n_faces = tethex_split(self.tet_xyz, self.tets, self.marker)
        m = len(self.tets)
        n_old = len(self.tet_xyz)
        self.t = {"node_xyz": nx.reshape(-1), "node_marker": nm.astype(np.int32), "hex_nodes": hexs.reshape(-1),
                  "hex_marker": hm, "tet_nodes": self.tets.reshape(-1), "tet_marker": self.marker}
        self.t["tet_nbor"] = face_neighbours(self.tets)
        self.t["tet_search"] = (self.marker == VACUUM).astype(np.int32)
        self.t["hex_coeffs"] = hex_coefficients(nx, hexs)
        # quadratic tet: vertices, then the edge nodes of edges 01, 12, 20, 03, 13, 23
        T = self.tets.astype(np.int64)
        qa, qb = [0, 1, 2, 0, 1, 2], [1, 2, 0, 3, 3, 3]
        a_, b_ = _local_edges(T)
        ekeys = np.unique((T[np.arange(m)[:, None], a_] << 32) | T[np.arange(m)[:, None], b_])
        q = np.empty((m, 10), dtype=np.int64)
        q[:, :4] = T
        for k in range(6):
            x, y = T[:, qa[k]], T[:, qb[k]]
            q[:, 4 + k] = n_old + np.searchsorted(ekeys, (np.maximum(x, y) << 32) | np.minimum(x, y))
        self.t["quad_nodes"] = q.astype(np.int32).reshape(-1)
        # vacuum compaction
        n_nodes = len(nx)
        vac_cells = np.flatnonzero(hm > 0).astype(np.int32)
        used = np.zeros(n_nodes, dtype=bool)
        used[hexs[vac_cells].reshape(-1)] = True
        n2v = np.full(n_nodes, -1, dtype=np.int32)
        n2v[used] = np.arange(int(used.sum()), dtype=np.int32)
        self.t["vac_node2vertex"] = n2v
        self.t["vac_cells"] = vac_cells
        # pseudo-Voronoi stencils of the tet vertices over the vacuum hexes
        hv = hexs[vac_cells]  # (nv, 8)
        tn = np.repeat(hm[vac_cells] - 1, 8)
        nd = hv.reshape(-1)
        keep = (nd != tn) & (nm[nd] >= EDGE_CENTROID)
        tn, nd = tn[keep], nd[keep]
        order = np.argsort(tn, kind="stable")
        self.t["voro_idx"] = nd[order].astype(np.int32)
        self.t["voro_ptr"] = np.r_[0, np.cumsum(np.bincount(tn, minlength=n_old))].astype(np.int32)
        # longest tet edge
        P = self.tet_xyz[self.tets]
        m2 = -1e300
        for i in range(4):
            for j in range(i + 1, 4):
                d = P[:, i] - P[:, j]
                m2 = max(m2, float(((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]).max()))
        self.t["edgemax"] = np.array([np.sqrt(m2)])
        self._sizes = {"n_nodes": n_nodes, "n_tetnodes": n_old, "n_tets": m, "n_hexs": 4 * m,
                       "n_vac_cells": len(vac_cells), "n_voro_idx": len(self.t["voro_idx"])}

    def sizes(self):
        return dict(self._sizes)

    def export(self, name):
        return self.t[name]
