"""Q2 restatement of the vacuum Poisson system -- TEST INFRASTRUCTURE ONLY (numpy/scipy, small
meshes).

The reference assembles Q1 only (`include/DealSolver.h:130`: no Q2 path); this is the
higher-order element on the same mesh with the reference's boundary treatment, written
independently of the CUDA code so the device assembly can be checked against it:

* DoFs: one per vacuum vertex, hex edge, hex face and hex interior (entities identified by
  their sorted corner node ids), element = 27-node Lagrange hexahedron (tensor quadratic
  Lagrange on {-1, 0, 1}^3) on the trilinear (Q1) geometry map;
* stiffness `K_e[i][j] = sum_q w_q |det J_q| grad N_i . grad N_j` with 3x3x3 Gauss points,
  the Q2 analogue of `PoissonSolver::assemble_local_cell` (`src/PoissonSolver.cpp:239-263`);
* boundary marking as `DealSolver::mark_boundary` (`src/DealSolver.cpp:461-518`): faces owned
  by one vacuum hex, sides (x/y extremes of the boundary-face centroids) natural, z max =
  top (Neumann value `bc` with 3x3 Gauss, `src/DealSolver.cpp:390-430`), all others copper
  (phi = 0, symmetric elimination as `MatrixTools::apply_boundary_values`,
  `src/DealSolver.cpp:433-440`).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

HX = np.array([-1, 1, 1, -1, -1, 1, 1, -1])
HY = np.array([-1, -1, 1, 1, -1, -1, 1, 1])
HZ = np.array([-1, -1, -1, -1, 1, 1, 1, 1])
G3 = np.array([-np.sqrt(0.6), 0.0, np.sqrt(0.6)])
W3 = np.array([5.0, 8.0, 5.0]) / 9.0


def _l(a, t):
    return [0.5 * t * (t - 1.0), 1.0 - t * t, 0.5 * t * (t + 1.0)][a]


def _dl(a, t):
    return [t - 0.5, -2.0 * t, t + 0.5][a]


def lattice(L):
    return L % 3, (L // 3) % 3, L // 9


def corner_of(a, b, c):
    """femocs local vertex at lattice corner (a, b, c), a, b, c in {0, 2}"""
    for k in range(8):
        if HX[k] + 1 == a and HY[k] + 1 == b and HZ[k] + 1 == c:
            return k
    raise ValueError


def entity_corners(L):
    a, b, c = lattice(L)
    ra = [0, 2] if a == 1 else [a]
    rb = [0, 2] if b == 1 else [b]
    rc = [0, 2] if c == 1 else [c]
    return [corner_of(i, j, k) for k in rc for j in rb for i in ra]


def _tables():
    dn = np.zeros((27, 27, 3))
    d1 = np.zeros((27, 8, 3))
    w = np.zeros(27)
    for q in range(27):
        qa, qb, qc = lattice(q)
        x, y, z = G3[qa], G3[qb], G3[qc]
        w[q] = W3[qa] * W3[qb] * W3[qc]
        for L in range(27):
            a, b, c = lattice(L)
            dn[q, L] = [_dl(a, x) * _l(b, y) * _l(c, z), _l(a, x) * _dl(b, y) * _l(c, z), _l(a, x) * _l(b, y) * _dl(c, z)]
        for k in range(8):
            d1[q, k] = [0.125 * HX[k] * (1 + y * HY[k]) * (1 + z * HZ[k]),
                        0.125 * (1 + x * HX[k]) * HY[k] * (1 + z * HZ[k]),
                        0.125 * (1 + x * HX[k]) * (1 + y * HY[k]) * HZ[k]]
    return dn, d1, w


def entity_key(cell_nodes, L):
    """key of the DoF entity of lattice node L in a cell (8 femocs-ordered node ids)"""
    return tuple(sorted(int(cell_nodes[k]) for k in entity_corners(L)))


class Q2System:
    """Assembled Q2 system (after Dirichlet elimination) on the vacuum hexes of a mesh.

    node_xyz (n_nodes, 3), hexes (n_hex, 8) femocs order, vac_cells: indices of vacuum hexes.
    bc: Neumann value on the top (PoissonSolver::setup passes -E0)."""

    def __init__(self, node_xyz, hexes, vac_cells, bc, anode_dirichlet=False, v0=0.0):
        X = np.asarray(node_xyz, dtype=np.float64).reshape(-1, 3)
        cells = np.asarray(hexes).reshape(-1, 8)[np.asarray(vac_cells)]
        nc = len(cells)
        keys = {}
        cd = np.zeros((nc, 27), dtype=np.int64)
        for c in range(nc):
            for L in range(27):
                k = ("i", c) if L == 13 else entity_key(cells[c], L)
                if k not in keys:
                    keys[k] = len(keys)
                cd[c, L] = keys[k]
        self.keys = keys
        self.cell_dofs = cd
        n = len(keys)
        self.n = n
        dn, d1, w = _tables()
        P = X[cells]  # (nc, 8, 3)
        J = np.einsum("cka,qkb->cqab", P, d1)  # dx_a / dxi_b
        det = np.linalg.det(J)
        inv = np.linalg.inv(J)  # (J^-1)[i][j]
        G = np.einsum("cqka,qlk->cqla", inv, dn)  # grad_x N = J^-T grad_xi N
        K = np.einsum("cq,cqia,cqja->cij", w[None, :] * np.abs(det), G, G)
        rows = np.repeat(cd, 27, axis=1).ravel()
        cols = np.tile(cd, (1, 27)).ravel()
        A = sp.csr_matrix((K.ravel(), (rows, cols)), shape=(n, n))
        A.sum_duplicates()
        self.nnz_pattern = A.nnz
        # boundary faces: face entities owned by one cell
        face_owner = {}
        for c in range(nc):
            for L in range(27):
                a, b, cc = lattice(L)
                if [a, b, cc].count(1) == 2:
                    k = entity_key(cells[c], L)
                    face_owner.setdefault(k, []).append((c, L))
        bfaces = [v[0] for v in face_owner.values() if len(v) == 1]
        ctr = np.array([X[[cells[c][k] for k in entity_corners(L)]].mean(axis=0) for c, L in bfaces])
        lo, hi = ctr.min(axis=0), ctr.max(axis=0)
        eps = 1e-6
        kind = np.zeros(n, dtype=np.int8)
        rhs = np.zeros(n)
        top = []
        for (c, L), x in zip(bfaces, ctr):
            if abs(x[0] - lo[0]) <= eps or abs(x[0] - hi[0]) <= eps or abs(x[1] - lo[1]) <= eps or \
                    abs(x[1] - hi[1]) <= eps:
                continue
            a0, b0, c0 = lattice(L)
            fd = np.zeros(9, dtype=np.int64)
            for v in range(3):
                for u in range(3):
                    if a0 != 1:
                        a, b, cc = a0, u, v
                    elif b0 != 1:
                        a, b, cc = u, b0, v
                    else:
                        a, b, cc = u, v, c0
                    fd[u + 3 * v] = cd[c, a + 3 * b + 9 * cc]
            if abs(x[2] - hi[2]) <= eps:
                top.append((c, fd))
            else:
                kind[fd] = 1
        for c, fd in top:
            kind[fd[kind[fd] == 0]] = 2
        # Neumann: 3x3 Gauss on the bilinear face through its corners (u, v) = (0,0),(2,0),(2,2),(0,2)
        dof_xyz = np.zeros((n, 3))
        for c in range(nc):
            for L in range(27):
                dof_xyz[cd[c, L]] = X[[cells[c][k] for k in entity_corners(L)]].mean(axis=0)
        self.dof_xyz = dof_xyz
        for c, fd in top:
            Pq = dof_xyz[fd[[0, 2, 8, 6]]]
            for iv in range(3):
                for iu in range(3):
                    s, t = G3[iu], G3[iv]
                    ds = 0.25 * (-(1 - t) * Pq[0] + (1 - t) * Pq[1] + (1 + t) * Pq[2] - (1 + t) * Pq[3])
                    dt = 0.25 * (-(1 - s) * Pq[0] - (1 + s) * Pq[1] + (1 + s) * Pq[2] + (1 - s) * Pq[3])
                    jac = np.linalg.norm(np.cross(ds, dt))
                    for q in range(9):
                        rhs[fd[q]] += W3[iu] * W3[iv] * _l(q % 3, s) * _l(q // 3, t) * bc * jac
        self.kind = kind
        fixed = (kind == 1) | ((kind == 2) if anode_dirichlet else False)
        g = np.where(kind == 2, v0, 0.0) * fixed
        diag = A.diagonal().copy()
        rhs = rhs - A @ g
        free = sp.diags((~fixed).astype(np.float64))
        fx = np.flatnonzero(fixed)
        A = (free @ A @ free).tocsr()
        A = A + sp.csr_matrix((diag[fx], (fx, fx)), shape=(n, n))
        rhs[fx] = g[fx] * diag[fx]
        self.A = A.tocsr()
        self.rhs = rhs
        self.fixed = fixed
        self.vertex_node = {k[0]: d for k, d in keys.items() if isinstance(k, tuple) and len(k) == 1}

    def solve(self):
        import scipy.sparse.linalg as spl
        return spl.spsolve(self.A.tocsc(), self.rhs)


def gpu_dof_keys(mesh, dof_cell, dof_local):
    """entity keys of GPU Q2 DoFs from (one cell, lattice index) per DoF"""
    cells = mesh.export("hex_nodes").reshape(-1, 8)[mesh.export("vac_cells")]
    out = []
    for c, L in zip(dof_cell, dof_local):
        out.append(("i", int(c)) if L == 13 else entity_key(cells[c], int(L)))
    return out
