"""Restatement of the reference's current and heat systems on the bulk hexahedra -- TEST
INFRASTRUCTURE ONLY (numpy/scipy, small meshes). Parity unpinned: the reference assembles these
inside deal.II 9.2 (absent); this follows its source line by line and is checked with known
answers (a linear potential through a flat slab, an unheated body staying at T_ambient).

* region: hexes with a negative marker (bulk), vertices compacted in ascending node order
  (src/DealSolver.cpp:192-208);
* boundary (CurrentHeatSolver::mark_mesh, src/CurrentHeatSolver.cpp:535-539, through
  DealSolver::mark_boundary, src/DealSolver.cpp:461-518): faces held by one bulk hex, their
  centroid bounding box; x/y extremes natural, z min -> copper bottom (Dirichlet), the rest ->
  copper surface (per-face Neumann values, numbered cells ascending and deal.II faces x-, x+,
  y-, y+, z-, z+ as DealSolver::assemble_rhs walks them, src/DealSolver.cpp:390-430);
* current (CurrentSolver::assemble_local_cell, :453-489): sigma = 1 stiffness, 2x2x2 Gauss;
* heat (HeatSolver::assemble_local_cell, :347-398): JxW (gamma N_i N_j + kappa(T_q) grad N_i .
  grad N_j), rhs JxW N_i (gamma T_q + sigma(T_q) |grad phi_q|^2), gamma = rho_cp / dt;
* material (PhysicalQuantities, src/PhysicalQuantities.cpp:31-64, 173-184);
* Dirichlet: symmetric elimination keeping the diagonal (MatrixTools::apply_boundary_values).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl

HX = np.array([-1, 1, 1, -1, -1, 1, 1, -1], dtype=float)
HY = np.array([-1, -1, 1, 1, -1, -1, 1, 1], dtype=float)
HZ = np.array([-1, -1, -1, -1, 1, 1, 1, 1], dtype=float)
# femocs hex faces (cyclic corner order) and the deal.II face order x-, x+, y-, y+, z-, z+
FACES = np.array([[0, 1, 2, 3], [4, 5, 6, 7], [0, 3, 7, 4], [1, 2, 6, 5], [0, 1, 5, 4], [3, 2, 6, 7]])
DEAL_ORDER = [2, 3, 0, 1, 4, 5]
G = 1.0 / np.sqrt(3.0)


def _q_points():
    pts = []
    for q in range(8):
        pts.append(((G if q & 1 else -G), (G if q & 2 else -G), (G if q & 4 else -G)))
    return np.array(pts)


def resistivity(T, tab_T, tab_rho):
    t = np.clip(T, tab_T[0], tab_T[-1])
    return 10.0 * np.interp(t, tab_T, tab_rho)


def sigma(T, tab_T, tab_rho):
    return 1.0 / resistivity(T, tab_T, tab_rho)


def kappa(T, tab_T, tab_rho, lorentz):
    return lorentz * np.clip(T, tab_T[0], tab_T[-1]) * sigma(T, tab_T, tab_rho)


class BulkSystem:
    def __init__(self, node_xyz, hexes, hex_marker):
        X = np.asarray(node_xyz, dtype=float).reshape(-1, 3)
        H = np.asarray(hexes).reshape(-1, 8)
        hm = np.asarray(hex_marker)
        self.cells_hex = np.flatnonzero(hm < 0)
        cells = H[self.cells_hex]
        used = np.unique(cells)
        n2v = -np.ones(len(X), dtype=np.int64)
        n2v[used] = np.arange(len(used))
        self.vertex2node = used
        self.cells = n2v[cells]
        self.xyz = X[used]
        self.n = len(used)
        # boundary faces
        keys = {}
        for c, cv in enumerate(self.cells):
            for f in range(6):
                k = tuple(sorted(cv[FACES[f]]))
                keys.setdefault(k, []).append((c, f))
        bnd = [v[0] for v in keys.values() if len(v) == 1]
        bnd.sort(key=lambda cf: (cf[0], DEAL_ORDER.index(cf[1])))
        ctr = np.array([self.xyz[self.cells[c][FACES[f]]].mean(axis=0) for c, f in bnd])
        lo, hi = ctr.min(axis=0), ctr.max(axis=0)
        eps = 1e-6
        self.fixed = np.zeros(self.n, dtype=bool)
        self.surface = []  # (cell, face) in value order
        for (c, f), x in zip(bnd, ctr):
            if abs(x[0] - lo[0]) <= eps or abs(x[0] - hi[0]) <= eps or abs(x[1] - lo[1]) <= eps or \
                    abs(x[1] - hi[1]) <= eps:
                continue
            if abs(x[2] - lo[2]) <= eps:
                self.fixed[self.cells[c][FACES[f]]] = True
            else:
                self.surface.append((c, f))
        self.surface_centroids = np.array([self.xyz[self.cells[c][FACES[f]]].mean(axis=0) for c, f in self.surface])
        self._geometry()

    def _geometry(self):
        qp = _q_points()
        N = np.array([[(1 + x * HX[k]) * (1 + y * HY[k]) * (1 + z * HZ[k]) / 8 for k in range(8)] for x, y, z in qp])
        dN = np.array([[[HX[k] * (1 + y * HY[k]) * (1 + z * HZ[k]) / 8, (1 + x * HX[k]) * HY[k] * (1 + z * HZ[k]) / 8,
                         (1 + x * HX[k]) * (1 + y * HY[k]) * HZ[k] / 8] for k in range(8)] for x, y, z in qp])
        P = self.xyz[self.cells]  # (nc, 8, 3)
        J = np.einsum("cka,qkb->cqab", P, dN)
        self.det = np.abs(np.linalg.det(J))
        inv = np.linalg.inv(J)
        self.grad = np.einsum("cqba,qkb->cqka", inv, dN)  # grad_x N_k at q
        self.N = N

    def _matrix(self, ke):
        rows = np.repeat(self.cells, 8, axis=1).ravel()
        cols = np.tile(self.cells, (1, 8)).ravel()
        return sp.csr_matrix((ke.ravel(), (rows, cols)), shape=(self.n, self.n))

    def _neumann(self, vals):
        b = np.zeros(self.n)
        for (c, f), v in zip(self.surface, vals):
            Pq = self.xyz[self.cells[c][FACES[f]]]
            for s in (-G, G):
                for t in (-G, G):
                    Nf = 0.25 * np.array([(1 - s) * (1 - t), (1 + s) * (1 - t), (1 + s) * (1 + t), (1 - s) * (1 + t)])
                    ds = 0.25 * (-(1 - t) * Pq[0] + (1 - t) * Pq[1] + (1 + t) * Pq[2] - (1 + t) * Pq[3])
                    dt = 0.25 * (-(1 - s) * Pq[0] - (1 + s) * Pq[1] + (1 + s) * Pq[2] + (1 - s) * Pq[3])
                    b[self.cells[c][FACES[f]]] += Nf * v * np.linalg.norm(np.cross(ds, dt))
        return b

    def _solve(self, A, b, g):
        fx = np.flatnonzero(self.fixed)
        gv = np.zeros(self.n)
        gv[fx] = g
        diag = A.diagonal().copy()
        b = b - A @ gv
        free = sp.diags((~self.fixed).astype(float))
        A2 = (free @ A @ free).tocsr() + sp.csr_matrix((diag[fx], (fx, fx)), shape=A.shape)
        b[fx] = diag[fx] * g
        return spl.spsolve(A2.tocsc(), b)

    def current(self, face_j):
        ke = np.einsum("cq,cqia,cqja->cij", self.det, self.grad, self.grad)
        return self._solve(self._matrix(ke), self._neumann(face_j), 0.0)

    def heat(self, T_prev, phi, dt, face_q, tab_T, tab_rho, lorentz, rho_cp, t_ambient):
        gamma = rho_cp / dt
        Tc = T_prev[self.cells]  # (nc, 8)
        Tq = np.einsum("qk,ck->cq", self.N, Tc)
        gp = np.einsum("cqka,ck->cqa", self.grad, phi[self.cells])
        kap = kappa(Tq, tab_T, tab_rho, lorentz)
        sig = sigma(Tq, tab_T, tab_rho)
        ke = np.einsum("cq,qi,qj->cij", self.det * gamma, self.N, self.N) + \
            np.einsum("cq,cqia,cqja->cij", self.det * kap, self.grad, self.grad)
        src = gamma * Tq + sig * (gp ** 2).sum(axis=2)
        fe = np.einsum("cq,qi->ci", self.det * src, self.N)
        b = np.zeros(self.n)
        np.add.at(b, self.cells.ravel(), fe.ravel())
        b += self._neumann(face_q)
        return self._solve(self._matrix(ke), b, t_ambient)
