"""Particle space charge restated in numpy -- TEST INFRASTRUCTURE ONLY.

`PoissonSolver<3>::assemble_space_charge_fast` (`src/PoissonSolver.cpp:300-319`): every super
particle adds `N_k(p) * q/eps0 * W_sp` to the rhs of its cell's DoFs, with N the trilinear
shape functions of the hex at the particle (`LinearHexahedra::shape_funs_dealii`,
`src/InterpolatorCells.cpp:1355-1358`, from `project_to_nat_coords` `:1272-1317` and
`shape_functions` `:1334-1353`). For Q2 elements the same natural coordinates feed the 27
tensor-quadratic Lagrange functions of the hex.
"""
from __future__ import annotations

import numpy as np


def natural_coords(F, p, max_iter=20, tol=1e-15):
    """Newton solve of p = f0 + f1 u + f2 v + f3 w + f4 uv + f5 uw + f6 vw + f7 uvw
    (F: 24 coefficients, 8 vectors), Cramer steps as LinearHexahedra::project_to_nat_coords."""
    F = np.asarray(F, dtype=np.float64).reshape(8, 3)
    f0 = np.asarray(p, dtype=np.float64) - F[0]
    u = v = w = 0.0
    for _ in range(max_iter):
        f = f0 - F[1] * u - F[2] * v - F[3] * w - F[4] * u * v - F[5] * u * w - F[6] * v * w - F[7] * u * v * w
        fu = F[1] + F[4] * v + F[5] * w + F[7] * v * w
        fv = F[2] + F[4] * u + F[6] * w + F[7] * u * w
        fw = F[3] + F[5] * u + F[6] * v + F[7] * u * v
        D = np.linalg.det(np.array([fu, fv, fw]))
        du = np.linalg.det(np.array([f, fv, fw])) / D
        dv = np.linalg.det(np.array([fu, f, fw])) / D
        dw = np.linalg.det(np.array([fu, fv, f])) / D
        u, v, w = u + du, v + dv, w + dw
        if du * du + dv * dv + dw * dw < tol:
            break
    return u, v, w


def trilinear(u, v, w):
    return np.array([(1 - u) * (1 - v) * (1 - w), (1 + u) * (1 - v) * (1 - w), (1 + u) * (1 + v) * (1 - w),
                     (1 - u) * (1 + v) * (1 - w), (1 - u) * (1 - v) * (1 + w), (1 + u) * (1 - v) * (1 + w),
                     (1 + u) * (1 + v) * (1 + w), (1 - u) * (1 + v) * (1 + w)]) / 8.0


def quadratic27(u, v, w):
    def l(t):
        return np.array([0.5 * t * (t - 1.0), 1.0 - t * t, 0.5 * t * (t + 1.0)])
    lu, lv, lw = l(u), l(v), l(w)
    return np.array([lu[L % 3] * lv[(L // 3) % 3] * lw[L // 9] for L in range(27)])


def space_charge_q1(hex_coeffs, hex_nodes, node2dof, n_dofs, pts, hexes, cf):
    """per-DoF rhs from particles at pts in vacuum hexes `hexes` (< 0: skipped)"""
    rhs = np.zeros(n_dofs)
    Fall = np.asarray(hex_coeffs).reshape(-1, 24)
    H = np.asarray(hex_nodes).reshape(-1, 8)
    for p, h in zip(pts, hexes):
        if h < 0:
            continue
        N = trilinear(*natural_coords(Fall[h], p))
        for k in range(8):
            d = node2dof[H[h, k]]
            if d >= 0:
                rhs[d] += N[k] * cf
    return rhs


def space_charge_q2(hex_coeffs, cell_of_hex, cell_dofs, n_dofs, pts, hexes, cf):
    """Q2 version: cell_dofs (n_cells, 27) in lattice order, cell_of_hex maps hex -> cell"""
    rhs = np.zeros(n_dofs)
    Fall = np.asarray(hex_coeffs).reshape(-1, 24)
    for p, h in zip(pts, hexes):
        if h < 0 or cell_of_hex.get(int(h), -1) < 0:
            continue
        N = quadratic27(*natural_coords(Fall[h], p))
        rhs[cell_dofs[cell_of_hex[int(h)]]] += N * cf
    return rhs
