"""ctypes wrapper of the plain-C oracle (oracle/femocs_oracle.c) -- TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "femocs_oracle.c")
SRCS = [SRC, os.path.join(HERE, "q2_oracle.c")]
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle.so")

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
i8p = C.POINTER(C.c_int8)

__all__ = ["build_oracle", "lib", "tet_tables", "System", "Q2CSystem", "neighbour_lists", "nodal_field", "smooth_field",
           "locate_interpolate", "surface_interpolate", "read_records", "write_msh", "test_solution"]


def build_oracle(force=False):
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            [os.path.getmtime(f) for f in SRCS] + [os.path.getmtime(os.path.join(HERE, "femocs_oracle.h"))]):
        return LIB
    subprocess.run(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp", *SRCS, "-o", LIB,
                    "-lm"], check=True)
    return LIB


class OrcSystem(C.Structure):
    _fields_ = [("n", C.c_int), ("nnz", C.c_int64), ("rowptr", i64p), ("col", ip), ("val", dp), ("rhs", dp),
                ("x", dp), ("constrained", i8p), ("n_top_faces", C.c_int)]


class OrcInterp(C.Structure):
    _fields_ = [("n_tets", C.c_int), ("tets", ip), ("search", i8p), ("det", dp), ("centroid", dp),
                ("nbr_ptr", ip), ("nbr_idx", ip), ("hexs", ip), ("hexf", dp), ("quad_nodes", ip), ("sol", dp)]


class OrcSurface(C.Structure):
    _fields_ = [("n_tris", C.c_int), ("tris", ip), ("tri2tet", ip), ("n_nodes", C.c_int), ("xyz", dp)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = C.CDLL(LIB)
        L.orc_tet_tables.argtypes = [C.c_int, ip, dp, dp, dp]
        L.orc_build_system.argtypes = [C.c_int, dp, C.c_int, ip, C.c_double, C.c_int, C.c_double, C.POINTER(OrcSystem)]
        L.orc_free_system.argtypes = [C.POINTER(OrcSystem)]
        L.orc_q2_build_system.argtypes = [C.c_int, dp, C.c_int, ip, C.c_double, C.c_int, C.c_double, C.c_int, ip,
                                          C.POINTER(OrcSystem), dp]
        L.orc_system_from_csr.argtypes = [C.c_int, i64p, ip, dp, dp, dp, C.POINTER(OrcSystem)]
        L.orc_ssor_cg.argtypes = [C.POINTER(OrcSystem), dp, C.c_double, C.c_double, C.c_int]
        L.orc_jacobi_cg.argtypes = [C.POINTER(OrcSystem), dp, C.c_double, C.c_int]
        L.orc_ssor_cg_fixed.argtypes = [C.POINTER(OrcSystem), dp, C.c_double, C.c_int]
        L.orc_ssor_cg_fixed.restype = C.c_double
        L.orc_spmv.argtypes = [C.POINTER(OrcSystem), dp, dp]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_residual_comp.argtypes = [C.POINTER(OrcSystem), dp, dp]
        L.orc_nodal_field.argtypes = [C.c_int, dp, C.c_int, ip, ip, i8p, dp, dp]
        L.orc_smooth_field.argtypes = [C.c_int, dp, ip, ip, C.c_double, dp]
        L.orc_locate_interpolate.argtypes = [C.POINTER(OrcInterp), C.c_int, C.c_int, dp, ip, dp]
        L.orc_surface_interpolate.argtypes = [C.POINTER(OrcInterp), C.POINTER(OrcSurface), C.c_int, C.c_int, dp, ip,
                                              dp]
        L.orc_tet_neighbour_lists.argtypes = [C.c_int, C.c_int, ip, ip, ip, ip, C.c_int]
        _lib = L
    return _lib


def _p(a, t=dp):
    return a.ctypes.data_as(t)


def tet_tables(tets, xyz):
    tets = np.ascontiguousarray(tets, dtype=np.int32).reshape(-1)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
    nt = len(tets) // 4
    det = np.zeros(17 * nt)
    ctr = np.zeros(3 * nt)
    lib().orc_tet_tables(nt, _p(tets, ip), _p(xyz), _p(det), _p(ctr))
    return det, ctr


class System:
    """Vacuum Q1 system (CSR) with boundary conditions, as the reference assembles it."""

    def __init__(self, xyz_vert=None, cells=None, applied_field=0.0, anode_dirichlet=False, applied_potential=0.0,
                 csr=None):
        self.s = OrcSystem()
        if csr is not None:
            rowptr, col, val, rhs = (np.ascontiguousarray(a) for a in csr)
            rc = lib().orc_system_from_csr(len(rhs), _p(rowptr.astype(np.int64), i64p), _p(col.astype(np.int32), ip),
                                           _p(val.astype(np.float64)), _p(rhs.astype(np.float64)), None, C.byref(self.s))
        else:
            self._xyz = np.ascontiguousarray(xyz_vert, dtype=np.float64).reshape(-1)
            self._cells = np.ascontiguousarray(cells, dtype=np.int32).reshape(-1)
            rc = lib().orc_build_system(len(self._xyz) // 3, _p(self._xyz), len(self._cells) // 8,
                                        _p(self._cells, ip), applied_field, int(anode_dirichlet), applied_potential,
                                        C.byref(self.s))
        if rc:
            raise MemoryError("oracle system build failed")
        n, nnz = self.s.n, self.s.nnz
        self.rowptr = np.ctypeslib.as_array(self.s.rowptr, shape=(n + 1,)).copy()
        self.col = np.ctypeslib.as_array(self.s.col, shape=(nnz,)).copy()
        self.val = np.ctypeslib.as_array(self.s.val, shape=(nnz,)).copy()
        self.rhs = np.ctypeslib.as_array(self.s.rhs, shape=(n,)).copy()
        self.x0 = np.ctypeslib.as_array(self.s.x, shape=(n,)).copy()
        self.constrained = np.ctypeslib.as_array(self.s.constrained, shape=(n,)).copy()
        self.n = n

    def __del__(self):
        if getattr(self, "s", None) is not None and self.s.rowptr:
            lib().orc_free_system(C.byref(self.s))

    def ssor_cg(self, omega=1.2, tol=1e-9, max_it=10000, x=None):
        x = self.x0.copy() if x is None else np.ascontiguousarray(x, dtype=np.float64).copy()
        it = lib().orc_ssor_cg(C.byref(self.s), _p(x), omega, tol, max_it)
        return it, x

    def jacobi_cg(self, tol=1e-9, max_it=100000, x=None):
        x = self.x0.copy() if x is None else np.ascontiguousarray(x, dtype=np.float64).copy()
        it = lib().orc_jacobi_cg(C.byref(self.s), _p(x), tol, max_it)
        return it, x

    def ssor_cg_fixed(self, n_it, omega=1.2, threads=1):
        """seconds of exactly n_it SSOR-CG iterations; `threads` for the SpMV and vector
        operations (the SSOR sweeps are sequential)"""
        x = self.x0.copy()
        lib().orc_set_threads(int(threads))
        try:
            return lib().orc_ssor_cg_fixed(C.byref(self.s), _p(x), omega, n_it)
        finally:
            lib().orc_set_threads(1)

    def residual(self, x):
        """(||b - A x|| compensated, rounding floor of a plain FP64 evaluation), both absolute"""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(2)
        lib().orc_residual_comp(C.byref(self.s), _p(x), _p(out))
        return float(out[0]), float(out[1])

    def spmv(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n)
        lib().orc_spmv(C.byref(self.s), _p(x), _p(y))
        return y


class Q2CSystem(System):
    """Q2 vacuum system from oracle/q2_oracle.c (same system as oracle/q2_oracle.py, fast
    enough for the benchmark meshes). node_xyz: all nodes; cells: 8 femocs-ordered node ids
    per vacuum hex; bc: Neumann value on the top (-E0). Arrays are views of the C memory.
    cell_dofs (n_cells, 27): DoF of each lattice node; dof_node: mesh node of each vertex DoF
    (-1 for edge, face and interior DoFs); timing_ms: cell matrices, serial scatter, total."""

    def __init__(self, node_xyz, cells, bc, anode_dirichlet=False, v0=0.0, n_threads=0):
        import time
        self.s = OrcSystem()
        xyz = np.ascontiguousarray(node_xyz, dtype=np.float64).reshape(-1)
        cl = np.ascontiguousarray(cells, dtype=np.int32).reshape(-1, 8)
        nc = len(cl)
        self.cell_dofs = np.zeros((nc, 27), dtype=np.int32)
        tm = np.zeros(2)
        t0 = time.perf_counter()
        rc = lib().orc_q2_build_system(len(xyz) // 3, _p(xyz), nc, _p(cl, ip), bc, int(anode_dirichlet), v0,
                                       int(n_threads), _p(self.cell_dofs, ip), C.byref(self.s), _p(tm))
        total = (time.perf_counter() - t0) * 1e3
        if rc:
            raise MemoryError("oracle Q2 system build failed")
        n, nnz = self.s.n, self.s.nnz
        self.n = n
        self.rowptr = np.ctypeslib.as_array(self.s.rowptr, shape=(n + 1,))
        self.col = np.ctypeslib.as_array(self.s.col, shape=(nnz,))
        self.val = np.ctypeslib.as_array(self.s.val, shape=(nnz,))
        self.rhs = np.ctypeslib.as_array(self.s.rhs, shape=(n,))
        self.x0 = np.ctypeslib.as_array(self.s.x, shape=(n,)).copy()
        self.constrained = np.ctypeslib.as_array(self.s.constrained, shape=(n,))
        self.dof_node = np.full(n, -1, dtype=np.int32)
        for L, k in Q2_CORNER_LATTICE.items():
            self.dof_node[self.cell_dofs[:, L]] = cl[:, k]
        self.timing_ms = {"cell_matrices": float(tm[0]), "scatter": float(tm[1]), "total": total}


# lattice node (x fastest, 0..26) of each femocs hex vertex k: (hx + 1, hy + 1, hz + 1)
Q2_CORNER_LATTICE = {((1 + hx) + 3 * (1 + hy) + 9 * (1 + hz)): k for k, (hx, hy, hz) in enumerate(
    zip([-1, 1, 1, -1, -1, 1, 1, -1], [-1, -1, 1, 1, -1, -1, 1, 1], [-1, -1, -1, -1, 1, 1, 1, 1]))}


def neighbour_lists(n_nodes, tets, face_nbr):
    tets = np.ascontiguousarray(tets, dtype=np.int32).reshape(-1)
    fn = np.ascontiguousarray(face_nbr, dtype=np.int32).reshape(-1)
    nt = len(tets) // 4
    ptr = np.zeros(nt + 1, dtype=np.int32)
    cap = 64 * nt + 16
    idx = np.zeros(cap, dtype=np.int32)
    n = lib().orc_tet_neighbour_lists(n_nodes, nt, _p(tets, ip), _p(fn, ip), _p(ptr, ip), _p(idx, ip), cap)
    if n > cap:
        idx = np.zeros(n, dtype=np.int32)
        lib().orc_tet_neighbour_lists(n_nodes, nt, _p(tets, ip), _p(fn, ip), _p(ptr, ip), _p(idx, ip), n)
    return ptr, idx[:n].copy()


def nodal_field(xyz, hexs, hex_marker, is_vac, phi):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
    hexs = np.ascontiguousarray(hexs, dtype=np.int32).reshape(-1)
    hm = np.ascontiguousarray(hex_marker, dtype=np.int32)
    iv = np.ascontiguousarray(is_vac, dtype=np.int8)
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    n = len(xyz) // 3
    E = np.zeros(3 * n)
    lib().orc_nodal_field(n, _p(xyz), len(hexs) // 8, _p(hexs, ip), _p(hm, ip), _p(iv, i8p), _p(phi), _p(E))
    return E


def smooth_field(n_tetnodes, xyz, vptr, vidx, decay, E):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
    vptr = np.ascontiguousarray(vptr, dtype=np.int32)
    vidx = np.ascontiguousarray(vidx, dtype=np.int32)
    E = np.ascontiguousarray(E, dtype=np.float64).reshape(-1).copy()
    lib().orc_smooth_field(n_tetnodes, _p(xyz), _p(vptr, ip), _p(vidx, ip), decay, _p(E))
    return E


def locate_interpolate(tables, rank, pts):
    """tables: dict with tets, search, det, centroid, nbr_ptr, nbr_idx, hexs, hexf, quad_nodes, sol."""
    keep = {}

    def a(name, dt):
        v = np.ascontiguousarray(tables[name], dtype=dt).reshape(-1)
        keep[name] = v
        return v

    m = OrcInterp()
    m.n_tets = len(tables["tets"]) // 4 if np.ndim(tables["tets"]) == 1 else len(tables["tets"])
    m.tets = _p(a("tets", np.int32), ip)
    m.search = _p(a("search", np.int8), i8p)
    m.det = _p(a("det", np.float64))
    m.centroid = _p(a("centroid", np.float64))
    m.nbr_ptr = _p(a("nbr_ptr", np.int32), ip)
    m.nbr_idx = _p(a("nbr_idx", np.int32), ip)
    m.hexs = _p(a("hexs", np.int32), ip)
    m.hexf = _p(a("hexf", np.float64))
    m.quad_nodes = _p(a("quad_nodes", np.int32), ip)
    m.sol = _p(a("sol", np.float64))
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1)
    n = len(pts) // 3
    cells = np.zeros(n, dtype=np.int32)
    out = np.zeros(5 * n)
    lib().orc_locate_interpolate(C.byref(m), rank, n, _p(pts), _p(cells, ip), _p(out))
    return cells, out.reshape(-1, 5)


def surface_interpolate(tables, tris, tri2tet, xyz, rank, pts):
    """Surface (2-D) location + interpolation of LinearTriangles (rank 1) / QuadraticTriangles
    (rank 2) over the tet tables of locate_interpolate; tris (n,3), tri2tet (n,2), xyz the node
    coordinates. Returns (triangle per point, 5 values per point)."""
    keep = {}

    def a(name, dt, src=None):
        v = np.ascontiguousarray(tables[name] if src is None else src, dtype=dt).reshape(-1)
        keep[name] = v
        return v

    m = OrcInterp()
    m.n_tets = len(np.asarray(tables["tets"]).reshape(-1)) // 4
    m.tets = _p(a("tets", np.int32), ip)
    m.search = _p(a("search", np.int8), i8p)
    m.det = _p(a("det", np.float64))
    m.centroid = _p(a("centroid", np.float64))
    m.nbr_ptr = _p(a("nbr_ptr", np.int32), ip)
    m.nbr_idx = _p(a("nbr_idx", np.int32), ip)
    m.hexs = _p(a("hexs", np.int32), ip)
    m.hexf = _p(a("hexf", np.float64))
    m.quad_nodes = _p(a("quad_nodes", np.int32), ip)
    m.sol = _p(a("sol", np.float64))
    sf = OrcSurface()
    t = a("tris", np.int32, tris)
    sf.n_tris = len(t) // 3
    sf.tris = _p(t, ip)
    sf.tri2tet = _p(a("tri2tet", np.int32, tri2tet), ip)
    x = a("xyz", np.float64, xyz)
    sf.n_nodes = len(x) // 3
    sf.xyz = _p(x)
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1)
    n = len(pts) // 3
    cells = np.zeros(n, dtype=np.int32)
    out = np.zeros(5 * n)
    lib().orc_surface_interpolate(C.byref(m), C.byref(sf), rank, n, _p(pts), _p(cells, ip), _p(out))
    return cells, out.reshape(-1, 5)


def test_solution(xyz):
    """Smooth nodal test field (same formula as oracle/ref_driver.cpp test_solution)."""
    p = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    phi = 0.25 * x - 0.5 * y + 0.125 * z + 1e-3 * x * z + 2e-4 * x * y * y - 3e-5 * z * z * y
    sol = np.zeros((len(p), 5))
    sol[:, 0] = 0.1 + 1e-3 * y
    sol[:, 1] = -0.2 + 2e-3 * z
    sol[:, 2] = 0.3 + 1e-3 * x
    sol[:, 3] = 1.0 + 1e-2 * z
    sol[:, 4] = phi
    return sol


def read_records(path):
    """Reader of oracle/ref_driver output records."""
    out = {}
    b = open(path, "rb").read()
    o = 0
    while o < len(b):
        name = b[o:o + 16].split(b"\0")[0].decode()
        o += 16
        t = chr(b[o])
        o += 1
        n = struct.unpack("<q", b[o:o + 8])[0]
        o += 8
        dt, sz = ("<f8", 8) if t == "d" else ("<i4", 4)
        out[name] = np.frombuffer(b[o:o + n * sz], dtype=dt).copy()
        o += n * sz
    return out


def write_msh(path, xyz, tets, markers, tris=None, tri_marker=2):
    """Gmsh 2.2 ASCII tetrahedral mesh, coordinates printed round-trip exact; optional surface
    triangles (element type 2) after the tets."""
    xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    tets = np.asarray(tets).reshape(-1, 4)
    tris = np.zeros((0, 3), dtype=np.int64) if tris is None else np.asarray(tris).reshape(-1, 3)
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(xyz))
        for i, p in enumerate(xyz):
            f.write("%d %r %r %r\n" % (i + 1, float(p[0]), float(p[1]), float(p[2])))
        f.write("$EndNodes\n$Elements\n%d\n" % (len(tets) + len(tris)))
        for i, (t, m) in enumerate(zip(tets, markers)):
            f.write("%d 4 2 %d %d %d %d %d %d\n" % (i + 1, m, m, t[0] + 1, t[1] + 1, t[2] + 1, t[3] + 1))
        for i, t in enumerate(tris):
            f.write("%d 2 2 %d %d %d %d %d\n" % (len(tets) + i + 1, tri_marker, tri_marker, t[0] + 1, t[1] + 1,
                                                  t[2] + 1))
        f.write("$EndElements\n")
