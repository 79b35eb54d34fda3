"""femocs_gb300: GB300-native field-solve path of FEMOCS (Poisson FEM, CG, nodal field,
cell location and interpolation onto atoms), exposed through the reference's C ABI.

Python here is a thin host-side mirror of the C ABI for tests and benchmarks; the
computation runs in libfemocs_gb300.so (C++ host code + sm_103a CUDA kernels).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import FgbNanotip, dp, i64p, ip, last_error, load, ptr


def _stats_dict(st):
    return dict(iterations=int(st[0]), outer=int(st[1]), status=int(st[2]), rel_residual=st[3], bnorm=st[4],
                ms=st[5], kernel_ms=st[6], setup_ms=st[7], levels=int(st[8]), smoother_ms=st[9],
                smoother_launches=int(st[10]), spmv_ms=st[11], spmv_launches=int(st[12]), smoother_bytes=st[13])

__all__ = ["Mesh", "Field", "Femocs", "Heat", "nanotip", "synth_atoms", "synth_probes", "load", "last_error",
           "CONFIG1", "CONFIG2", "FgbNanotip", "DeviceBuffer"]


def nanotip(radius=20.0, height=80.0, box_half=100.0, slab=20.0, top=600.0, h=8.0, growth=1.3, margin=10.0):
    """Nanotip geometry + grid grading (Angstrom)."""
    return FgbNanotip(radius, height, box_half, slab, top, h, growth, margin)


# Synthetic stand-ins for the benchmark configurations (tip radius/height, slab, vacuum top as
# in the workload descriptions; grid spacing chosen for the stated hex counts).
CONFIG1 = dict(radius=20.0, height=80.0, box_half=100.0, slab=20.0, top=600.0, h=7.0, growth=1.25, margin=12.0)
CONFIG2 = dict(radius=50.0, height=400.0, box_half=400.0, slab=40.0, top=2500.0, h=9.5, growth=1.18, margin=20.0)


class Mesh:
    """Host-prepared tetrahedral mesh (tet->hex split, neighbour lists, interpolation tables)."""

    SIZE_NAMES = ["n_tetnodes", "n_tets", "n_nodes", "n_hexs", "n_vac_vertices", "n_vac_cells", "n_nbr_idx",
                  "n_voro_idx"]

    def __init__(self, handle):
        if not handle:
            raise RuntimeError("mesh construction failed: " + last_error())
        self.h = handle
        self._sizes = None

    @classmethod
    def from_arrays(cls, xyz, tets, markers, device=False):
        """Prepare a tet mesh (vertices, 4 vertex ids per tet, one region marker per tet) on
        the host or, with device=True, by kernels on the current CUDA device (same tables)."""
        lib = load()
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        tets = np.ascontiguousarray(tets, dtype=np.int32).reshape(-1)
        markers = np.ascontiguousarray(markers, dtype=np.int32).reshape(-1)
        fn = lib.fgb_mesh_from_arrays_device if device else lib.fgb_mesh_from_arrays
        return cls(fn(len(xyz) // 3, ptr(xyz), len(tets) // 4, ptr(tets, ip), ptr(markers, ip)))

    @classmethod
    def synthetic(cls, device=False, **kw):
        spec = nanotip(**kw)
        fn = load().fgb_mesh_synthetic_device if device else load().fgb_mesh_synthetic
        return cls(fn(C.byref(spec)))

    def set_surface(self, tris, tri2tet):
        """Replace the surface triangles (3 tet-mesh node ids and 2 tets per triangle)."""
        tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1)
        tri2tet = np.ascontiguousarray(tri2tet, dtype=np.int32).reshape(-1)
        if load().fgb_mesh_set_surface(self.h, len(tris) // 3, ptr(tris, ip), ptr(tri2tet, ip)) != 0:
            raise RuntimeError(last_error())

    def surface(self):
        """(tris (n,3), tri2tet (n,2), geo (n,19)) of the surface triangles"""
        n = int(load().fgb_mesh_surface_tris(self.h))
        out = []
        for name, dt, k in (("surf_tris", np.int32, 3), ("surf_tri2tet", np.int32, 2), ("surf_geo", np.float64, 19)):
            a = np.zeros(max(k * n, 1), dtype=dt)
            if load().fgb_mesh_export(self.h, name.encode(), a.ctypes.data_as(C.c_void_p)) != 0:
                raise RuntimeError(last_error())
            out.append(a[: k * n].reshape(n, k))
        return tuple(out)

    def prep_timing(self):
        """{"kernel_ms": device time of the preparation kernels (0 on the host),
        "total_ms": wall time of the preparation}"""
        o = np.zeros(2)
        load().fgb_mesh_prep_timing(self.h, ptr(o))
        return dict(kernel_ms=float(o[0]), total_ms=float(o[1]))

    @classmethod
    def read_gmsh(cls, path):
        return cls(load().fgb_mesh_read_gmsh(path.encode()))

    def __del__(self):
        if getattr(self, "h", None):
            load().fgb_mesh_free(self.h)
            self.h = None

    def sizes(self):
        if self._sizes is None:
            o = np.zeros(12, dtype=np.int64)
            load().fgb_mesh_sizes(self.h, ptr(o, i64p))
            self._sizes = dict(zip(self.SIZE_NAMES, o[:8].tolist()))
        return self._sizes

    def q2_sizes(self):
        """Q2 structure built on the host: DoFs, nonzeros, top faces, longest row."""
        o = np.zeros(4, dtype=np.int64)
        if load().fgb_mesh_q2_sizes(self.h, ptr(o, i64p)) != 0:
            raise RuntimeError(last_error())
        return dict(n_dofs=int(o[0]), nnz=int(o[1]), n_top_faces=int(o[2]), max_row=int(o[3]))

    def cell_blocks(self, cells_per_block=256, max_dofs=4096):
        """Cell blocks of the Q2 structure (host-built and validated against every invariant the
        Q2 element-by-element kernels rely on): counts and a digest of all arrays."""
        o = np.zeros(8, dtype=np.int64)
        if load().fgb_mesh_cell_blocks(self.h, int(cells_per_block), int(max_dofs), ptr(o, i64p)) != 0:
            raise RuntimeError(last_error())
        keys = ("n_blocks", "max_cells", "max_dofs", "n_local", "n_slots", "n_split", "n_complete")
        d = dict(zip(keys, (int(v) for v in o[:7])))
        d["digest"] = int(o[7].view(np.uint64))
        return d

    def export(self, name):
        s = self.sizes()
        shapes = {
            "tet_nodes": (np.int32, 4 * s["n_tets"]), "tet_marker": (np.int32, s["n_tets"]),
            "tet_nbor": (np.int32, 4 * s["n_tets"]), "node_xyz": (np.float64, 3 * s["n_nodes"]),
            "node_marker": (np.int32, s["n_nodes"]), "hex_nodes": (np.int32, 8 * s["n_hexs"]),
            "hex_marker": (np.int32, s["n_hexs"]), "tet_det": (np.float64, 17 * s["n_tets"]),
            "tet_centroid": (np.float64, 3 * s["n_tets"]), "hex_coeffs": (np.float64, 24 * s["n_hexs"]),
            "nbr_ptr": (np.int32, s["n_tets"] + 1), "nbr_idx": (np.int32, s["n_nbr_idx"]),
            "quad_nodes": (np.int32, 10 * s["n_tets"]), "voro_ptr": (np.int32, s["n_tetnodes"] + 1),
            "voro_idx": (np.int32, s["n_voro_idx"]), "vac_node2vertex": (np.int32, s["n_nodes"]),
            "vac_cells": (np.int32, s["n_vac_cells"]), "tet_search": (np.int32, s["n_tets"]),
            "edgemax": (np.float64, 1), "node_parents": (np.int32, 4 * s["n_nodes"]),
        }
        if name.startswith("surf_"):
            nt = int(load().fgb_mesh_surface_tris(self.h))
            n_nbr = int(self.export("surf_nbr_ptr")[-1]) if name == "surf_nbr_idx" and nt > 0 else 0
            shapes.update({"surf_tris": (np.int32, 3 * nt), "surf_tri2tet": (np.int32, 2 * nt),
                           "surf_geo": (np.float64, 19 * nt), "surf_nbr_ptr": (np.int32, nt + 1 if nt else 0),
                           "surf_nbr_idx": (np.int32, n_nbr)})
        dt, n = shapes[name]
        out = np.zeros(max(n, 1), dtype=dt)
        if load().fgb_mesh_export(self.h, name.encode(), out.ctypes.data_as(C.c_void_p)) != 0:
            raise RuntimeError(last_error())
        return out[:n]


class Field:
    """Device-resident Poisson system + interpolator of one mesh (PoissonSolver verbs)."""

    def __init__(self, mesh: Mesh, order=1):
        self.mesh = mesh
        self.order = order
        self.h = load().fgb_field_create_order(mesh.h, int(order))
        if not self.h:
            raise RuntimeError("field creation failed: " + last_error())
        o = np.zeros(4, dtype=np.int64)
        load().fgb_field_sizes(self.h, ptr(o, i64p))
        self.n_dofs, self.nnz, self.n_top_faces, self.n_sell = (int(v) for v in o)

    @classmethod
    def borrowed(cls, handle, mesh_sizes):
        """Wrap a field handle owned elsewhere (e.g. femocs_field of a FEMOCS instance)."""
        if not handle:
            raise RuntimeError(last_error())
        f = cls.__new__(cls)
        f.mesh = None
        f._mesh_sizes = mesh_sizes
        f.h = handle
        o = np.zeros(4, dtype=np.int64)
        load().fgb_field_sizes(f.h, ptr(o, i64p))
        f.n_dofs, f.nnz, f.n_top_faces, f.n_sell = (int(v) for v in o)
        return f

    def __del__(self):
        if getattr(self, "h", None):
            load().fgb_field_free(self.h)
            self.h = None

    def _n_nodes(self):
        return self.mesh.sizes()["n_nodes"] if self.mesh is not None else self._mesh_sizes["n_nodes"]

    def _ok(self, rc):
        if rc != 0:
            raise RuntimeError(last_error())

    def setup(self, applied_field, applied_potential=0.0):
        self._ok(load().fgb_field_setup(self.h, applied_field, applied_potential))

    def assemble(self, full_run=True, anode_dirichlet=False):
        self._ok(load().fgb_field_assemble(self.h, int(full_run), int(anode_dirichlet)))

    def solve(self, precision=2, rel_tol=1e-9, abs_tol=0.0, max_iter=10000, inner_tol=0.0):
        """precision 0: FP64 Jacobi-PCG; 1: FP32 Jacobi-PCG with FP64 refinement;
        2: FP64 CG with an FP32 multigrid V-cycle as preconditioner; 3: FP32 CG with the
        V-cycle and its level-0 operator, inside FP64 refinement. inner_tol: residual
        reduction per refinement (0: 0.1 for precision 1, 1e-3 for precision 3)."""
        rc = load().fgb_field_solve(self.h, precision, rel_tol, abs_tol, max_iter, inner_tol, None)
        if rc == -(2 ** 31):
            raise RuntimeError(last_error())
        st = np.zeros(14)
        self._ok(load().fgb_field_last_stats(self.h, ptr(st)))
        return rc, _stats_dict(st)

    def set_outer_spmv(self, mode=1):
        """Outer SpMV of the multigrid PCG: 1 the SELL matrix as FP32 hi/lo pairs (Q1 default),
        2 the same arithmetic over cell blocks (Q2 default), 0 the FP64 SELL matrix."""
        self._ok(load().fgb_field_set_outer_spmv(self.h, int(mode)))

    def set_cell_blocks(self, cells_per_block=256, max_dofs=4096):
        """Q2: limits of the cell blocks (hexes 1..256, DoFs 27..4096 per block)."""
        self._ok(load().fgb_field_set_cell_blocks(self.h, int(cells_per_block), int(max_dofs)))

    def outer_spmv_bytes(self):
        """Algorithmic bytes of one outer SpMV launch in the current mode."""
        b = load().fgb_field_outer_spmv_bytes(self.h)
        if b < 0:
            raise RuntimeError(last_error())
        return b

    def set_level0_ebe(self, on=True):
        """Q2: finest multigrid level element by element by cell blocks (True, the default) or
        through the SELL matrix (False)."""
        self._ok(load().fgb_field_set_level0_ebe(self.h, int(on)))

    def set_ke_tensor(self, on=True):
        """Q2 element matrices on the tensor cores (True) or as FP32 hi/lo pairs (False)."""
        self._ok(load().fgb_field_set_ke_tensor(self.h, int(on)))

    def element_matrices(self):
        """Element matrices of the last full assembly (Q2: (cells, 378) packed upper triangles)."""
        n = int(load().fgb_field_export_element_matrices(self.h, None))
        if n < 0:
            raise RuntimeError(last_error())
        out = np.zeros(max(n, 1))
        if load().fgb_field_export_element_matrices(self.h, ptr(out)) < 0:
            raise RuntimeError(last_error())
        return out[:n]

    def set_level0_stream(self, on=True):
        """Q2 level 0 by cell blocks: element matrices through the bulk-copy ring (True) or
        loaded by the applying warps (False, the default)."""
        self._ok(load().fgb_field_set_level0_stream(self.h, int(on)))

    def set_level0_operator(self, kind):
        """Q2 level 0 by cell blocks: 0 element matrices, 1 / 2 geometric factors in FP32 / FP16
        applied by sum factorisation. Returns the kind in use."""
        rc = load().fgb_field_set_level0_operator(self.h, int(kind))
        if rc < 0:
            raise RuntimeError(last_error())
        return rc

    def set_level0_prefetch(self, cells):
        """Q2 level 0 by cell blocks: L2 prefetch of the element matrices `cells` cells ahead of
        each warp's loads (0 = off)."""
        self._ok(load().fgb_field_set_level0_prefetch(self.h, int(cells)))

    def set_coarse_cycles(self, level=0, cycles=1):
        """Multigrid: cycles of level+1 per coarse-grid correction at `level` (1 = V-cycle)."""
        self._ok(load().fgb_field_set_coarse_cycles(self.h, level, cycles))

    def set_smoothing(self, degree=0, lo=0.0):
        """Chebyshev degree and interval of the finest multigrid level (0: defaults)."""
        self._ok(load().fgb_field_set_smoothing(self.h, int(degree), float(lo)))

    def set_lazy_matrix(self, on=True):
        """Q2: form the assembled SELL matrices only when something reads them (default) or
        at every assembly (False); results are the same."""
        self._ok(load().fgb_field_set_lazy_matrix(self.h, int(bool(on))))

    def set_level_smoothing(self, level, degree=0, lo=0.0):
        """Chebyshev degree and interval of coarser multigrid level `level` >= 1 (Q2: level 1
        is the Q1 system); 0 restores the default, from the next solve, without a rebuild."""
        self._ok(load().fgb_field_set_level_smoothing(self.h, int(level), int(degree), float(lo)))

    def set_profiling(self, on=True):
        """Record CUDA event pairs around the multigrid path's hot launches."""
        self._ok(load().fgb_field_set_profiling(self.h, int(on)))

    def amg_levels(self):
        buf = C.create_string_buffer(4096)
        self._ok(load().fgb_field_amg_levels(self.h, buf, 4096))
        return buf.value.decode()

    def space_charge(self, xyz, charge_factor, hex_cells=None, accumulate=False):
        """PIC space charge of particles (host xyz, optional vacuum hex ids) for the next
        assemble; returns the number of particles outside the vacuum hexes."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        n = len(xyz)
        d_pts = DeviceBuffer(max(24 * n, 8))
        d_pts.upload(xyz)
        d_hex = None
        if hex_cells is not None:
            hc = np.ascontiguousarray(hex_cells, dtype=np.int32)
            d_hex = DeviceBuffer(max(4 * n, 4))
            d_hex.upload(hc)
        sk = C.c_int(0)
        self._ok(load().fgb_field_space_charge(self.h, n, C.c_void_p(d_pts.ptr),
                                               C.c_void_p(d_hex.ptr) if d_hex is not None else None,
                                               float(charge_factor), int(accumulate), C.byref(sk)))
        self._ok(load().fgb_device_sync())
        return sk.value

    def clear_space_charge(self):
        self._ok(load().fgb_field_clear_space_charge(self.h))

    def solution(self):
        """The solution vector in the field's DoF order."""
        out = np.zeros(self.n_dofs)
        self._ok(load().fgb_field_export_solution(self.h, ptr(out)))
        return out

    def q2_dofs(self):
        """(cell, lattice index) holding every Q2 DoF."""
        dc = np.zeros(self.n_dofs, dtype=np.int32)
        dl = np.zeros(self.n_dofs, dtype=np.int32)
        self._ok(load().fgb_field_q2_dofs(self.h, ptr(dc, ip), ptr(dl, ip)))
        return dc, dl

    def extract(self, smoothen=True):
        self._ok(load().fgb_field_extract(self.h, int(smoothen)))

    def phi_nodes(self):
        out = np.zeros(self._n_nodes())
        self._ok(load().fgb_field_export_phi_nodes(self.h, ptr(out)))
        return out

    def set_phi_nodes(self, phi):
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        self._ok(load().fgb_field_import_phi_nodes(self.h, ptr(phi)))

    def nodal(self):
        out = np.zeros(5 * self._n_nodes())
        self._ok(load().fgb_field_get_nodal(self.h, ptr(out)))
        return out.reshape(-1, 5)

    def set_nodal(self, sol5):
        sol5 = np.ascontiguousarray(sol5, dtype=np.float64).reshape(-1)
        self._ok(load().fgb_field_set_nodal(self.h, ptr(sol5)))

    def interpolate(self, xyz, rank=3, stats=False):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        n = len(xyz) // 3
        cells = np.zeros(max(n, 1), dtype=np.int32)
        out = np.zeros(max(5 * n, 1))
        st = np.zeros(5, dtype=np.int64)
        self._ok(load().fgb_field_interpolate(self.h, n, ptr(xyz), rank, ptr(cells, ip), ptr(out), ptr(st, i64p)))
        res = (cells[:n], out[:5 * n].reshape(-1, 5))
        if stats:
            return res + (dict(zip(["n", "walk_failed", "fallback", "dependent", "longest_run"], st.tolist())),)
        return res

    def interpolate_surface(self, xyz, rank=1):
        """Surface (2-D) location + interpolation (rank 1 linear, 2 quadratic in the tet, 3
        trilinear in the hex of the quadrangle): (triangle, or quadrangle for rank 3, per point,
        negative when no triangle holds it; 5 values per point)."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        n = len(xyz) // 3
        cells = np.zeros(max(n, 1), dtype=np.int32)
        out = np.zeros(max(5 * n, 1))
        self._ok(load().fgb_field_interpolate_surface(self.h, n, ptr(xyz), rank, ptr(cells, ip), ptr(out)))
        return cells[:n], out[:5 * n].reshape(-1, 5)

    def mark(self, slot):
        """Record CUDA event `slot` (0..7) on the field's stream."""
        self._ok(load().fgb_field_mark(self.h, slot))

    def elapsed(self, a, b):
        """Milliseconds between events a and b (waits for b)."""
        return load().fgb_field_elapsed(self.h, a, b)

    def interpolate_device(self, n, d_xyz, rank, d_cells, d_out):
        self._ok(load().fgb_field_interpolate_device(self.h, n, d_xyz, rank, d_cells, d_out))

    def system(self):
        rowptr = np.zeros(self.n_dofs + 1, dtype=np.int64)
        col = np.zeros(self.nnz, dtype=np.int32)
        val = np.zeros(self.nnz)
        rhs = np.zeros(self.n_dofs)
        d2n = np.zeros(self.n_dofs, dtype=np.int32)
        self._ok(load().fgb_field_export_system(self.h, ptr(rowptr, i64p), ptr(col, ip), ptr(val), ptr(rhs),
                                                ptr(d2n, ip)))
        return rowptr, col, val, rhs, d2n

    def time_spmv(self, precision, reps=20):
        return load().fgb_field_time_spmv(self.h, precision, reps)


class Heat:
    """Current and heat on the bulk hexahedra of a mesh (CurrentHeatSolver verbs, Q1 on the GPU).

    Surface values are per copper-surface face, in the order of surface_faces()."""

    def __init__(self, mesh: Mesh):
        self.mesh = mesh
        self.h = load().fgb_heat_create(mesh.h)
        if not self.h:
            raise RuntimeError("heat solver creation failed: " + last_error())
        o = np.zeros(3, dtype=np.int64)
        self._ok(load().fgb_heat_sizes(self.h, ptr(o, i64p)))
        self.n_dofs, self.nnz, self.n_faces = (int(v) for v in o)

    def __del__(self):
        if getattr(self, "h", None):
            load().fgb_heat_free(self.h)
            self.h = None

    @staticmethod
    def _ok(rc):
        if rc != 0:
            raise RuntimeError(last_error())

    def surface_faces(self):
        """(centroids (n,3), (hex id, femocs local face) (n,2)) of the copper-surface faces"""
        c = np.zeros(max(3 * self.n_faces, 1))
        hf = np.zeros(max(2 * self.n_faces, 1), dtype=np.int32)
        self._ok(load().fgb_heat_surface_faces(self.h, ptr(c), ptr(hf, ip)))
        return c[: 3 * self.n_faces].reshape(-1, 3), hf[: 2 * self.n_faces].reshape(-1, 2)

    def set_resistivity(self, T, rho):
        T = np.ascontiguousarray(T, dtype=np.float64)
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        self._ok(load().fgb_heat_set_resistivity(self.h, len(T), ptr(T), ptr(rho)))

    def setup(self, t_ambient=300.0, lorentz=2.44e-8, rho_cp=3.4496e-24):
        self._ok(load().fgb_heat_setup(self.h, t_ambient, lorentz, rho_cp))

    def _solve(self, fn, args, precision, rel_tol, max_iter):
        st = np.zeros(14)
        rc = fn(self.h, *args, precision, rel_tol, max_iter, ptr(st))
        if rc == -2 ** 31:
            raise RuntimeError(last_error())
        return rc, _stats_dict(st)

    def solve_current(self, face_j, precision=0, rel_tol=1e-9, max_iter=100000):
        j = np.ascontiguousarray(face_j, dtype=np.float64)
        assert len(j) == self.n_faces
        return self._solve(load().fgb_heat_solve_current, (ptr(j),), precision, rel_tol, max_iter)

    def solve_heat(self, delta_time_s, face_q, precision=0, rel_tol=1e-9, max_iter=100000):
        q = np.ascontiguousarray(face_q, dtype=np.float64)
        assert len(q) == self.n_faces
        return self._solve(load().fgb_heat_solve_heat, (float(delta_time_s), ptr(q)), precision, rel_tol, max_iter)

    def nodes(self):
        """(temperature, current potential) per hex-mesh node; NaN outside the bulk"""
        n = self.mesh.sizes()["n_nodes"]
        T, p = np.zeros(n), np.zeros(n)
        self._ok(load().fgb_heat_export(self.h, ptr(T), ptr(p)))
        return T, p

    def temperature_range(self):
        o = np.zeros(2)
        self._ok(load().fgb_heat_temperature_range(self.h, ptr(o)))
        return float(o[0]), float(o[1])


class Femocs:
    """Mirror of the reference's C wrapper (create_femocs / femocs_run / femocs_interpolate_*)."""

    def __init__(self, conf_path: str):
        self.lib = load()
        self.h = self.lib.create_femocs(conf_path.encode())
        if not self.h:
            raise RuntimeError("create_femocs failed: " + last_error())

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.delete_femocs(self.h)
            self.h = None

    def run(self, timestep=-1, time=-1.0):
        rv = C.c_int(0)
        self.lib.femocs_run(self.h, C.byref(rv), timestep, time)
        return rv.value

    def import_mesh(self, xyz, tets, markers):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        tets = np.ascontiguousarray(tets, dtype=np.int32).reshape(-1)
        markers = np.ascontiguousarray(markers, dtype=np.int32).reshape(-1)
        rv = C.c_int(0)
        self.lib.femocs_import_mesh(self.h, C.byref(rv), len(xyz) // 3, ptr(xyz), len(tets) // 4, ptr(tets, ip),
                                    ptr(markers, ip))
        return rv.value

    def import_atoms(self, x, y, z, types):
        x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
        types = np.ascontiguousarray(types, dtype=np.int32)
        rv = C.c_int(0)
        self.lib.femocs_import_atoms(self.h, C.byref(rv), len(x), ptr(x), ptr(y), ptr(z), ptr(types, ip))
        return rv.value

    def interpolate_elfield(self, x, y, z):
        x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
        n = len(x)
        Ex, Ey, Ez, En = (np.zeros(n) for _ in range(4))
        flag = np.zeros(n, dtype=np.int32)
        rv = C.c_int(0)
        self.lib.femocs_interpolate_elfield(self.h, C.byref(rv), n, ptr(x), ptr(y), ptr(z), ptr(Ex), ptr(Ey), ptr(Ez),
                                            ptr(En), ptr(flag, ip))
        return rv.value, Ex, Ey, Ez, En, flag

    def interpolate_surface_elfield(self, x, y, z):
        x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
        n = len(x)
        Ex, Ey, Ez, En = (np.zeros(n) for _ in range(4))
        flag = np.zeros(n, dtype=np.int32)
        rv = C.c_int(0)
        self.lib.femocs_interpolate_surface_elfield(self.h, C.byref(rv), n, ptr(x), ptr(y), ptr(z), ptr(Ex), ptr(Ey),
                                                    ptr(Ez), ptr(En), ptr(flag, ip))
        return rv.value, Ex, Ey, Ez, En, flag

    def interpolate_phi(self, x, y, z):
        x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
        n = len(x)
        phi = np.zeros(n)
        flag = np.zeros(n, dtype=np.int32)
        rv = C.c_int(0)
        self.lib.femocs_interpolate_phi(self.h, C.byref(rv), n, ptr(x), ptr(y), ptr(z), ptr(phi), ptr(flag, ip))
        return rv.value, phi, flag

    def export_data(self, n, label):
        data = np.zeros(3 * n if label.lower() == "elfield" else n)
        rv = C.c_int(0)
        self.lib.femocs_export_data(self.h, C.byref(rv), ptr(data), n, label.encode())
        return rv.value, data

    def field(self, mesh_sizes):
        """Borrowed device field of this instance (valid after run())."""
        return Field.borrowed(self.lib.femocs_field(self.h), mesh_sizes)

    def last_solve(self):
        out = np.zeros(8)
        rv = C.c_int(0)
        self.lib.femocs_last_solve(self.h, C.byref(rv), ptr(out))
        return dict(iterations=int(out[0]), outer=int(out[1]), status=int(out[2]), rel_residual=out[3], ms=out[4],
                    n_dofs=int(out[5]), levels=int(out[7]))

    def last_stats(self):
        """All solver statistics of the last run (see Field.solve)."""
        st = np.zeros(14)
        if self.lib.fgb_femocs_last_stats(self.h, ptr(st)) != 0:
            raise RuntimeError(last_error())
        return _stats_dict(st)

    def enhancement(self):
        """M/A field-enhancement ratio of the last run's check (0 when it did not run)."""
        v = C.c_double(0)
        if self.lib.fgb_femocs_enhancement(self.h, C.byref(v)) != 0:
            raise RuntimeError(last_error())
        return v.value

    def parse_double(self, cmd):
        v = C.c_double(0)
        rv = C.c_int(0)
        self.lib.femocs_parse_double(self.h, C.byref(rv), cmd.encode(), C.byref(v))
        return rv.value, v.value


def device_info():
    """(free bytes, total bytes, UUID as nvidia-smi prints it) of the current device."""
    fr, tot = C.c_size_t(0), C.c_size_t(0)
    uuid = C.create_string_buffer(48)
    if load().fgb_device_info(C.byref(fr), C.byref(tot), uuid) != 0:
        raise RuntimeError(last_error())
    return fr.value, tot.value, uuid.value.decode()


class DeviceBuffer:
    """Plain device allocation (cudaMalloc) used by tests and the benchmark."""

    def __init__(self, nbytes):
        self.nbytes = int(nbytes)
        self.ptr = load().fgb_device_alloc(self.nbytes)
        if not self.ptr:
            raise MemoryError(last_error())

    def upload(self, a: np.ndarray):
        a = np.ascontiguousarray(a)
        assert a.nbytes <= self.nbytes
        if load().fgb_memcpy_htod(self.ptr, a.ctypes.data_as(C.c_void_p), a.nbytes) != 0:
            raise RuntimeError(last_error())

    def download(self, a: np.ndarray):
        assert a.flags.c_contiguous and a.nbytes <= self.nbytes
        if load().fgb_memcpy_dtoh(a.ctypes.data_as(C.c_void_p), self.ptr, a.nbytes) != 0:
            raise RuntimeError(last_error())
        return a

    def __del__(self):
        if getattr(self, "ptr", None):
            load().fgb_device_free(self.ptr)
            self.ptr = None


def synth_atoms(spec_kw, latconst=3.615, sigma=0.05, cutoff=3.1, seed=12345):
    spec = nanotip(**spec_kw)
    lib = load()
    n = lib.fgb_synth_atoms(C.byref(spec), latconst, sigma, cutoff, seed, None, None)
    if n < 0:
        raise RuntimeError(last_error())
    xyz = np.zeros(3 * n)
    types = np.zeros(n, dtype=np.int32)
    lib.fgb_synth_atoms(C.byref(spec), latconst, sigma, cutoff, seed, ptr(xyz), ptr(types, ip))
    return xyz.reshape(-1, 3), types


def synth_probes(spec_kw, n, seed=777):
    spec = nanotip(**spec_kw)
    xyz = np.zeros(3 * n)
    if load().fgb_synth_probes(C.byref(spec), n, seed, ptr(xyz)) < 0:
        raise RuntimeError(last_error())
    return xyz.reshape(-1, 3)


class Batch:
    """Many meshes resident on the device, solved together (block-diagonal multigrid PCG,
    one CUDA graph launch per step). Solves: admit(slot, E0, ...) then step()/collect(), or
    solve_all(). Each slot keeps its last solution as the warm start of its next solve."""

    def __init__(self, use_graph=True, autotune=True, grid_ctas=0, persistent=False):
        mode = 2 if persistent else int(bool(use_graph))
        self.h = load().fgb_batch_create(mode, int(autotune), int(grid_ctas))
        if not self.h:
            raise RuntimeError("batch creation failed: " + last_error())
        self._meshes = {}

    def __del__(self):
        if getattr(self, "h", None):
            load().fgb_batch_free(self.h)
            self.h = None

    def _ok(self, rc):
        if rc != 0:
            raise RuntimeError(last_error())

    def add_mesh(self, mesh: Mesh, hbm_reserve=0.0):
        """Slot of the placed mesh, or -1 when free device memory does not admit it."""
        slot = load().fgb_batch_add_mesh(self.h, mesh.h, float(hbm_reserve))
        if slot == -(2 ** 31):
            raise RuntimeError(last_error())
        if slot >= 0:
            self._meshes[slot] = mesh
        return slot

    def add_synthetic(self, specs, n_threads=0, hbm_reserve=0.0):
        """Build and add nanotip meshes from spec dicts on host threads; returns the slots."""
        arr = (FgbNanotip * len(specs))(*[nanotip(**s) for s in specs])
        slots = np.full(len(specs), -1, dtype=np.int32)
        self._ok(load().fgb_batch_add_synthetic(self.h, len(specs), arr, int(n_threads), float(hbm_reserve),
                                                ptr(slots, ip)))
        return slots

    def remove_mesh(self, slot):
        self._ok(load().fgb_batch_remove_mesh(self.h, slot))
        self._meshes.pop(slot, None)

    def admit(self, slot, E0, rel_tol=1e-9, max_iter=1000):
        self._ok(load().fgb_batch_admit(self.h, slot, float(E0), float(rel_tol), int(max_iter)))

    def step(self, max_iters=1000):
        still = load().fgb_batch_step(self.h, int(max_iters))
        if still == -(2 ** 31):
            raise RuntimeError(last_error())
        return still

    def collect(self, cap=4096):
        slots = np.zeros(cap, dtype=np.int32)
        res = np.zeros(4 * cap)
        n = load().fgb_batch_collect(self.h, cap, ptr(slots, ip), ptr(res))
        if n == -(2 ** 31):
            raise RuntimeError(last_error())
        return {int(slots[k]): dict(iterations=int(res[4 * k]), status=int(res[4 * k + 1]),
                                    rel_residual=res[4 * k + 2], bnorm=res[4 * k + 3]) for k in range(n)}

    def solve_all(self, fields, rel_tol=1e-9, max_iter=1000):
        """fields: {slot: E0}. Admits all, steps until all finish; returns {slot: result}."""
        for slot, E0 in fields.items():
            self.admit(slot, E0, rel_tol, max_iter)
        out = {}
        while True:
            still = self.step(max_iter + 1)
            out.update(self.collect())
            if still == 0:
                break
        return out

    def extract(self, slot, smoothen=True):
        self._ok(load().fgb_batch_extract(self.h, slot, int(smoothen)))

    def interpolate_device(self, slot, n, d_xyz, rank, d_cells, d_out5):
        self._ok(load().fgb_batch_interpolate(self.h, slot, int(n), C.c_void_p(d_xyz), int(rank), C.c_void_p(d_cells),
                                              C.c_void_p(d_out5)))

    def sync(self, slot):
        self._ok(load().fgb_batch_sync_slot(self.h, slot))

    def info(self, slot):
        o = np.zeros(4, dtype=np.int64)
        self._ok(load().fgb_batch_info(self.h, slot, ptr(o, i64p)))
        return dict(n_dofs=int(o[0]), n_nodes=int(o[1]), levels=int(o[2]))

    def phi_nodes(self, slot):
        out = np.zeros(self.info(slot)["n_nodes"])
        self._ok(load().fgb_batch_export_phi_nodes(self.h, slot, ptr(out)))
        return out

    def nodal(self, slot):
        out = np.zeros(5 * self.info(slot)["n_nodes"])
        self._ok(load().fgb_batch_export_nodal(self.h, slot, ptr(out)))
        return out.reshape(-1, 5)

    def reset_solution(self, slot):
        self._ok(load().fgb_batch_reset_solution(self.h, slot))

    def true_residual(self, slot):
        v = C.c_double(0)
        self._ok(load().fgb_batch_true_residual(self.h, slot, C.byref(v)))
        return v.value

    def stats(self):
        o = np.zeros(6)
        self._ok(load().fgb_batch_stats(self.h, ptr(o)))
        return dict(total_dofs=int(o[0]), device_bytes=int(o[1]), last_iterations=int(o[2]),
                    kernels_per_iteration=int(o[3]), graph_launches=int(o[4]), slots=int(o[5]))

    def tuning(self):
        buf = C.create_string_buffer(1024)
        self._ok(load().fgb_batch_tuning(self.h, buf, 1024))
        return buf.value.decode()

    def mark(self, k):
        self._ok(load().fgb_batch_mark(self.h, int(k)))

    def elapsed(self, k0, k1):
        ms = load().fgb_batch_elapsed(self.h, int(k0), int(k1))
        if ms < 0:
            raise RuntimeError(last_error())
        return ms


def nanotip_vacuum_hexes(spec_kw):
    """Vacuum hexahedra of the synthetic nanotip mesh of this spec (no mesh is built)."""
    n = load().fgb_nanotip_vacuum_hexes(C.byref(nanotip(**spec_kw)))
    if n < 0:
        raise RuntimeError(last_error())
    return int(n)


def batch_specs(n, seed=2024, lo_hexes=2e4, hi_hexes=8e5, n_threads=0):
    """Nanotip specs of a batch of independent tips: tip radius uniform 1-6 nm, aspect ratio
    (height / radius) uniform 2-8, applied field uniform 0.5-3 GV/m, vacuum hex count
    log-uniform in [lo_hexes, hi_hexes] (the core spacing is fitted to it). Slab half width
    6 radii, slab thickness max(2 nm, radius), vacuum top 6 tip heights above the slab.
    Returns (specs, fields in V/A)."""
    rng = np.random.default_rng(seed)
    specs, fields = [], []
    for _ in range(n):
        r = rng.uniform(10.0, 60.0)
        hgt = r * rng.uniform(2.0, 8.0)
        target = float(np.exp(rng.uniform(np.log(lo_hexes), np.log(hi_hexes))))
        s = dict(radius=r, height=hgt, box_half=6.0 * r, slab=max(20.0, r), top=6.0 * hgt + 2.0 * r,
                 h=r / 4, growth=1.25, margin=0.5 * r)
        h = load().fgb_nanotip_fit_spacing(C.byref(nanotip(**s)), target)
        if h <= 0:
            raise RuntimeError(last_error())
        s["h"] = h
        specs.append(s)
        fields.append(rng.uniform(0.05, 0.3))
    return specs, np.array(fields)


class Server:
    """Serving loop over a Batch: MD runs with resident meshes and atoms submit field solves
    (Gaussian atom step on the device, warm-started solve, nodal field, interpolation at the
    atoms); a scheduler thread batches them continuously."""

    def __init__(self, batch: Batch, rel_tol=1e-9, max_iter=500, iters_per_launch=4, rank=1, smoothen=True,
                 hbm_reserve=2e9):
        self.batch = batch
        self.h = load().fgb_server_create(batch.h, float(rel_tol), int(max_iter), int(iters_per_launch), int(rank),
                                          int(smoothen), float(hbm_reserve))
        if not self.h:
            raise RuntimeError("server creation failed: " + last_error())
        self._meshes = []

    def __del__(self):
        if getattr(self, "h", None):
            load().fgb_server_free(self.h)
            self.h = None

    def _ok(self, rc):
        if rc != 0:
            raise RuntimeError(last_error())

    def set_launch_policy(self, idle_iters=0, stop_at_first=False):
        """Before start(): iterations per launch while no request waits (0: iters_per_launch),
        and whether a launch ends after the iteration in which one of its solves finished."""
        self._ok(load().fgb_server_set_launch_policy(self.h, int(idle_iters), int(bool(stop_at_first))))

    def add_run(self, mesh: Mesh, xyz, seed=1):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        rid = load().fgb_server_add_run(self.h, mesh.h, ptr(xyz), len(xyz) // 3, int(seed))
        if rid == -(2 ** 31):
            raise RuntimeError(last_error())
        self._meshes.append(mesh)
        return rid

    def add_synthetic_runs(self, specs, n_atoms, seed=1, n_threads=0):
        arr = (FgbNanotip * len(specs))(*[nanotip(**s) for s in specs])
        self._ok(load().fgb_server_add_synthetic_runs(self.h, len(specs), arr, int(n_atoms), int(seed), int(n_threads)))

    def place_pending(self, n_threads=0):
        n = load().fgb_server_place_pending(self.h, int(n_threads))
        if n == -(2 ** 31):
            raise RuntimeError(last_error())
        return n

    def submit(self, run, E0, sigma=0.02):
        rid = load().fgb_server_submit(self.h, int(run), float(E0), float(sigma))
        if rid < 0:
            raise RuntimeError(last_error())
        return rid

    def start(self):
        self._ok(load().fgb_server_start(self.h))

    def stop(self):
        self._ok(load().fgb_server_stop(self.h))

    def drain(self, timeout=600.0):
        rc = load().fgb_server_drain(self.h, float(timeout))
        if rc < 0:
            raise RuntimeError(last_error())
        return rc == 0

    def run_poisson(self, rate, n, base_fields, sigma=0.02, seed=7):
        bf = np.ascontiguousarray(base_fields, dtype=np.float64)
        self._ok(load().fgb_server_run_poisson(self.h, float(rate), int(n), float(sigma), int(seed), ptr(bf)))

    def records(self, cap=1 << 20):
        out = np.zeros(10 * cap)
        n = load().fgb_server_records(self.h, cap, ptr(out))
        if n == -(2 ** 31):
            raise RuntimeError(last_error())
        a = out[:10 * n].reshape(-1, 10)
        keys = ["id", "run", "E0", "iterations", "status", "rel_residual", "t_submit", "t_admit", "t_solved", "t_done"]
        return {k: a[:, i] for i, k in enumerate(keys)}

    def clear_records(self):
        self._ok(load().fgb_server_clear_records(self.h))

    def run_info(self, run):
        o = np.zeros(2, dtype=np.int64)
        self._ok(load().fgb_server_run_info(self.h, int(run), ptr(o, i64p)))
        return dict(slot=int(o[0]), n_atoms=int(o[1]))

    def last_result(self, run):
        n = self.run_info(run)["n_atoms"]
        out = np.zeros(5 * n)
        cells = np.zeros(n, dtype=np.int32)
        self._ok(load().fgb_server_last_result(self.h, int(run), ptr(out), ptr(cells, ip)))
        return cells, out.reshape(-1, 5)

    def reset_run(self, run):
        self._ok(load().fgb_server_reset_run(self.h, int(run)))

    def info(self):
        o = np.zeros(4)
        self._ok(load().fgb_server_info(self.h, ptr(o)))
        return dict(runs=int(o[0]), solver_launches=int(o[1]), max_in_flight=int(o[2]))
