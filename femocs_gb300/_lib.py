"""ctypes binding of libfemocs_gb300.so (the C ABI declared in include/femocs_gb300.h).

The library is built in-tree by femocs_gb300.build; loading fails loudly when it is missing
-- there is no CPU fallback for the field path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfemocs_gb300.so")

_lib = None

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)
i64p = C.POINTER(C.c_int64)
vp = C.c_void_p


class FgbNanotip(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("radius", "height", "box_half", "slab", "top", "h", "growth", "margin")]


_PROTOS = {
    # Part 1
    "create_femocs": (vp, [C.c_char_p]),
    "delete_femocs": (None, [vp]),
    "femocs_run": (None, [vp, ip, C.c_int, C.c_double]),
    "femocs_import_file": (None, [vp, ip, C.c_char_p]),
    "femocs_import_parcas": (None, [vp, ip, C.c_int, dp, dp, dp, ip]),
    "femocs_import_atoms": (None, [vp, ip, C.c_int, dp, dp, dp, ip]),
    "femocs_import_mesh": (None, [vp, ip, C.c_int, dp, C.c_int, ip, ip]),
    "femocs_interpolate_elfield": (None, [vp, ip, C.c_int, dp, dp, dp, dp, dp, dp, dp, ip]),
    "femocs_interpolate_surface_elfield": (None, [vp, ip, C.c_int, dp, dp, dp, dp, dp, dp, dp, ip]),
    "femocs_interpolate_phi": (None, [vp, ip, C.c_int, dp, dp, dp, dp, ip]),
    "femocs_export_data": (None, [vp, ip, dp, C.c_int, C.c_char_p]),
    "femocs_export_int": (None, [vp, ip, ip, C.c_int, C.c_char_p]),
    "femocs_interpolate": (None, [vp, ip, dp, ip, C.c_int, C.c_char_p, C.c_int, dp, dp, dp]),
    "femocs_parse_int": (None, [vp, ip, C.c_char_p, ip]),
    "femocs_parse_double": (None, [vp, ip, C.c_char_p, dp]),
    "femocs_parse_string": (None, [vp, ip, C.c_char_p, C.c_char_p]),
    "femocs_last_solve": (None, [vp, ip, dp]),
    "fgb_femocs_last_stats": (C.c_int, [vp, dp]),
    "fgb_femocs_enhancement": (C.c_int, [vp, dp]),
    "femocs_last_error": (C.c_char_p, []),
    "fgb_kernel_launches": (C.c_longlong, []),
    # Part 2
    "fgb_mesh_from_arrays": (vp, [C.c_int, dp, C.c_int, ip, ip]),
    "fgb_mesh_read_gmsh": (vp, [C.c_char_p]),
    "fgb_mesh_synthetic": (vp, [C.POINTER(FgbNanotip)]),
    "fgb_mesh_from_arrays_device": (vp, [C.c_int, dp, C.c_int, ip, ip]),
    "fgb_mesh_synthetic_device": (vp, [C.POINTER(FgbNanotip)]),
    "fgb_mesh_prep_timing": (C.c_int, [vp, dp]),
    "fgb_mesh_set_surface": (C.c_int, [vp, C.c_int, ip, ip]),
    "fgb_mesh_surface_tris": (C.c_int64, [vp]),
    "fgb_mesh_free": (None, [vp]),
    "fgb_heat_create": (vp, [vp]),
    "fgb_heat_free": (None, [vp]),
    "fgb_heat_sizes": (C.c_int, [vp, i64p]),
    "fgb_heat_surface_faces": (C.c_int, [vp, dp, ip]),
    "fgb_heat_set_resistivity": (C.c_int, [vp, C.c_int, dp, dp]),
    "fgb_heat_setup": (C.c_int, [vp, C.c_double, C.c_double, C.c_double]),
    "fgb_heat_solve_current": (C.c_int, [vp, dp, C.c_int, C.c_double, C.c_int, dp]),
    "fgb_heat_solve_heat": (C.c_int, [vp, C.c_double, dp, C.c_int, C.c_double, C.c_int, dp]),
    "fgb_heat_export": (C.c_int, [vp, dp, dp]),
    "fgb_heat_temperature_range": (C.c_int, [vp, dp]),
    "fgb_mesh_sizes": (C.c_int, [vp, i64p]),
    "fgb_mesh_export": (C.c_int, [vp, C.c_char_p, vp]),
    "fgb_synth_atoms": (C.c_int64, [C.POINTER(FgbNanotip), C.c_double, C.c_double, C.c_double, C.c_uint64, dp, ip]),
    "fgb_synth_probes": (C.c_int64, [C.POINTER(FgbNanotip), C.c_int, C.c_uint64, dp]),
    "fgb_field_create": (vp, [vp]),
    "fgb_field_create_order": (vp, [vp, C.c_int]),
    "fgb_field_q2_dofs": (C.c_int, [vp, ip, ip]),
    "fgb_field_export_solution": (C.c_int, [vp, dp]),
    "fgb_field_space_charge": (C.c_int, [vp, C.c_int, vp, vp, C.c_double, C.c_int, ip]),
    "fgb_field_clear_space_charge": (C.c_int, [vp]),
    "fgb_device_sync": (C.c_int, []),
    "fgb_device_info": (C.c_int, [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), C.c_char_p]),
    "fgb_tc_selftest": (C.c_int, [dp]),
    "fgb_mesh_q2_sizes": (C.c_int, [vp, i64p]),
    "fgb_mesh_cell_blocks": (C.c_int, [vp, C.c_int, C.c_int, i64p]),
    "fgb_mesh_q1_sizes": (C.c_int, [vp, i64p]),
    "fgb_mesh_structure_digest": (C.c_uint64, [vp, C.c_int, C.c_int]),
    "fgb_field_free": (None, [vp]),
    "fgb_field_sizes": (C.c_int, [vp, i64p]),
    "fgb_field_setup": (C.c_int, [vp, C.c_double, C.c_double]),
    "fgb_field_assemble": (C.c_int, [vp, C.c_int, C.c_int]),
    "fgb_field_solve": (C.c_int, [vp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double, dp]),
    "fgb_field_last_stats": (C.c_int, [vp, dp]),
    "fgb_field_set_profiling": (C.c_int, [vp, C.c_int]),
    "fgb_field_set_coarse_cycles": (C.c_int, [vp, C.c_int, C.c_int]),
    "fgb_field_set_level0_stream": (C.c_int, [vp, C.c_int]),
    "fgb_field_set_level0_prefetch": (C.c_int, [vp, C.c_int]),
    "fgb_field_set_level0_operator": (C.c_int, [vp, C.c_int]),
    "fgb_field_set_ke_tensor": (C.c_int, [vp, C.c_int]),
    "fgb_field_export_element_matrices": (C.c_longlong, [vp, dp]),
    "fgb_field_set_smoothing": (C.c_int, [vp, C.c_int, C.c_double]),
    "fgb_field_set_level_smoothing": (C.c_int, [vp, C.c_int, C.c_int, C.c_double]),
    "fgb_field_set_lazy_matrix": (C.c_int, [vp, C.c_int]),
    "fgb_field_set_level0_ebe": (C.c_int, [vp, C.c_int]),
    "fgb_field_set_outer_spmv": (C.c_int, [vp, C.c_int]),
    "fgb_field_outer_spmv_bytes": (C.c_double, [vp]),
    "fgb_field_set_cell_blocks": (C.c_int, [vp, C.c_int, C.c_int]),
    "fgb_field_amg_levels": (C.c_int, [vp, C.c_char_p, C.c_int]),
    "fgb_field_export_phi_nodes": (C.c_int, [vp, dp]),
    "fgb_field_import_phi_nodes": (C.c_int, [vp, dp]),
    "fgb_field_extract": (C.c_int, [vp, C.c_int]),
    "fgb_field_get_nodal": (C.c_int, [vp, dp]),
    "fgb_field_set_nodal": (C.c_int, [vp, dp]),
    "fgb_field_interpolate": (C.c_int, [vp, C.c_int, dp, C.c_int, ip, dp, i64p]),
    "fgb_field_interpolate_device": (C.c_int, [vp, C.c_int, vp, C.c_int, vp, vp]),
    "fgb_field_interpolate_surface": (C.c_int, [vp, C.c_int, dp, C.c_int, ip, dp]),
    "fgb_field_interpolate_surface_device": (C.c_int, [vp, C.c_int, vp, C.c_int, vp, vp]),
    "fgb_field_interpolate_device_noalloc": (C.c_int, [vp, C.c_int, vp, C.c_int, vp, vp]),
    "fgb_field_export_system": (C.c_int, [vp, i64p, ip, dp, dp, ip]),
    "fgb_field_time_spmv": (C.c_double, [vp, C.c_int, C.c_int]),
    "fgb_field_stream": (vp, [vp]),
    "femocs_field": (vp, [vp]),
    "fgb_field_mark": (C.c_int, [vp, C.c_int]),
    "fgb_field_elapsed": (C.c_double, [vp, C.c_int, C.c_int]),
    "fgb_device_alloc": (vp, [C.c_size_t]),
    "fgb_device_free": (None, [vp]),
    "fgb_memcpy_htod": (C.c_int, [vp, vp, C.c_size_t]),
    "fgb_memcpy_dtoh": (C.c_int, [vp, vp, C.c_size_t]),
    "fgb_nanotip_vacuum_hexes": (C.c_longlong, [C.POINTER(FgbNanotip)]),
    "fgb_nanotip_fit_spacing": (C.c_double, [C.POINTER(FgbNanotip), C.c_double]),
    # Part 3: batches
    "fgb_batch_create": (vp, [C.c_int, C.c_int, C.c_int]),
    "fgb_batch_free": (None, [vp]),
    "fgb_batch_add_mesh": (C.c_int, [vp, vp, C.c_double]),
    "fgb_batch_add_synthetic": (C.c_int, [vp, C.c_int, C.POINTER(FgbNanotip), C.c_int, C.c_double, ip]),
    "fgb_batch_remove_mesh": (C.c_int, [vp, C.c_int]),
    "fgb_batch_admit": (C.c_int, [vp, C.c_int, C.c_double, C.c_double, C.c_int]),
    "fgb_batch_step": (C.c_int, [vp, C.c_int]),
    "fgb_batch_collect": (C.c_int, [vp, C.c_int, ip, dp]),
    "fgb_batch_extract": (C.c_int, [vp, C.c_int, C.c_int]),
    "fgb_batch_interpolate": (C.c_int, [vp, C.c_int, C.c_int, vp, C.c_int, vp, vp]),
    "fgb_batch_sync_slot": (C.c_int, [vp, C.c_int]),
    "fgb_batch_export_phi_nodes": (C.c_int, [vp, C.c_int, dp]),
    "fgb_batch_export_nodal": (C.c_int, [vp, C.c_int, dp]),
    "fgb_batch_reset_solution": (C.c_int, [vp, C.c_int]),
    "fgb_batch_true_residual": (C.c_int, [vp, C.c_int, dp]),
    "fgb_batch_info": (C.c_int, [vp, C.c_int, i64p]),
    "fgb_batch_stats": (C.c_int, [vp, dp]),
    "fgb_batch_tuning": (C.c_int, [vp, C.c_char_p, C.c_int]),
    "fgb_batch_mark": (C.c_int, [vp, C.c_int]),
    "fgb_batch_elapsed": (C.c_double, [vp, C.c_int, C.c_int]),
    # Part 4: serving
    "fgb_server_create": (vp, [vp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double]),
    "fgb_server_free": (None, [vp]),
    "fgb_server_set_launch_policy": (C.c_int, [vp, C.c_int, C.c_int]),
    "fgb_server_add_run": (C.c_int, [vp, vp, dp, C.c_int, C.c_ulonglong]),
    "fgb_server_add_synthetic_runs": (C.c_int, [vp, C.c_int, C.POINTER(FgbNanotip), C.c_int, C.c_ulonglong, C.c_int]),
    "fgb_server_place_pending": (C.c_int, [vp, C.c_int]),
    "fgb_server_submit": (C.c_longlong, [vp, C.c_int, C.c_double, C.c_double]),
    "fgb_server_start": (C.c_int, [vp]),
    "fgb_server_stop": (C.c_int, [vp]),
    "fgb_server_drain": (C.c_int, [vp, C.c_double]),
    "fgb_server_run_poisson": (C.c_int, [vp, C.c_double, C.c_int, C.c_double, C.c_ulonglong, dp]),
    "fgb_server_records": (C.c_int, [vp, C.c_int, dp]),
    "fgb_server_clear_records": (C.c_int, [vp]),
    "fgb_server_last_result": (C.c_int, [vp, C.c_int, dp, ip]),
    "fgb_server_reset_run": (C.c_int, [vp, C.c_int]),
    "fgb_server_info": (C.c_int, [vp, dp]),
    "fgb_server_run_info": (C.c_int, [vp, C.c_int, i64p]),
}


def exported_symbols():
    return list(_PROTOS)


def load():
    """Load the shared library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run femocs_gb300.build.build() first "
                           "(the field path has no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in _PROTOS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    e = load().femocs_last_error()
    return e.decode() if e else ""


def ptr(a: np.ndarray, kind=dp):
    return a.ctypes.data_as(kind)
