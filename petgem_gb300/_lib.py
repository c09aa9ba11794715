"""ctypes binding of the C ABI declared in ``include/petgem_gb300.h``.

The shared library is the only implementation: if it is missing or fails to
load, every entry point raises; there is no CPU fallback.
"""
import ctypes
import os
import threading

from . import _build

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_INT = ctypes.c_int
_SZ = ctypes.c_size_t
_D = ctypes.c_double


class GmresOpts(ctypes.Structure):
    """pg_gmres_opts (include/petgem_gb300.h)."""
    _fields_ = [("restart", ctypes.c_int), ("max_it", ctypes.c_int), ("rtol", ctypes.c_double),
                ("precision", ctypes.c_int), ("reorth", ctypes.c_int), ("block_p", ctypes.c_int),
                ("block_edges", ctypes.c_int64), ("block_faces", ctypes.c_int64), ("block_volumes", ctypes.c_int64),
                ("grad_cols", ctypes.c_int64), ("grad_rowptr", ctypes.c_void_p), ("grad_col", ctypes.c_void_p),
                ("grad_val", ctypes.c_void_p), ("gradt_rowptr", ctypes.c_void_p), ("gradt_row", ctypes.c_void_p),
                ("gradt_val", ctypes.c_void_p)]


class GmresResult(ctypes.Structure):
    """pg_gmres_result (include/petgem_gb300.h)."""
    _fields_ = [("iterations", ctypes.c_int64), ("restarts", ctypes.c_int64), ("relres", ctypes.c_double),
                ("status", ctypes.c_int)]


class CocgOpts(ctypes.Structure):
    """pg_cocg_opts (include/petgem_gb300.h)."""
    _fields_ = [("max_it", ctypes.c_int), ("rtol", ctypes.c_double), ("precision", ctypes.c_int),
                ("check_every", ctypes.c_int), ("block_p", ctypes.c_int), ("block_edges", ctypes.c_int64),
                ("block_faces", ctypes.c_int64), ("block_volumes", ctypes.c_int64), ("inner_rtol", ctypes.c_double),
                ("grad_cols", ctypes.c_int64), ("grad_rowptr", ctypes.c_void_p), ("grad_col", ctypes.c_void_p),
                ("grad_val", ctypes.c_void_p), ("gradt_rowptr", ctypes.c_void_p), ("gradt_row", ctypes.c_void_p),
                ("gradt_val", ctypes.c_void_p)]


_PO = ctypes.POINTER(GmresOpts)
_PC = ctypes.POINTER(CocgOpts)
_PR = ctypes.POINTER(GmresResult)

# name -> (restype, argtypes); mirrors include/petgem_gb300.h
SIGNATURES = {
    "pg_abi_version": (_INT, []),
    "pg_last_error": (ctypes.c_char_p, []),
    "pg_fp64_probe": (_INT, [_P, _INT, _INT, _P]),
    "pg_fp64_probe_flops": (_I64, [_INT, _INT]),
    "pg_copy_bytes": (_INT, [_P, _P, _I64, _INT, _P]),
    "pg_table_doubles": (_I64, [_INT]),
    "pg_tuples_workspace_bytes": (_SZ, [_I64]),
    "pg_orientation_tuples": (_INT, [_P, _P, _I64, _P, _P, _P, _P, _SZ, _P]),
    "pg_tuple_tables": (_INT, [_P, _I64, _INT, _P, _P]),
    "pg_elemental_matrices": (_INT, [_P, _P, _P, _P, _P, _I64, _INT, _P, _P, _P, _P]),
    "pg_topology_workspace_bytes": (_SZ, [_I64]),
    "pg_topology": (_INT, [_P, _I64, _I64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "pg_connectivity_dofs": (_INT, [_P, _P, _I64, _I64, _I64, _INT, _P, _P]),
    "pg_element_orientation": (_INT, [_P, _P, _P, _P, _P, _I64, _P, _P, _P]),
    "pg_boundary_workspace_bytes": (_SZ, [_I64, _I64]),
    "pg_boundary_dofs": (_INT, [_P, _P, _I64, _I64, _INT, _P, _P, _P, _SZ, _P]),
    "pg_faces_edges": (_INT, [_P, _P, _I64, _I64, _P, _P, _P, _P]),
    "pg_face_counts": (_INT, [_P, _I64, _I64, _P, _P]),
    "pg_flag_edges_of_pairs": (_INT, [_P, _I64, _P, _I64, _P, _P]),
    "pg_select_workspace_bytes": (_SZ, [_I64]),
    "pg_select_equal": (_INT, [_P, _I64, _INT, _P, _P, _P, _SZ, _P]),
    "pg_select_equal_noalloc_max_n": (_I64, []),
    "pg_select_equal_noalloc": (_INT, [_P, _I64, _INT, _P, _P, _P]),
    "pg_pattern_local_entities": (_INT, [_INT]),
    "pg_pattern_workspace_bytes": (_SZ, [_I64, _I64, _I64, _INT]),
    "pg_pattern_build": (_INT, [_P, _P, _I64, _I64, _I64, _INT, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "pg_pattern_columns": (_INT, [_P, _P, _P, _I64, _P, _P, _I64, _I64, _I64, _INT, _P, _P, _P]),
    "pg_assemble_values": (_INT, [_P, _P, _P, _P, _P, _I64, _P, _P, _I64, _I64, _I64, _INT, _P, _D, _P, _P]),
    "pg_element_coefficients": (_INT, [_P, _P, _P, _I64, _D, _P, _P, _P]),
    "pg_element_coefficients_df": (_INT, [_P, _P, _P, _I64, _D, _P, _P, _P]),
    "pg_pattern_items_workspace_bytes": (_SZ, [_I64, _I64]),
    "pg_pattern_items": (_INT, [_P, _P, _I64, _P, _P, _I64, _I64, _I64, _INT, _I64, _P, _P, _P, _P, _SZ, _P]),
    "pg_assemble_fused": (_INT, [_P, _P, _P, _P, _P, _P, _P, _P, _I64, _I64, _P, _P, _I64, _I64, _I64, _INT, _P, _P,
                                 _P]),
    "pg_apply_pec": (_INT, [_P, _P, _P, _I64, _P, _I64, _P, _P, _P]),
    "pg_assemble_fused_ex": (_INT, [_P, _P, _P, _P, _P, _P, _P, _P, _I64, _I64, _P, _P, _I64, _I64, _I64, _INT, _P, _P,
                                    _INT, _P, _P]),
    "pg_to_double_float": (_INT, [_P, _I64, _P, _P]),
    "pg_assembly_record_bytes": (_I64, [_I64]),
    "pg_assembly_records": (_INT, [_P, _P, _P, _P, _P, _I64, _P, _P, _I64, _I64, _I64, _INT, _P, _I64, _P, _P, _P, _P]),
    "pg_tuple_tables_entry_major": (_INT, [_P, _I64, _INT, _INT, _P, _P]),
    "pg_assemble_records": (_INT, [_P, _P, _P, _P, _P, _I64, _I64, _INT, _INT, _INT, _P, _P]),
    "pg_pec_flags": (_INT, [_P, _I64, _I64, _P, _P]),
    "pg_pec_rhs": (_INT, [_P, _I64, _INT, _P, _P]),
    "pg_locate_points": (_INT, [_P, _P, _I64, _P, _I64, _D, _P, _P]),
    "pg_source_rhs": (_INT, [_P, _P, _P, _P, _P, _INT, _P, _P, _P, _D, _D, _P, _P, _P]),
    "pg_gather_fields": (_INT, [_P, _P, _P, _P, _P, _P, _INT, _P, _P, _I64, _D, _P, _P]),
    "pg_boundary_faces_workspace_bytes": (_SZ, [_I64]),
    "pg_boundary_faces": (_INT, [_P, _P, _I64, _I64, _P, _P, _P, _P, _P, _SZ, _P]),
    "pg_face_planes": (_INT, [_P, _P, _P, _P, _P, _P, _I64, _P, _P, _P, _P, _P]),
    "pg_mt_face_z": (_INT, [_P, _P, _P, _P, _I64, _P, _INT, _P, _P]),
    "pg_mt_plan_workspace_bytes": (_SZ, [_I64, _INT]),
    "pg_mt_plan": (_INT, [_P, _P, _I64, _INT, _I64, _P, _P, _P, _P, _P, _SZ, _P]),
    "pg_mt_rhs_workspace_bytes": (_SZ, [_I64, _INT]),
    "pg_mt_rhs": (_INT, [_P, _P, _P, _P, _INT, _P, _P, _P, _I64, _P, _INT, _P, _INT, _D, _D, _P, _P, _P, _I64, _P, _INT,
                         _INT, _P, _SZ, _P]),
    "pg_node_fields_workspace_bytes": (_SZ, [_I64, _I64]),
    "pg_node_fields": (_INT, [_P, _P, _P, _P, _P, _P, _INT, _I64, _I64, _D, _P, _P, _SZ, _P]),
    "pg_receiver_adjoint_workspace_bytes": (_SZ, [_INT, _I64]),
    "pg_receiver_adjoint": (_INT, [_P, _P, _P, _P, _P, _INT, _P, _P, _I64, _P, _P, _P, _SZ, _P]),
    "pg_element_mass_bilinear": (_INT, [_P, _P, _P, _P, _P, _P, _I64, _INT, _P, _P]),
    "pg_spmv_z": (_INT, [_P, _P, _P, _I64, _P, _P, _INT, _P]),
    "pg_spmv_c": (_INT, [_P, _P, _P, _I64, _P, _P, _INT, _P]),
    "pg_gmres_default_opts": (None, [_PO]),
    "pg_gmres_workspace_bytes": (_SZ, [_I64, _I64, _INT, _PO]),
    "pg_gmres": (_INT, [_P, _P, _P, _I64, _I64, _P, _P, _INT, _PO, _PR, _P, _P, _SZ, _P]),
    "pg_gradient_map_sizes": (_INT, [_I64, _I64, _I64, _I64, _INT, _INT, _P, _P]),
    "pg_gradient_map_workspace_bytes": (_SZ, [_I64, _I64, _I64, _I64, _I64, _INT, _INT]),
    "pg_gradient_map": (_INT, [_P, _P, _P, _P, _P, _P, _P, _I64, _I64, _I64, _I64, _I64, _INT, _INT, _P, _P, _P, _P,
                               _P, _P, _P, _P, _SZ, _P]),
    "pg_cocg_default_opts": (None, [_PC]),
    "pg_cocg_workspace_bytes": (_SZ, [_I64, _I64, _INT, _PC]),
    "pg_cocg": (_INT, [_P, _P, _P, _I64, _I64, _P, _P, _INT, _PC, _PR, _P, _P, _SZ, _P]),
    "pg_cocg_multifreq_workspace_bytes": (_SZ, [_I64, _I64, _INT, _PC]),
    "pg_cocg_multifreq": (_INT, [_P, _P, _P, _I64, _I64, _P, _P, _INT, _P, _PC, _PR, _P, _P, _SZ, _P]),
    "pg_cocg_segments_workspace_bytes": (_SZ, [_I64, _I64, _INT, _P, _INT, _P, _PC]),
    "pg_cocg_segments": (_INT, [_P, _P, _P, _I64, _I64, _P, _INT, _P, _P, _P, _INT, _PC, _PR, _P, _P, _P, _SZ, _P]),
    "pg_segments_block_map": (_INT, [_P, _INT, _INT, _P, _P]),
}

STATUS = {
    0: "PG_OK", -1: "PG_ERR_ARG", -2: "PG_ERR_CUDA", -3: "PG_ERR_WORKSPACE", -4: "PG_ERR_UNSUPPORTED",
    -5: "PG_ERR_DEGENERATE", -6: "PG_ERR_NOT_FOUND", -7: "PG_ERR_NOT_CONVERGED", -8: "PG_ERR_BREAKDOWN",
    -9: "PG_ERR_NONFINITE",
}


class PetgemError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, name, status, msg):
        self.status = status
        super().__init__(f"{name} -> {STATUS.get(status, status)}: {msg}")


_lock = threading.Lock()
_lib = None


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load (building first if needed) and return the ctypes library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_missing and _build.needs_build():
            _build.build()
        path = _build.LIB
        if not os.path.exists(path):
            raise ImportError(f"petgem_gb300 native library not found at {path}; run petgem_gb300._build.build()")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def call(name, *args):
    """Call a status-returning entry point; raise PetgemError on failure."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != 0:
        msg = lib.pg_last_error()
        raise PetgemError(name, st, msg.decode() if msg else "")
    return st


def query(name, *args):
    """Call a size/value query entry point and return its result."""
    return getattr(load(), name)(*args)
