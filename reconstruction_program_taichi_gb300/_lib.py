"""ctypes binding of libmandoct_gb300.so (declared in include/mandoct_gb300.h).

The library is the ONLY compute path of this package: if it is missing or cannot
be loaded, every operator raises ``NativeLibraryError`` (there is no CPU fallback).
"""
import ctypes
import os
import threading

from ._build import LIB_PATH

MCT_OK = 0
MCT_CONE = 1
MCT_CURVED = 2
MCT_SHORT_SCAN = 4
MCT_PMATRIX = 8
MCT_ACCUMULATE = 16
MCT_F32 = 0
MCT_BF16 = 1
MCT_F16 = 2


class NativeLibraryError(RuntimeError):
    """The CUDA library is missing, failed to load, or a call returned an error."""


class Geom(ctypes.Structure):
    """Mirror of struct mct_geom."""

    _fields_ = [
        ("nu", ctypes.c_int32), ("nv", ctypes.c_int32), ("views", ctypes.c_int32), ("nv_total", ctypes.c_int32),
        ("row_begin", ctypes.c_int32), ("nx", ctypes.c_int32), ("nz", ctypes.c_int32), ("flags", ctypes.c_int32),
        ("view_mode", ctypes.c_int32), ("fp_steps", ctypes.c_int32),
        ("du", ctypes.c_float), ("dv", ctypes.c_float), ("u0", ctypes.c_float), ("u_step", ctypes.c_float),
        ("v0", ctypes.c_float), ("v_step", ctypes.c_float), ("px", ctypes.c_float), ("pz", ctypes.c_float),
        ("cx", ctypes.c_float), ("cy", ctypes.c_float), ("cz", ctypes.c_float), ("sid", ctypes.c_float),
        ("sdd", ctypes.c_float), ("img_rot", ctypes.c_float), ("total_scan_angle", ctypes.c_float),
        ("fp_step", ctypes.c_float), ("fp_z_per_view", ctypes.c_float),
        ("view_begin", ctypes.c_int32), ("views_total", ctypes.c_int32),
    ]

    def copy(self, **kw):
        g = Geom()
        ctypes.pointer(g)[0] = self
        for k, v in kw.items():
            setattr(g, k, v)
        return g


class Tables(ctypes.Structure):
    """Mirror of struct mct_tables (device pointers)."""

    _fields_ = [("angles", ctypes.c_void_p), ("u", ctypes.c_void_p), ("v", ctypes.c_void_p), ("cz", ctypes.c_void_p),
                ("pmatrix", ctypes.c_void_p), ("pmat_a", ctypes.c_void_p), ("pmat_xs", ctypes.c_void_p)]


class Helical(ctypes.Structure):
    """Mirror of struct mct_helical."""

    _fields_ = [("nu", ctypes.c_int32), ("nv", ctypes.c_int32), ("views", ctypes.c_int32),
                ("view_count", ctypes.c_int32), ("n_slices", ctypes.c_int32), ("dv", ctypes.c_float),
                ("sdd", ctypes.c_float), ("mag", ctypes.c_float), ("det_offset_vertical", ctypes.c_float),
                ("dis_per_view", ctypes.c_float)]


_P = ctypes.c_void_p
_G = ctypes.POINTER(Geom)
_T = ctypes.POINTER(Tables)
_i32, _i64, _f32, _u64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_uint64

# name -> (restype, argtypes); mirrors include/mandoct_gb300.h
SIGNATURES = {
    "mct_version": (ctypes.c_char_p, []),
    "mct_last_error_string": (ctypes.c_char_p, []),
    "mct_launch_count": (_u64, []),
    "mct_weight": (ctypes.c_int, [_G, _T, _P, _i64, _i64, _P, _i32, _P, _P]),
    "mct_vgauss": (ctypes.c_int, [_G, _P, _P, _P, _P]),
    "mct_filter": (ctypes.c_int, [_G, _P, _P, _P, _P]),
    "mct_filter_tc_workspace_size": (ctypes.c_size_t, [_G, _i32]),
    "mct_filter_tc_prepare": (ctypes.c_int, [_G, _P, _i32, _P, _P]),
    "mct_filter_tc": (ctypes.c_int, [_G, _P, _i32, _P, _P, _P]),
    "mct_filter_tc_status": (ctypes.c_int, [_G, _i32, _P, _P]),
    "mct_packed_size": (ctypes.c_size_t, [_G, _i32]),
    "mct_pack": (ctypes.c_int, [_G, _P, _P, _i32, _P]),
    "mct_pack_strided": (ctypes.c_int, [_G, _P, _i64, _i64, _P, _i32, _P]),
    "mct_bp_ref_unmatched_packed": (ctypes.c_int, [_G, _T, _P, _i32, _P, _P]),
    "mct_fdk_bp": (ctypes.c_int, [_G, _T, _P, _i32, _P, _P]),
    "mct_fdk_bp_finish": (ctypes.c_int, [_G, _P, _P]),
    "mct_helical_rebin": (ctypes.c_int, [ctypes.POINTER(Helical), _P, _P, _P, _P]),
    "mct_fp_workspace_size": (ctypes.c_size_t, [_G]),
    "mct_fp": (ctypes.c_int, [_G, _T, _P, _P, _P, _P, _P]),
    "mct_fp_storage_workspace_size": (ctypes.c_size_t, [_G, _i32]),
    "mct_fp_storage": (ctypes.c_int, [_G, _T, _P, _P, _P, _P, _i32, _P]),
    "mct_fp_adjoint": (ctypes.c_int, [_G, _T, _P, _P, _P, _P]),
    "mct_fp_adjoint_workspace_size": (ctypes.c_size_t, [_G]),
    "mct_fp_adjoint_cells": (ctypes.c_int, [_G, _T, _P, _P, _P, _P, _P]),
    "mct_effective_map": (ctypes.c_int, [_G, _T, _P, _P]),
    "mct_fp_count_samples": (ctypes.c_int, [_G, _T, _P, _P, _P]),
    "mct_bin_noise": (ctypes.c_int, [_G, _P, _i32, _f32, _u64, _P, _P]),
    "mct_bp_ref_unmatched": (ctypes.c_int, [_G, _T, _P, _P, _P]),
    "mct_tv_weights": (ctypes.c_int, [_G, _P, _f32, _P, _P]),
    "mct_dtwd": (ctypes.c_int, [_G, _P, _P, _f32, _P, _f32, _P, _P]),
    "mct_dtwd_dot": (ctypes.c_int, [_G, _P, _P, _f32, _P, _f32, _P, _P, _P, _P]),
    "mct_admm_shrink": (ctypes.c_int, [_G, _P, _f32, _f32, _P, _P, _P, _P, _P]),
    "mct_admm_rhs": (ctypes.c_int, [_G, _P, _P, _P, _P, _P, _f32, _P, _P]),
    "mct_tv_penalty": (ctypes.c_int, [_G, _P, _f32, _P, _P, _P]),
    "mct_reduce_scratch_size": (ctypes.c_size_t, []),
    "mct_dot_f64": (ctypes.c_int, [_P, _P, _i64, _P, _P, _P]),
    "mct_dot_f64_noalloc": (ctypes.c_int, [_P, _P, _i64, _P, _P]),
    "mct_cgls_update": (ctypes.c_int, [_i64, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "mct_cgls_direction": (ctypes.c_int, [_i64, _P, _P, _P, _P, _P]),
    "mct_project_ellipsoids": (ctypes.c_int, [_G, _T, _P, _i32, _P, _P]),
    "mct_fp_storage_in": (ctypes.c_int, [_G, _T, _P, _i32, _P, _P, _P, _i32, _P]),
    "mct_bp_ref_unmatched_packed_out": (ctypes.c_int, [_G, _T, _P, _i32, _P, _i32, _P]),
    "mct_tv_weights_t": (ctypes.c_int, [_G, _P, _i32, _f32, _P, _P]),
    "mct_dtwd_t": (ctypes.c_int, [_G, _P, _P, _f32, _P, _f32, _P, _i32, _P, _P, _P]),
    "mct_dot_f64_t": (ctypes.c_int, [_P, _P, _i64, _i32, _P, _P, _P]),
    "mct_cgls_update_t": (ctypes.c_int, [_i64, _i32, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "mct_cgls_direction_t": (ctypes.c_int, [_i64, _i32, _P, _P, _P, _P, _P]),
    "mct_bp_cg_partials_size": (ctypes.c_size_t, [_G]),
    "mct_weight_filter": (ctypes.c_int, [_G, _T, _P, _i64, _i64, _P, _i32, _i32, _P, _P, _P]),
    "mct_bp_ref_unmatched_packed_cg": (ctypes.c_int, [_G, _T, _P, _i32, _P, _P, _f32, _P, _f32, _P, _i32, _P, _P,
                                                      _P]),
}

_lock = threading.Lock()
_lib = None


def load(path=None):
    """Load the shared library (once) and bind every declared symbol."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = path or os.environ.get("MANDOCT_GB300_LIB", LIB_PATH)
        if not os.path.exists(path):
            raise NativeLibraryError(
                f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(this package has no CPU fallback)")
        try:
            lib = ctypes.CDLL(path)
        except OSError as e:
            raise NativeLibraryError(f"cannot load {path}: {e}") from e
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def call(name, *args):
    """Call a status-returning entry point; raise NativeLibraryError on failure."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != MCT_OK:
        msg = lib.mct_last_error_string().decode(errors="replace")
        raise NativeLibraryError(f"{name} failed ({rc}): {msg}")
    return rc


def launch_count():
    return int(load().mct_launch_count())
