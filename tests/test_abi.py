"""The C-ABI library loads on any machine and exports every function that
include/mandoct_gb300.h declares (no compute calls: no GPU needed)."""
import ctypes
import os
import re

from conftest import ROOT
from reconstruction_program_taichi_gb300 import _lib


def _declared():
    src = open(os.path.join(ROOT, "include", "mandoct_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mct_\w+)\s*\(", src)))


def test_header_declares_the_bound_symbols():
    declared = _declared()
    assert set(_lib.SIGNATURES) == set(declared), set(declared) ^ set(_lib.SIGNATURES)


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for name in _declared():
        assert hasattr(lib, name), name
    assert lib.mct_version().startswith(b"mandoct-gb300")
    assert lib.mct_reduce_scratch_size() > 0


def test_invalid_geometry_is_rejected_without_a_gpu():
    lib = _lib.load()
    g = _lib.Geom()  # all zeros: invalid
    rc = lib.mct_filter(ctypes.byref(g), None, None, None, None)
    assert rc == -1
    assert b"bad detector size" in lib.mct_last_error_string()


def _valid_geom(**kw):
    g = _lib.Geom(nu=64, nv=16, views=90, nv_total=16, nx=32, nz=8, flags=_lib.MCT_CONE, view_mode=1, fp_steps=100,
                  du=1.0, dv=1.0, u0=31.5, u_step=-1.0, v0=-7.5, v_step=1.0, px=1.0, pz=1.0, sid=300.0, sdd=600.0,
                  total_scan_angle=6.2832, fp_step=0.2)
    for k, v in kw.items():
        setattr(g, k, v)
    return g


def _status(name, *args):
    lib = _lib.load()
    rc = getattr(lib, name)(*args)
    return rc, lib.mct_last_error_string().decode()


FAKE = ctypes.c_void_p(4096)  # never dereferenced: every call below fails its checks first


def test_entry_points_reject_bad_arguments_before_any_launch():
    """Error behaviour of the C ABI: each call returns MCT_E_INVALID (-1) with a message
    naming the entry point, before touching device memory."""
    t = _lib.Tables(angles=4096, u=4096, v=4096)
    cases = [
        # volume of 2^31 voxels or more
        ("mct_fp", (ctypes.byref(_valid_geom(nx=46341, nz=1024)), ctypes.byref(t), FAKE, None, FAKE, None, None),
         "2^31"),
        # unsupported storage type
        ("mct_fdk_bp", (ctypes.byref(_valid_geom()), ctypes.byref(t), FAKE, 7, FAKE, None), "dtype"),
        # a view chunk outside the scan
        ("mct_fdk_bp", (ctypes.byref(_valid_geom(view_begin=80, views=20, views_total=90)), ctypes.byref(t), FAKE,
                        0, FAKE, None), "view chunk"),
        # view chunks are only for weighting and FDK backprojection
        ("mct_fp", (ctypes.byref(_valid_geom(view_begin=10, views=20, views_total=90)), ctypes.byref(t), FAKE,
                    None, FAKE, None, None), "view-chunked"),
        # packed operand must be 16-byte aligned
        ("mct_pack", (ctypes.byref(_valid_geom()), FAKE, ctypes.c_void_p(4100), 0, None), "aligned"),
        # the cone-beam gather copies are read with 16-byte loads
        ("mct_fp", (ctypes.byref(_valid_geom()), ctypes.byref(t), FAKE, None, FAKE, ctypes.c_void_p(4104), None),
         "16-byte"),
        # the cell-space adjoint reduces 16 bytes at a time, into a workspace it needs
        ("mct_fp_adjoint_cells", (ctypes.byref(_valid_geom()), ctypes.byref(t), FAKE, None, FAKE,
                                  ctypes.c_void_p(4104), None), "16-byte"),
        ("mct_fp_adjoint_cells", (ctypes.byref(_valid_geom()), ctypes.byref(t), FAKE, None, FAKE, None, None),
         "NULL buffer"),
        # 16-bit forward projection needs a workspace
        ("mct_fp_storage", (ctypes.byref(_valid_geom()), ctypes.byref(t), FAKE, None, FAKE, None, 1, None),
         "workspace"),
        # fan beam backprojection needs a slice per detector row
        ("mct_fdk_bp", (ctypes.byref(_valid_geom(flags=0, nz=32)), ctypes.byref(t), FAKE, 0, FAKE, None),
         "fan beam"),
        # unknown view mode
        ("mct_weight", (ctypes.byref(_valid_geom(view_mode=4)), ctypes.byref(t), FAKE, 0, 0, None, 0, FAKE, None),
         "view_mode"),
        # the fused weighting + tensor-core filter: two storage types, a 1 KiB-aligned workspace
        ("mct_weight_filter", (ctypes.byref(_valid_geom()), ctypes.byref(t), FAKE, 0, 0, None, 0, 2, FAKE, FAKE,
                               None), "dtype"),
        ("mct_weight_filter", (ctypes.byref(_valid_geom()), ctypes.byref(t), FAKE, 0, 0, None, 0, 0,
                               ctypes.c_void_p(4096 + 512), FAKE, None), "1 KiB"),
        # the CG step in the backprojector's epilogue: axial cone beam, float32 / bf16 vectors,
        # the second TV term only with a first
        ("mct_bp_ref_unmatched_packed_cg", (ctypes.byref(_valid_geom(view_mode=2)), ctypes.byref(t), FAKE, 0, FAKE,
                                            FAKE, 1.0, None, 0.0, FAKE, 0, FAKE, FAKE, None), "axial"),
        ("mct_bp_ref_unmatched_packed_cg", (ctypes.byref(_valid_geom()), ctypes.byref(t), FAKE, 0, FAKE, FAKE, 1.0,
                                            None, 0.0, FAKE, 2, FAKE, FAKE, None), "vec_dtype"),
        ("mct_bp_ref_unmatched_packed_cg", (ctypes.byref(_valid_geom()), ctypes.byref(t), FAKE, 0, FAKE, None, 0.0,
                                            FAKE, 1.0, ctypes.c_void_p(8192), 0, FAKE, FAKE, None), "wr2"),
        # a float16 volume is not an iterate type
        ("mct_fp_storage_in", (ctypes.byref(_valid_geom()), ctypes.byref(t), FAKE, 2, None, FAKE, FAKE, 0, None),
         "vol_dtype"),
    ]
    for name, args, text in cases:
        rc, msg = _status(name, *args)
        assert rc == -1, (name, rc, msg)
        assert text in msg, (name, msg)
    h = _lib.Helical(nu=64, nv=16, views=1, view_count=10, n_slices=4, dv=1.0, sdd=600.0, mag=2.0,
                     dis_per_view=0.1)
    rc, msg = _status("mct_helical_rebin", ctypes.byref(h), FAKE, FAKE, FAKE, None)
    assert rc == -1 and "bad sizes" in msg
    rc, msg = _status("mct_dot_f64_noalloc", FAKE, FAKE, (1 << 27) + 1, FAKE, None)
    assert rc == -1 and "134217728" in msg


def test_packed_and_workspace_sizes():
    """Sizes the host allocates from: coefficient operand nv rows (incl. the NaN row)
    x (nu-1) columns per view, 16 B float32 / 8 B 16-bit (+16 for the float16 scale);
    FP copies 32 B per voxel in float32 (quads) and in 16 bits (cells), both orientations; the fan
    beam's transposed copy 4 B per voxel."""
    lib = _lib.load()
    g = _valid_geom()
    n = 90 * 16 * 63
    assert lib.mct_packed_size(ctypes.byref(g), 0) == n * 16
    assert lib.mct_packed_size(ctypes.byref(g), 1) == n * 8
    assert lib.mct_packed_size(ctypes.byref(g), 2) == n * 8 + 16
    fan = _valid_geom(flags=0, nz=16)
    assert lib.mct_packed_size(ctypes.byref(fan), 0) == n * 8
    assert lib.mct_fp_storage_workspace_size(ctypes.byref(g), 1) == 2 * 32 * 32 * 8 * 16
    assert lib.mct_fp_storage_workspace_size(ctypes.byref(g), 2) == 2 * 32 * 32 * 8 * 16 + 16
    assert lib.mct_fp_storage_workspace_size(ctypes.byref(fan), 1) == 0
    assert lib.mct_fp_workspace_size(ctypes.byref(g)) == 2 * 32 * 32 * 8 * 16
    assert lib.mct_fp_storage_workspace_size(ctypes.byref(g), 0) == 2 * 32 * 32 * 8 * 16
    assert lib.mct_fp_workspace_size(ctypes.byref(fan)) == 32 * 32 * 16 * 4
    assert lib.mct_fp_adjoint_workspace_size(ctypes.byref(g)) == 32 * 32 * 8 * 32
    assert lib.mct_fp_adjoint_workspace_size(ctypes.byref(fan)) == 32 * 32 * 16 * 16
    # one float64 partial per block of the CG epilogue (32 x 8 columns x 16 slices)
    assert lib.mct_bp_cg_partials_size(ctypes.byref(g)) == 1 * 4 * 1 * 8
