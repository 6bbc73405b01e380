"""Host-side parameter handling of the drop-in against the reference objects' own
arrays (u, v, angles, filter taps) captured in the golden fixtures."""
import copy
import json
import os
import re

import numpy as np
import pytest

from conftest import golden_names, load_golden, rel_l2
from reconstruction_program_taichi_gb300 import ConfigError, config, geometry


class _Obj:
    verbose = False


def _parse(cfg, kind, tmp_path, z=None):
    cfg = copy.deepcopy(cfg)
    cfg["InputDir"] = str(tmp_path)
    cfg["OutputDir"] = str(tmp_path / "out")
    if z is not None and "pmatrix_input" in z:
        p = tmp_path / "pmatrix.jsonc"
        p.write_text(json.dumps({"Value": [float(v) for v in z["pmatrix_input"]]}))
        cfg["PMatrixFile"] = str(p)
    o = _Obj()
    config.parse_fbp(o, cfg)
    if kind in ("fpj", "ir"):
        config.parse_fpj(o, cfg)
        config.parse_fpj_v3(o, cfg)
    if kind == "ir":
        config.parse_ir(o, cfg)
    return o


@pytest.mark.parametrize("name", golden_names("fbp", exclude=["fbpv2"]) + golden_names("fdk"))
def test_fbp_arrays_and_taps(name, tmp_path):
    z = load_golden(name)
    o = _parse(z["config"], "fbp", tmp_path, z)
    u, v, angles = geometry.fbp_arrays(o)
    # with projection matrices the offsets come out of a float32 decomposition of the
    # matrices (run_mgfbp.py:721-831), reproduced to float32 rounding, not bit for bit
    atol = 5e-6 if "pmatrix_input" in z else 1e-9
    np.testing.assert_allclose(u, z["u"], rtol=0, atol=atol)
    np.testing.assert_allclose(v, z["v"], rtol=0, atol=atol)
    np.testing.assert_allclose(angles, z["angles"], rtol=0, atol=1e-12)
    assert rel_l2(geometry.recon_taps(o), z["taps"]) < 1e-12
    if "gauss_v" in z:
        g = geometry.gaussian_taps(o.det_elem_count_vertical_actual, o.det_elem_height,
                                   o.det_elem_vertical_gauss_filter_size)
        assert rel_l2(g, z["gauss_v"]) < 1e-12


@pytest.mark.parametrize("name", golden_names("fpj_"))
def test_fpj_arrays(name, tmp_path):
    z = load_golden(name)
    o = _parse(z["config"], "fpj", tmp_path)
    u, v, angles = geometry.fpj_arrays(o)
    np.testing.assert_allclose(u, z["u"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(v, z["v"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(angles, z["angles"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(o.array_img_center_z, z["cz"], rtol=0, atol=1e-6)  # float32 in the reference


@pytest.mark.parametrize("name", golden_names("ir", exclude=["ir_admm"]))
def test_ir_arrays(name, tmp_path):
    z = load_golden(name)
    o = _parse(z["config"], "ir", tmp_path)
    u, v, angles = geometry.ir_arrays(o)
    np.testing.assert_allclose(u, z["u"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(v, z["v"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(angles, z["angles"], rtol=0, atol=1e-12)
    assert o.pixel_count_ratio == pytest.approx(
        o.det_elem_count_vertical * o.view_num * o.det_elem_count_horizontal / (o.img_dim_z * o.img_dim ** 2))


def test_missing_and_invalid_keys_raise(tmp_path):
    base = load_golden("fdk_cone")["config"]
    for key, msg in [("Views", "Can not find number of views!"), ("ImageDimension", "can not find ImageDimension!"),
                     ("DetectorElementHeight", "Can not find detector element height for cone beam recon!")]:
        cfg = copy.deepcopy(base)
        del cfg[key]
        with pytest.raises(ConfigError, match=re.escape(msg)):
            _parse(cfg, "fbp", tmp_path)
    for key, val, msg in [("ReconViewMode", "Coronal", "ReconViewMode can only be axial, coronal or sagittal!"),
                          ("ConeBeam", 1, "ConeBeam must be true or false!"),
                          ("OutputFileFormat", "png", "Output file format can only be"),
                          ("ImageDimension", 12.5, "ImageDimension must be a positive integer!")]:
        cfg = copy.deepcopy(base)
        cfg[key] = val
        with pytest.raises(ConfigError, match=re.escape(msg)):
            _parse(cfg, "fbp", tmp_path)


def test_aliases_and_defaults(tmp_path):
    base = load_golden("fdk_cone")["config"]
    cfg = copy.deepcopy(base)
    cfg["SinogramWidth"] = cfg.pop("DetectorElementCountHorizontal")
    cfg["DetectorElementSize"] = cfg.pop("DetectorElementWidth")
    cfg["SliceCount"] = cfg.pop("DetectorElementCountVertical")
    cfg["SliceThickness"] = cfg.pop("DetectorElementHeight")
    cfg["ImageSliceCount"] = cfg.pop("ImageDimensionZ")
    cfg["ImageSliceThickness"] = cfg.pop("VoxelHeight")
    cfg["SliceOffCenter"] = cfg.pop("DetectorOffsetVertical")
    del cfg["SourceIsocenterDistance"]
    o = _parse(cfg, "fbp", tmp_path)
    ref = _parse(base, "fbp", tmp_path)
    for attr in ("det_elem_count_horizontal", "det_elem_width", "det_elem_count_vertical", "det_elem_height",
                 "img_dim_z", "img_voxel_height", "det_offset_vertical"):
        assert getattr(o, attr) == getattr(ref, attr)
    assert o.source_isocenter_dis == o.det_elem_count_horizontal * o.det_elem_width * 1000.0  # "infinity"
    assert o.short_scan == 0 and o.total_scan_angle == pytest.approx(2 * config.PI)


def test_jsonc_comment_stripping(tmp_path):
    p = tmp_path / "c.jsonc"
    p.write_text('// header\n{ "a": 1, /* block\n comment */ "b": "x//y" // tail\n}\n')
    with pytest.raises(Exception):
        config.load_jsonc(str(p))  # the reference's regex also strips '//' inside strings
    p.write_text('// header\n{ "a": 1, /* block\n comment */ "b": 2 // tail\n}\n')
    assert config.load_jsonc(str(p)) == {"a": 1, "b": 2}


@pytest.mark.parametrize("name", golden_names("fpjv"))
def test_fpj_variant_arrays(name, tmp_path):
    z = load_golden(name)
    cfg = copy.deepcopy(z["config"])
    cfg["InputDir"], cfg["OutputDir"] = str(tmp_path), str(tmp_path / "out")
    o = _Obj()
    if name.startswith("fpjv1"):
        config.parse_fpj_v1(o, cfg)
        u, v, angles = geometry.fpj_v1_arrays(o)
    else:
        config.parse_fbp(o, cfg)
        config.parse_fpj(o, cfg)
        u, v, angles = geometry.fpj_v2_arrays(o)
    np.testing.assert_allclose(u, z["u"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(v, z["v"][:len(v)], rtol=0, atol=1e-9)
    np.testing.assert_allclose(angles, z["angles"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("name", golden_names("fdk_pmatrix"))
def test_pmatrix_processing_matches_reference(name, tmp_path):
    """run_mgfbp.py:549-627 and 721-874: source-trajectory fit (optionally to the
    standard form), pixel-size rescaling and vertical recon range applied to the
    projection matrices; derived SID, SDD, offsets and scan angle."""
    z = load_golden(name)
    o = _parse(z["config"], "fbp", tmp_path, z)
    assert o.bool_apply_pmatrix
    np.testing.assert_allclose(np.asarray(o.array_pmatrix, np.float64), z["pmatrix"], rtol=2e-6, atol=2e-6)
    got = [o.source_isocenter_dis, o.source_det_dis, o.det_offset_horizontal, o.det_offset_vertical,
           o.total_scan_angle, o.img_center_z]
    np.testing.assert_allclose(got, z["pm_params"], rtol=1e-6, atol=1e-5)


def test_strided_sinogram_extent():
    """The element count a strided sinogram must hold, which the weighting entry points
    check before any launch: both file layouts fill their buffer exactly, and a view
    chunk of a larger [rows][views][cols] buffer reaches only its own last element."""
    from reconstruction_program_taichi_gb300.ops import strided_extent
    nv, views, nu = 12, 50, 72
    assert strided_extent(nv, views, nu, views * nu, nu) == nv * views * nu  # [rows][views][cols]
    assert strided_extent(nv, views, nu, nu, nv * nu) == nv * views * nu  # post-log [views][rows][cols]
    assert strided_extent(nv, 7, nu, 120 * nu, nu) == (nv - 1) * 120 * nu + 7 * nu
    for rs, vs in ((-1, nu), (nu, -nu)):
        with pytest.raises(ValueError, match="non-negative"):
            strided_extent(nv, views, nu, rs, vs)
