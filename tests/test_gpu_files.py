"""Folders of several scans: the drivers read the next file and write the previous
result while the GPU works on the current one; every output file must be what a
single-file run writes, and the returned array the last file's (after its in-place
conversion, HU here), as in the reference's sequential loop."""
import json
import os

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _folder_case(tmp_path, name, cfg, arrays, in_prefix, out_prefix):
    d_in, d_out = tmp_path / (name + "_in"), tmp_path / (name + "_out")
    d_in.mkdir()
    for tag, a in arrays.items():
        a.astype(np.float32).tofile(d_in / f"{in_prefix}_{tag}.raw")
    cfg = dict(cfg, InputDir=str(d_in), OutputDir=str(d_out))
    p = tmp_path / (name + ".jsonc")
    p.write_text(json.dumps(cfg))
    return str(p), d_in, d_out


def _last_listed(d_in, in_prefix):
    return [f for f in os.listdir(d_in) if f.startswith(in_prefix + "_")][-1]


def test_run_mgfbp_over_a_folder_matches_single_file_runs(tmp_path, cuda):
    from reconstruction_program_taichi_gb300 import run_mgfbp
    z = load_golden("fdk_cone")
    cfg = dict(z["config"], WaterMu=0.02)
    scans = {t: z["input_sgm"] * s for t, s in (("a", 1.0), ("b", 0.5), ("c", 2.0), ("d", 1.5))}
    path, d_in, d_out = _folder_case(tmp_path, "all", cfg, scans, "sgm", "rec")
    ret = run_mgfbp(path, verbose=False)
    assert sorted(os.listdir(d_out)) == ["rec_a.raw", "rec_b.raw", "rec_c.raw", "rec_d.raw"]
    for t, s in scans.items():
        p1, _, d1 = _folder_case(tmp_path, "one_" + t, cfg, {t: s}, "sgm", "rec")
        one = run_mgfbp(p1, verbose=False)
        got = np.fromfile(d_out / f"rec_{t}.raw", dtype=np.float32)
        assert np.array_equal(got, np.fromfile(d1 / f"rec_{t}.raw", dtype=np.float32)), t
        assert np.array_equal(got.reshape(one.shape), one), t
    last = _last_listed(d_in, "sgm").replace("sgm", "rec")
    assert np.array_equal(ret.ravel(), np.fromfile(d_out / last, dtype=np.float32))


def test_run_mgfpj_v3_over_a_folder_matches_single_file_runs(tmp_path, cuda):
    from reconstruction_program_taichi_gb300 import run_mgfpj_v3
    z = load_golden("fpj_cone")
    cfg = dict(z["config"])
    vols = {t: z["input_vol"] * s for t, s in (("a", 1.0), ("b", 0.25), ("c", 3.0))}
    path, d_in, d_out = _folder_case(tmp_path, "all", cfg, vols, "img", "sgm")
    ret = run_mgfpj_v3(path, verbose=False)
    assert sorted(os.listdir(d_out)) == ["sgm_a.raw", "sgm_b.raw", "sgm_c.raw"]
    for t, v in vols.items():
        p1, _, d1 = _folder_case(tmp_path, "one_" + t, cfg, {t: v}, "img", "sgm")
        run_mgfpj_v3(p1, verbose=False)
        assert np.array_equal(np.fromfile(d_out / f"sgm_{t}.raw", dtype=np.float32),
                              np.fromfile(d1 / f"sgm_{t}.raw", dtype=np.float32)), t
    last = _last_listed(d_in, "img").replace("img", "sgm")
    assert np.array_equal(ret.ravel(), np.fromfile(d_out / last, dtype=np.float32))


def test_tiff_output_format(tmp_path, cuda):
    """OutputFileFormat 'tif' (run_mgfbp.py:1199-1203, 1306-1309): the output file is
    named *.tif and holds the returned volume, one page per slice; SaveFilteredSinogram
    writes the filtered sinogram as a TIFF with one page per view, [views, rows, cols]
    (the reference transposes its [rows, views, cols] array before writing, :1293-1298)."""
    from test_tiff import read_tiff
    from reconstruction_program_taichi_gb300 import run_mgfbp
    z = load_golden("fdk_cone")
    cfg = dict(z["config"], OutputFileFormat="tif", SaveFilteredSinogram=True)
    path, d_in, d_out = _folder_case(tmp_path, "tif", cfg, {"a": z["input_sgm"]}, "sgm", "rec")
    vol = run_mgfbp(path, verbose=False)
    assert sorted(os.listdir(d_out)) == ["rec_a.tif", "sgm_filtered_rec_a.tif"]
    back = read_tiff(d_out / "rec_a.tif")
    assert back.shape == vol.shape and np.array_equal(back, vol)
    filt = read_tiff(d_out / "sgm_filtered_rec_a.tif")
    want = z["filtered"].transpose(1, 0, 2)
    assert filt.shape == want.shape
    assert np.linalg.norm(filt - want) / np.linalg.norm(want) < 1e-4
