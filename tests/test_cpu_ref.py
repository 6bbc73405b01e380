"""The OpenMP C restatement (CPU baseline) against the reference's golden outputs."""
import numpy as np

from conftest import load_golden, rel_l2
from oracle import PI, cpu_ref
from oracle import fpj_ops as P
from reconstruction_program_taichi_gb300._lib import MCT_CONE, Geom


def test_cpu_fdk_matches_reference():
    z = load_golden("fdk_cone")
    c = z["config"]
    g = Geom()
    g.nu, g.nv, g.views = c["DetectorElementCountHorizontal"], c["DetectorElementCountVertical"], c["Views"]
    g.nx, g.nz = c["ImageDimension"], c["ImageDimensionZ"]
    g.flags = MCT_CONE
    g.du, g.dv, g.px, g.pz = c["DetectorElementWidth"], c["DetectorElementHeight"], c["PixelSize"], c["VoxelHeight"]
    g.u0, g.u_step = z["u"][0], z["u"][1] - z["u"][0]
    g.v0, g.v_step = z["v"][0], z["v"][1] - z["v"][0]
    g.sid, g.sdd = c["SourceIsocenterDistance"], c["SourceDetectorDistance"]
    g.total_scan_angle = 2 * PI
    mid = (c["DetectorElementCountVertical"] - 1) / 2.0
    g.cz = (c["DetectorOffsetVertical"] + ((g.nv - 1) / 2 - mid) * g.dv) * g.sid / g.sdd
    w = z["weighted"].astype(np.float32).copy()
    taps = z["taps"].astype(np.float32)
    F = np.zeros_like(w)
    cpu_ref.filter_rows(g, w, taps, F, 0, g.nv * g.views)
    assert rel_l2(F, z["filtered"]) < 1e-5
    vol = np.zeros((g.nz, g.nx, g.nx), np.float32)
    alive = np.ones(vol.shape, np.uint8)
    ang = z["angles"].astype(np.float32)
    cpu_ref.fdk_bp(g, ang, F, vol, alive, 0, 10)  # two view blocks, as bench.py samples them
    cpu_ref.fdk_bp(g, ang, F, vol, alive, 10, g.views)
    assert rel_l2(vol, z["recon"]) < 1e-4


def test_cpu_fp_matches_reference():
    z = load_golden("fpj_cone")
    c = z["config"]
    g = Geom()
    g.nu, g.nv, g.views = c["DetectorElementCountHorizontal"], c["DetectorElementCountVertical"], c["Views"]
    g.nx, g.nz = c["ImageDimension"], c["ImageDimensionZ"]
    g.flags = MCT_CONE
    g.px, g.pz, g.cx, g.cy, g.cz = c["PixelSize"], c["VoxelHeight"], c["ImageCenter"][0], c["ImageCenter"][1], c["ImageCenterZ"]
    g.sid, g.sdd, g.fp_step = c["SourceIsocenterDistance"], c["SourceDetectorDistance"], c["ForwardProjectionStepSize"]
    g.fp_steps = P.count_steps(g.nx, g.nz, g.px, g.pz, g.fp_step)
    out = np.zeros((g.nv, g.views, g.nu), np.float32)
    cpu_ref.fp(g, z["angles"].astype(np.float32), z["u"].astype(np.float32), z["v"].astype(np.float32),
               z["input_vol"].astype(np.float32), out, 0, g.views)
    assert rel_l2(out[::-1], z["sgm"]) < 1e-4
    assert cpu_ref.threads() >= 1
