"""The OpenMP C restatement against the reference's golden outputs (float32 build:
the CPU baseline) and against the float64 NumPy restatement (float64 build: the FP64
checker of benchmark-size results, including its slab and row-block mode)."""
import numpy as np
import pytest

from conftest import load_golden, rel_l2
from oracle import PI, cpu_ref
from oracle import fbp_ops as F
from oracle import fpj_ops as P


def _fdk_geom(z):
    c = z["config"]
    nv = c["DetectorElementCountVertical"]
    g = cpu_ref.CpuGeom(nu=c["DetectorElementCountHorizontal"], nv=nv, views=c["Views"], nx=c["ImageDimension"],
                        nz=c["ImageDimensionZ"], cone=True, du=c["DetectorElementWidth"], dv=c["DetectorElementHeight"],
                        u0=z["u"][0], u_step=z["u"][1] - z["u"][0], v0=z["v"][0], v_step=z["v"][1] - z["v"][0],
                        px=c["PixelSize"], pz=c["VoxelHeight"], sid=c["SourceIsocenterDistance"],
                        sdd=c["SourceDetectorDistance"], total_scan_angle=2 * PI)
    g.cz = (c["DetectorOffsetVertical"] + ((nv - 1) / 2 - (nv - 1) / 2.0) * g.dv) * g.sid / g.sdd
    return g


def _fp_geom(z):
    c = z["config"]
    g = cpu_ref.CpuGeom(nu=c["DetectorElementCountHorizontal"], nv=c["DetectorElementCountVertical"],
                        views=c["Views"], nx=c["ImageDimension"], nz=c["ImageDimensionZ"], cone=True,
                        px=c["PixelSize"], pz=c["VoxelHeight"], cx=c["ImageCenter"][0], cy=c["ImageCenter"][1],
                        cz=c["ImageCenterZ"], sid=c["SourceIsocenterDistance"], sdd=c["SourceDetectorDistance"],
                        fp_step=c["ForwardProjectionStepSize"])
    g.fp_steps = P.count_steps(g.nx, g.nz, g.px, g.pz, g.fp_step)
    return g


def test_cpu_fdk_matches_reference():
    z = load_golden("fdk_cone")
    g = _fdk_geom(z)
    w = z["weighted"].astype(np.float32).copy()
    taps = z["taps"].astype(np.float32)
    filt = np.zeros_like(w)
    cpu_ref.filter_rows(g, w, taps, filt, 0, g.nv * g.views)
    assert rel_l2(filt, z["filtered"]) < 1e-5
    vol = np.zeros((g.nz, g.nx, g.nx), np.float32)
    alive = np.ones(vol.shape, np.uint8)
    ang = z["angles"].astype(np.float32)
    assert cpu_ref.fdk_bp(g, ang, filt, vol, alive, 0, 10) == 0  # two view blocks, as bench.py samples them
    assert cpu_ref.fdk_bp(g, ang, filt, vol, alive, 10, g.views) == 0
    assert rel_l2(vol, z["recon"]) < 1e-4


def test_cpu_fp_matches_reference():
    z = load_golden("fpj_cone")
    g = _fp_geom(z)
    out = np.zeros((g.nv, g.views, g.nu), np.float32)
    cpu_ref.fp(g, z["angles"].astype(np.float32), z["u"].astype(np.float32), z["v"].astype(np.float32),
               z["input_vol"].astype(np.float32), out, 0, g.views)
    assert rel_l2(out[::-1], z["sgm"]) < 1e-4
    assert cpu_ref.threads() >= 1


def test_f64_build_matches_the_numpy_oracle_fdk():
    """Float64 weighting, filter and backprojection against oracle/fbp_ops on the
    golden case, to float64 rounding; the reference's own float32 result within 1e-4."""
    z = load_golden("fdk_cone")
    g = _fdk_geom(z)
    rng = np.random.default_rng(3)
    sgm = rng.uniform(0, 1, (g.nv, g.views, g.nu))
    u = z["u"].astype(np.float64)
    v = z["v"].astype(np.float64)
    ang = z["angles"].astype(np.float64)
    w = sgm.copy()
    cpu_ref.weight(g, w, 64)
    w_ref = F.weight_sgm(sgm, u, v, ang, g.sdd)
    assert rel_l2(w, w_ref) < 1e-13
    taps = z["taps"].astype(np.float64)
    filt = np.empty_like(w)
    cpu_ref.filter_rows(g, w.reshape(-1, g.nu), taps, filt.reshape(-1, g.nu), 0, g.nv * g.views, 64)
    filt_ref = F.filter_rows(w_ref, taps, g.du)
    assert rel_l2(filt, filt_ref) < 1e-13
    vol = np.zeros((g.nz, g.nx, g.nx))
    alive = np.ones(vol.shape, np.uint8)
    assert cpu_ref.fdk_bp(g, ang, filt, vol, alive, 0, g.views, 64) == 0
    ref = F.fdk_bp(filt_ref, ang, u, v, nx=g.nx, nz=g.nz, px=g.px, pz=g.pz, cx=0.0, cy=0.0, cz=g.cz, sid=g.sid,
                   sdd=g.sdd, dv=g.dv, img_rot=0.0, total_scan_angle=2 * PI, short_scan=0, cone_beam=True)
    assert np.array_equal(vol == 0, ref == 0)
    assert rel_l2(vol, ref) < 1e-12
    # the reference's own pipeline on its sinogram
    full, rows = cpu_ref.fdk_slab_f64(g, ang, z["input_sgm"], taps, 0, g.nz)
    assert rel_l2(full, z["recon"]) < 1e-4


@pytest.mark.parametrize("z0,z1", [(0, 3), (3, 5), (6, 8)])
def test_f64_slab_matches_whole_volume(z0, z1):
    """A slab from the detector rows it reads equals the same slices of the whole-volume
    result (and the row block is smaller than the detector for the central slab)."""
    z = load_golden("fdk_cone")
    g = _fdk_geom(z)
    rng = np.random.default_rng(4)
    sgm = rng.uniform(0, 1, (g.nv, g.views, g.nu))
    taps = z["taps"].astype(np.float64)
    ang = z["angles"].astype(np.float64)
    keep = sgm.copy()
    whole, rows = cpu_ref.fdk_slab_f64(g, ang, sgm, taps, 0, g.nz)
    slab, rows = cpu_ref.fdk_slab_f64(g, ang, sgm, taps, z0, z1)
    assert np.array_equal(sgm, keep)  # the input is not modified
    assert np.array_equal(slab, whole[z0:z1])
    assert 0 <= rows[0] < rows[1] <= g.nv and rows[1] - rows[0] < g.nv


def test_f64_build_matches_the_numpy_oracle_fp():
    z = load_golden("fpj_cone")
    g = _fp_geom(z)
    vol = z["input_vol"].astype(np.float64)
    ang, u, v = (z[k].astype(np.float64) for k in ("angles", "u", "v"))
    views = [0, 3, g.views - 1]
    got = cpu_ref.fp_views_f64(g, ang, u, v, vol, views)
    for i, j in enumerate(views):
        ref = P.march(vol, j, ang, u, v, nx=g.nx, nz=g.nz, px=g.px, pz=g.pz, cx=g.cx, cy=g.cy, cz_view=g.cz,
                      sid=g.sid, sdd=g.sdd, step=g.fp_step, cone_beam=True, K=g.fp_steps)
        assert rel_l2(got[:, i], ref) < 1e-13


def test_errors_helper():
    e = cpu_ref.errors(np.array([1.0, 2.0, 3.5]), np.array([1.0, 2.0, 3.0]))
    assert e["max_abs"] == 0.5 and abs(e["rel_l2"] - 0.5 / np.sqrt(14.0)) < 1e-15


def test_f64_unmatched_backprojector_matches_the_numpy_oracle():
    """The IR driver's per-view backprojector (float64 C, slab and row block) against
    oracle/ir_ops.bp_unmatched."""
    from oracle import ir_ops as I
    nx, nz, nu, nv, views = 20, 8, 40, 12, 24
    sid, sdd, px, pz, du, dv = 300.0, 550.0, 0.6, 0.6, 0.8, 1.2
    ang = np.arange(views) * (2 * PI / views) + 0.1
    u = (np.arange(nu) - (nu - 1) / 2.0) * (-du) - 0.3
    v = (np.arange(nv) - (nv - 1) / 2.0) * (-dv) + 0.2
    cz = np.full(views, 0.15)
    g = cpu_ref.CpuGeom(nu=nu, nv=nv, views=views, nx=nx, nz=nz, cone=True, du=du, dv=dv, u0=u[0],
                        u_step=u[1] - u[0], v0=v[0], v_step=v[1] - v[0], px=px, pz=pz, cx=0.4, cy=-0.3, sid=sid,
                        sdd=sdd, img_rot=0.05)
    rng = np.random.default_rng(12)
    sgm = rng.uniform(0, 1, (nv, views, nu))
    ref = I.bp_unmatched(sgm, ang, u, v, cz, nx=nx, nz=nz, px=px, pz=pz, cx=0.4, cy=-0.3, sid=sid, sdd=sdd, dv=dv,
                         img_rot=0.05, cone_beam=True)
    whole, _ = cpu_ref.bp_unmatched_slab_f64(g, ang, cz, sgm, 0, nz)
    assert np.array_equal(whole == 0, ref == 0)
    assert rel_l2(whole, ref) < 1e-12
    slab, rows = cpu_ref.bp_unmatched_slab_f64(g, ang, cz, sgm, 3, 5)
    assert np.array_equal(slab, whole[3:5])
