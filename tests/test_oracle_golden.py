"""The CPU oracle against fixtures produced by running the reference's own sources
(tests/golden/make_golden.py).  Pins the oracle before it is used as the checker."""
import math

import numpy as np
import pytest

from conftest import golden_names, load_golden, rel_l2
from oracle import PI
from oracle import fbp_ops as F
from oracle import fpj_ops as P
from oracle import ir_ops as I


def _fbp_params(c):
    cone = c.get("ConeBeam", False)
    scan = c.get("TotalScanAngle", 360) / 180 * PI
    short = not (abs(scan % (2 * PI)) < (0.01 / 180 * PI))
    rr = c.get("DetectorElementVerticalReconRange")
    nz = c["ImageDimensionZ"] if cone else c["DetectorElementCountVertical"]
    cz = c.get("ImageCenterZ")
    if cz is None and cone:
        b, e = rr if rr else (0, c["DetectorElementCountVertical"] - 1)
        dist = ((e + b) / 2 - (c["DetectorElementCountVertical"] - 1) / 2) * c["DetectorElementHeight"]
        if c.get("FirstSinogramSliceIsDetectorTopRow", False) or c.get("InputFileForm") == "post_log_images":
            dist = -dist
        cz = (c.get("DetectorOffsetVertical", 0) + dist) * c["SourceIsocenterDistance"] / c["SourceDetectorDistance"]
    return dict(cone=cone, scan=scan, short=short, rr=rr, nz=nz, cz=cz or 0.0)


@pytest.mark.parametrize("name", golden_names("fbp", exclude=["fbpv2"]) + golden_names("fdk"))
def test_fbp_oracle_matches_reference(name):
    z = load_golden(name)
    c = z["config"]
    p = _fbp_params(c)
    nu, du, sdd = c["DetectorElementCountHorizontal"], c["DetectorElementWidth"], c["SourceDetectorDistance"]
    curved = c.get("CurvedDetector", False)
    if "HammingFilter" in c:
        taps = F.hamming_taps(nu, du, c["HammingFilter"], sdd, curved, c.get("DBTMode", False))
    else:
        taps = F.gaussian_apodized_ramp_taps(nu, du, c["GaussianApodizedRamp"], sdd, curved, c.get("DBTMode", False))
    assert rel_l2(taps, z["taps"]) < 1e-12
    sid, cz, pm = c["SourceIsocenterDistance"], p["cz"], None
    if "pmatrix" in z:  # parameters the reference derived from the projection matrices
        sid, sdd, cz, pm = z["pm_params"][0], z["pm_params"][1], z["pm_params"][5], z["pmatrix"]
    sgm = z["input_sgm"].astype(np.float64)
    if p["rr"]:
        sgm = sgm[p["rr"][0]:p["rr"][1] + 1]
    if "BeamHardeningCorrectionCoefficients" in c:
        sgm = F.bh_correct(sgm, c["BeamHardeningCorrectionCoefficients"])
    w = F.weight_sgm(sgm, z["u"], z["v"], z["angles"], sdd, curved, p["short"], p["scan"])
    assert rel_l2(w, z["weighted"]) < 1e-6  # the reference stores the weighted sinogram in float32
    filt = F.filter_rows(z["weighted"], z["taps"], du, z.get("gauss_v"), c.get("DetectorElementHeight", 0.0))
    assert rel_l2(filt, z["filtered"]) < 1e-12
    rec = F.fdk_bp(z["filtered"], z["angles"], z["u"], z["v"], nx=c["ImageDimension"], nz=p["nz"],
                   px=c["PixelSize"], pz=c.get("VoxelHeight", 0.0) if p["cone"] else 0.0,
                   cx=c.get("ImageCenter", [0, 0])[0], cy=c.get("ImageCenter", [0, 0])[1], cz=cz, pmatrix=pm,
                   sid=sid, sdd=sdd, dv=c.get("DetectorElementHeight", 0.0),
                   img_rot=c.get("ImageRotation", 0) / 180 * PI, total_scan_angle=p["scan"], short_scan=p["short"],
                   cone_beam=p["cone"], curved=curved,
                   view_mode={"axial": 1, "coronal": 2, "sagittal": 3}[c.get("ReconViewMode", "axial")])
    if "WaterMu" in c:
        rec = (rec / c["WaterMu"] - 1) * 1000
    assert rel_l2(rec, z["recon"]) < 1e-12
    np.testing.assert_array_equal(rec == 0, z["recon"] == 0)


@pytest.mark.parametrize("name", golden_names("fpj_"))
def test_fp_oracle_matches_reference(name):
    z = load_golden(name)
    c = z["config"]
    cone = c.get("ConeBeam", False)
    nv, nu, os_ = c["DetectorElementCountVertical"], c["DetectorElementCountHorizontal"], c.get("OversampleSize", 1)
    nx = c["ImageDimension"]
    nz = c["ImageDimensionZ"] if cone else nv
    px, pz = c["PixelSize"], (c.get("VoxelHeight", 0.0) if cone else 0.0)
    step = c.get("ForwardProjectionStepSize", 0.2)
    K = P.count_steps(nx, nz, px, pz, step)
    zpv = P.helical_z_per_view(z["angles"], z["v"], nv, c["HelicalPitch"], c["SourceIsocenterDistance"],
                               c["SourceDetectorDistance"]) if "HelicalPitch" in c else 0.0
    out = np.zeros((nv, c["Views"], nu))
    for j in range(c["Views"]):
        big = P.march(z["input_vol"], j, z["angles"], z["u"], z["v"], nx=nx, nz=nz, px=px, pz=pz,
                      cx=c["ImageCenter"][0], cy=c["ImageCenter"][1], cz_view=z["cz"][j],
                      sid=c["SourceIsocenterDistance"], sdd=c["SourceDetectorDistance"], step=step, cone_beam=cone,
                      curved=c.get("CurvedDetector", False), zpv=zpv, rows=nv, K=K)
        out[:, j, :] = P.bin_sinogram(big, os_)
    if cone and c.get("OutputFileForm", "sinogram") == "sinogram":
        out = out[::-1]
    assert rel_l2(out, z["sgm"]) < 1e-6  # the reference stores projections in float32


@pytest.mark.parametrize("name", golden_names("ir", exclude=["ir_admm"]))
def test_ir_oracle_matches_reference(name):
    z = load_golden(name)
    c = z["config"]
    g = dict(rows=c["DetectorElementCountVertical"], views=c["Views"], nu=c["DetectorElementCountHorizontal"],
             nx=c["ImageDimension"], nz=c["ImageDimensionZ"], px=c["PixelSize"], pz=c["VoxelHeight"], cx=0.0,
             cy=0.0, cz=z["cz"], sid=c["SourceIsocenterDistance"], sdd=c["SourceDetectorDistance"],
             step=c["ForwardProjectionStepSize"], cone=True, curved=False, zpv=0.0, angles=z["angles"], u=z["u"],
             v=z["v"], dv=c["DetectorElementHeight"], img_rot=0.0)
    g["K"] = P.count_steps_ir(g["nx"], g["nz"], g["px"], g["pz"], g["step"], g["sid"])
    ops = I.IrOperators(g)
    em = ops.emap()
    assert np.array_equal(em, z["emap"]) and 0.0 < em.mean() < 1.0
    sgm = z["input_sgm"].astype(np.float64)
    assert rel_l2(ops.bp(sgm * em), z["bp_b"]) < 1e-12
    assert rel_l2(ops.fp(z["probe_x"], em), z["probe_fp"]) < 1e-6
    assert rel_l2(ops.ptp(z["probe_x"], em), z["probe_ptp"]) < 1e-12
    wr = I.generate_wr(z["probe_x"], c["BetaTV"])
    assert rel_l2(wr, z["probe_wr"]) < 1e-12
    assert rel_l2(I.dtwd(z["probe_x"], wr), z["probe_dtwd"]) < 1e-12
    assert math.isclose(I.tv_penalty(z["probe_x"], c["BetaTV"]), float(z["probe_tv"]), rel_tol=1e-12)
    mu = c["WaterMu"]
    ops.calls = 0
    if "Alpha" in c:
        prior = (z["prior"].astype(np.float64) / 1000 + 1) * mu
        x = I.irn_piccs(ops, sgm, prior, c["Lambda"], c["Alpha"], c["BetaTV"], c["NumberOfIRNIterations"],
                        c["NumberOfIterations"])
    else:
        seed = (z["fbp_seed"] / 1000 + 1) * mu
        x = I.irn_tv(ops, sgm, seed, c["Lambda"], c["BetaTV"], c["NumberOfIRNIterations"], c["NumberOfIterations"])
    assert ops.calls == int(z["ptp_calls"])
    assert rel_l2((x / mu - 1) * 1000, z["recon"]) < 1e-6


@pytest.mark.parametrize("name", golden_names("fpjv"))
def test_fp_variant_oracle_matches_reference(name):
    """run_mgfpj.py (v1) and run_mgfpj_v2.py (v2) projectors."""
    z = load_golden(name)
    c = z["config"]
    cone = c.get("ConeBeam", False)
    nu, os_ = c["DetectorElementCountHorizontal"], c.get("OversampleSize", 1)
    nx = c["ImageDimension"]
    nz = c["ImageDimensionZ"]
    nv = c["DetectorElementCountVertical"] if cone else nz
    px, pz = c["PixelSize"], (c.get("VoxelHeight", 0.0) if cone else 0.0)
    step = c.get("ForwardProjectionStepSize", 0.2)
    K = P.count_steps_ir(nx, nz, px, pz, step, c["SourceIsocenterDistance"])
    rr = c.get("DetectorElementVerticalReconRange", [0, nv - 1])
    rows = rr[1] - rr[0] + 1
    out = np.zeros((nv, c["Views"], nu))
    for j in range(c["Views"]):
        big = P.march(z["input_vol"], j, z["angles"], z["u"], z["v"], nx=nx, nz=nz, px=px, pz=pz,
                      cx=c["ImageCenter"][0], cy=c["ImageCenter"][1], cz_view=c.get("ImageCenterZ", 0.0),
                      sid=c["SourceIsocenterDistance"], sdd=c["SourceDetectorDistance"], step=step, cone_beam=cone,
                      rows=rows, K=K)
        out[rr[0]:rr[1] + 1, j, :] = P.bin_sinogram(big, os_)
    if cone and c.get("OutputFileForm", "sinogram") == "sinogram":
        out = out[::-1]
    assert rel_l2(out, z["sgm"]) < 1e-6


@pytest.mark.parametrize("name", golden_names("helical"))
def test_helical_rebin_oracle_matches_reference(name):
    """run_mgfbp_helical.py:59-95 parameters and :178-205 rebinning."""
    z = load_golden(name)
    c = z["config"]
    sid, sdd = c["SourceIsocenterDistance"], c["SourceDetectorDistance"]
    nv, dv, nb = c["DetectorElementCountVertical"], c["DetectorElementHeight"], c["Views"]
    scan = c["TotalScanAngle"] / 180 * PI
    mag = sdd / sid
    coverage = nv * dv / mag
    dis_per_view = c["HelicalPitch"] * coverage / (nb / (abs(scan) / (2 * PI)))
    angle_per_view = scan / nb
    gamma_max = 2 * np.arctan(0.5 * c["DetectorElementCountHorizontal"] * c["DetectorElementWidth"] / sdd) / PI
    short = max(2 * PI / abs(c["HelicalPitch"]), PI + gamma_max)
    view_count = int(np.ceil(short / abs(angle_per_view)))
    assert z["rebinned"].shape[1] == view_count
    out = F.helical_rebin(z["input_sgm"], z["z_pos"], view_count=view_count, dis_per_view=dis_per_view, mag=mag,
                          det_offset_vertical=c.get("DetectorOffsetVertical", 0.0), dv=dv, sdd=sdd)
    # the reference writes the stack as float32
    assert rel_l2(out, z["rebinned"]) < 1e-6
    np.testing.assert_array_equal(out == 0, z["rebinned"] == 0)


def test_admm_oracle_matches_reference():
    """run_mgfbp_iterative_recon_ADMM_CGLS.py: x-, v- and p-steps, the hard threshold."""
    z = load_golden("ir_admm")
    c = z["config"]
    g = dict(rows=c["DetectorElementCountVertical"], views=c["Views"], nu=c["DetectorElementCountHorizontal"],
             nx=c["ImageDimension"], nz=c["ImageDimensionZ"], px=c["PixelSize"], pz=c["VoxelHeight"], cx=0.0,
             cy=0.0, cz=z["cz"], sid=c["SourceIsocenterDistance"], sdd=c["SourceDetectorDistance"],
             step=c["ForwardProjectionStepSize"], cone=True, curved=False, zpv=0.0, angles=z["angles"], u=z["u"],
             v=z["v"], dv=c["DetectorElementHeight"], img_rot=0.0)
    g["K"] = P.count_steps_ir(g["nx"], g["nz"], g["px"], g["pz"], g["step"], g["sid"])
    ops = I.IrOperators(g)
    mu = c["WaterMu"]
    seed = (z["fbp_seed"] / 1000 + 1) * mu
    ops.calls = 0
    x, vy, vx, py, px = I.admm_tv(ops, z["input_sgm"].astype(np.float64), seed, c["Lambda"],
                                  c["NumberOfIRNIterations"], c["NumberOfIterations"])
    assert ops.calls == int(z["ptp_calls"])
    assert rel_l2((x / mu - 1) * 1000, z["recon"]) < 1e-5
    # the reference's v_x / p_x are along axis 1 (y here), v_y / p_y along axis 2
    assert rel_l2(vy, z["v_x"]) < 1e-5 and rel_l2(vx, z["v_y"]) < 1e-5
    assert rel_l2(py, z["p_x"]) < 1e-5 and rel_l2(px, z["p_y"]) < 1e-5
    np.testing.assert_array_equal(vy == 0, z["v_x"] == 0)


@pytest.mark.parametrize("name", ["fpj_cone", "fpj_helical", "fpj_cone_postlog_curved", "fpj_fan_oversample2"])
def test_oracle_adjoint_is_the_transpose_of_the_oracle_projector(name):
    """<P x, y> = <x, P^T y> in float64 to 1e-12 for the oracle's 'adjoint' mode, on the
    geometries of the reference's projector fixtures (cone, helical, curved, fan), with a
    ray mask: the oracle adjoint the GPU's exact adjoint is compared with is itself the
    transpose of the projector pinned to the reference above."""
    z = load_golden(name)
    c = z["config"]
    cone = c.get("ConeBeam", False)
    nv, nu = c["DetectorElementCountVertical"], c["DetectorElementCountHorizontal"] * c.get("OversampleSize", 1)
    nx = c["ImageDimension"]
    nz = c["ImageDimensionZ"] if cone else nv
    px, pz = c["PixelSize"], (c.get("VoxelHeight", 0.0) if cone else 0.0)
    step = c.get("ForwardProjectionStepSize", 0.2)
    K = P.count_steps(nx, nz, px, pz, step)
    zpv = P.helical_z_per_view(z["angles"], z["v"], nv, c["HelicalPitch"], c["SourceIsocenterDistance"],
                               c["SourceDetectorDistance"]) if "HelicalPitch" in c else 0.0
    rng = np.random.default_rng(17)
    x = rng.uniform(0, 1, (nz, nx, nx))
    views = min(c["Views"], 6)
    y = rng.uniform(-1, 1, (views, nv, nu))
    mask = (rng.uniform(0, 1, (views, nv, nu)) > 0.2).astype(np.float64)
    kw = dict(nx=nx, nz=nz, px=px, pz=pz, cx=c["ImageCenter"][0], cy=c["ImageCenter"][1],
              sid=c["SourceIsocenterDistance"], sdd=c["SourceDetectorDistance"], step=step, cone_beam=cone,
              curved=c.get("CurvedDetector", False), zpv=zpv, rows=nv, K=K)
    lhs, aty = 0.0, np.zeros_like(x)
    for j in range(views):
        ax = P.march(x, j, z["angles"], z["u"], z["v"], cz_view=z["cz"][j], mask=mask[j], **kw)
        lhs += float((ax * y[j]).sum())
        P.march(None, j, z["angles"], z["u"], z["v"], cz_view=z["cz"][j], mask=mask[j], mode="adjoint",
                ray_values=y[j], out=aty, **kw)
    rhs = float((x * aty).sum())
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)
    assert np.count_nonzero(aty) > 0
