"""Generate golden fixtures by running the REFERENCE's own Python sources.

The reference (MandoCT-Taichi) is a set of Python scripts whose kernels are
Taichi DSL.  Taichi is not installable here, so this script puts
``tests/golden/refshim`` (a small stand-in for the ``taichi``, ``crip.io`` and
``matplotlib`` APIs that executes kernel bodies sequentially in float64) ahead
of the reference directory on ``sys.path`` and drives the reference classes
exactly as its entry points do (run_mgfbp.py:18-47, run_mgfpj_v3.py:45-77,
run_mgfbp_iterative_recon_IRN_CGLS.py:14-49, ..._piccs.py:13-45).

Usage (needs the reference checkout; writes tests/golden/*.npz):
    python tests/golden/make_golden.py /path/to/reference [case ...]

Each fixture holds the jsonc config (as text), the inputs and the reference's
outputs, plus intermediate arrays read back from the reference objects.
"""
import contextlib
import copy
import json
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# ---------------------------------------------------------------- cases
BASE_FAN = {
    "InputFiles": "sgm_.*.raw", "OutputFilePrefix": "", "OutputFileReplace": ["sgm", "rec"],
    "DetectorElementCountHorizontal": 40, "DetectorElementWidth": 1.2, "DetectorOffsetHorizontal": 0.7,
    "DetectorElementCountVertical": 2, "Views": 30, "TotalScanAngle": 360,
    "SourceIsocenterDistance": 300, "SourceDetectorDistance": 600,
    "ImageDimension": 16, "PixelSize": 1.5, "ImageRotation": 15, "ImageCenter": [1.0, -0.5],
    "HammingFilter": 1,
}
BASE_CONE = {
    "InputFiles": "sgm_.*.raw", "OutputFilePrefix": "", "OutputFileReplace": ["sgm", "rec"],
    "DetectorElementCountHorizontal": 28, "DetectorElementWidth": 1.6, "DetectorOffsetHorizontal": -0.4,
    "DetectorElementCountVertical": 14, "DetectorElementHeight": 1.6, "DetectorOffsetVertical": 0.5,
    "Views": 20, "TotalScanAngle": 360, "SourceIsocenterDistance": 200, "SourceDetectorDistance": 400,
    "ImageDimension": 12, "PixelSize": 1.2, "ImageDimensionZ": 8, "VoxelHeight": 1.2,
    "ConeBeam": True, "HammingFilter": 1,
}


def _upd(base, **kw):
    d = copy.deepcopy(base)
    d.update(kw)
    return d


FBP_CASES = {
    "fbp2d_ramp": _upd(BASE_FAN),
    "fbp2d_curved_short": _upd(BASE_FAN, CurvedDetector=True, TotalScanAngle=250, Views=36,
                               HammingFilter=0.6, BeamHardeningCorrectionCoefficients=[1.0, 0.05]),
    "fbp2d_gauss_dbt_hu": _upd(BASE_FAN, TotalScanAngle=720, Views=48, DBTMode=True, WaterMu=0.02,
                               HammingFilter=None, GaussianApodizedRamp=1.3),
    "fdk_cone": _upd(BASE_CONE),
    "fdk_cone_postlog_coronal": _upd(BASE_CONE, InputFileForm="post_log_images", ReconViewMode="coronal",
                                     DetectorElementVerticalReconRange=[1, 12],
                                     DetectorElementVerticalGaussFilterSize=1.5, ImageCenterZ=0.3,
                                     HammingFilter=0.8),
    "fdk_cone_sagittal_curved_short": _upd(BASE_CONE, ReconViewMode="sagittal", CurvedDetector=True,
                                           TotalScanAngle=200, Views=24, ImageRotation=30,
                                           FirstSinogramSliceIsDetectorTopRow=True),
}

BASE_FPJ = {
    "InputFiles": "img_.*.raw", "OutputFilePrefix": "", "OutputFileReplace": ["img", "sgm"],
    "DetectorElementCountHorizontal": 24, "DetectorElementWidth": 1.6, "DetectorOffsetHorizontal": 0.5,
    "DetectorElementCountVertical": 12, "DetectorElementHeight": 1.6, "DetectorOffsetVertical": -0.3,
    "Views": 12, "TotalScanAngle": 360, "SourceIsocenterDistance": 200, "SourceDetectorDistance": 400,
    "ImageDimension": 14, "PixelSize": 1.2, "ImageDimensionZ": 8, "VoxelHeight": 1.2,
    "ImageRotation": 10, "ImageCenter": [0.5, -0.4], "ImageCenterZ": 0.2,
    "ConeBeam": True, "ForwardProjectionStepSize": 0.4,
}

FPJ_CASES = {
    "fpj_cone": _upd(BASE_FPJ),
    "fpj_cone_postlog_curved": _upd(BASE_FPJ, OutputFileForm="post_log_images", CurvedDetector=True,
                                    ImageCenterZ=None),
    "fpj_fan_oversample2": _upd(BASE_FPJ, ConeBeam=False, DetectorElementCountVertical=3,
                                ImageDimensionZ=3, OversampleSize=2, DetectorElementHeight=None,
                                DetectorOffsetVertical=None, VoxelHeight=None, ImageCenterZ=None,
                                ImageDimension=12),
    "fpj_helical": _upd(BASE_FPJ, HelicalPitch=0.5, TotalScanAngle=720, Views=16),
}

# the original stand-alone projector (run_mgfpj.py) and the Mgfbp-derived one
# (run_mgfpj_v2.py)
FPJ_V1_CASES = {
    "fpjv1_cone": _upd(BASE_FPJ, StartAngle=20, ImageRotation=None, DetectorOffsetVertical=None,
                       DetectorZOffcenter=0.4),
    "fpjv1_fan_oversample2": _upd(BASE_FPJ, ConeBeam=False, OversampleSize=2, ImageDimensionZ=3,
                                  ImageDimension=12, PhotonNumber=None),
}
FPJ_V2_CASES = {
    "fpjv2_cone_rowrange": _upd(BASE_FPJ, DetectorElementVerticalReconRange=[2, 9]),
}

BASE_IR = {
    "InputFiles": "sgm_.*.raw", "OutputFilePrefix": "", "OutputFileReplace": ["sgm", "rec"],
    "InputFileForm": "post_log_images",
    "DetectorElementCountHorizontal": 16, "DetectorElementWidth": 1.6, "DetectorOffsetHorizontal": 0.3,
    "DetectorElementCountVertical": 10, "DetectorElementHeight": 2.0, "DetectorOffsetVertical": 0.4,
    "Views": 10, "TotalScanAngle": 360, "SourceIsocenterDistance": 200, "SourceDetectorDistance": 400,
    "ImageDimension": 10, "PixelSize": 1.2, "ImageDimensionZ": 6, "VoxelHeight": 1.2,
    "ConeBeam": True, "HammingFilter": 1, "ForwardProjectionStepSize": 0.5,
    "WaterMu": 0.02, "Lambda": 1e-3, "BetaTV": 1e-6, "NumberOfIRNIterations": 1, "NumberOfIterations": 2,
}

IR_CASES = {
    "ir_tv": _upd(BASE_IR),
    "ir_piccs": _upd(BASE_IR, Alpha=0.5),
}

# ADMM-TV (run_mgfbp_iterative_recon_ADMM_CGLS.py); Lambda puts the shrink threshold
# (lambda * ratio / rho) inside the range of the image gradients
ADMM_CASES = {
    "ir_admm": _upd(BASE_IR, Alpha=0.5, Lambda=4e-4, NumberOfIRNIterations=3, NumberOfIterations=2),
}

# the view-by-view FBP (run_mgfbp_v2.py): same configs, its own driver
FBPV2_CASES = {
    "fbpv2_cone": _upd(BASE_CONE),
    "fbpv2_fan_short_curved": _upd(BASE_FAN, CurvedDetector=True, TotalScanAngle=250, Views=36,
                                   HammingFilter=0.6, BeamHardeningCorrectionCoefficients=[1.0, 0.05]),
}

# helical FBP by per-slice rebinning (run_mgfbp_helical.py)
BASE_HELICAL = _upd(BASE_CONE, Views=72, TotalScanAngle=1080, HelicalPitch=1.0, DetectorOffsetVertical=0.0)
HELICAL_CASES = {
    "helical_full": _upd(BASE_HELICAL),
    "helical_short_curved": _upd(BASE_HELICAL, Views=90, HelicalPitch=-1.5, CurvedDetector=True, HammingFilter=0.8,
                                 DetectorOffsetVertical=0.8, ImageRotation=12,
                                 BeamHardeningCorrectionCoefficients=[1.0, 0.03]),
}

# FDK with projection matrices (run_mgfbp.py:549-627, 721-874, 1134-1141): the matrices
# are synthesised from a circular geometry (see pmatrices()); "tilt" raises the source
# path out of the z = 0 plane so that ModifyPMatrixToStandardForm has work to do.
PM_CASES = {
    "fdk_pmatrix": (_upd(BASE_CONE, DetectorOffsetHorizontal=0.0, DetectorOffsetVertical=0.0),
                    dict(u_shift=0.3, v_shift=-0.2, tilt=0.0, scale=1.0)),
    "fdk_pmatrix_standardise": (_upd(BASE_CONE, DetectorOffsetHorizontal=0.0, DetectorOffsetVertical=0.0,
                                     ModifyPMatrixToStandardForm=True, PMatrixDetectorElementWidth=0.8,
                                     PMatrixDetectorElementHeight=0.8, DetectorElementVerticalReconRange=[1, 12]),
                                dict(u_shift=-0.4, v_shift=0.25, tilt=0.02, scale=0.5)),
}


def pmatrices(cfg, u_shift, v_shift, tilt, scale):
    """3x4 matrices P_j = [e_u e_v d]^-1 [I | -s] of a circular scan: source s at angle
    beta_j on a circle of radius SID (z = tilt * SID * sin(beta) when tilted), flat
    detector at SDD with pixel vectors e_u, e_v (lengths = pixel size * scale, i.e. a
    detector binned 1/scale relative to the scan) and the origin shifted by
    (u_shift, v_shift) pixels.  Returned flattened, 12 values per view."""
    nb, nu, nv = cfg["Views"], cfg["DetectorElementCountHorizontal"], cfg["DetectorElementCountVertical"]
    sid, sdd = float(cfg["SourceIsocenterDistance"]), float(cfg["SourceDetectorDistance"])
    du, dv = cfg["DetectorElementWidth"] * scale, cfg["DetectorElementHeight"] * scale
    nu_p, nv_p = nu / scale, nv / scale
    out = []
    for j in range(nb):
        b = 2 * np.pi * j / nb
        c, s_ = np.cos(b), np.sin(b)
        src = np.array([sid * c, sid * s_, tilt * sid * s_])
        e_u = du * np.array([s_, -c, 0.0])
        e_v = dv * np.array([0.0, 0.0, -1.0])
        center = src - sdd * np.array([c, s_, tilt * s_]) / np.sqrt(1 + (tilt * s_) ** 2)
        origin = center - ((nu_p - 1) / 2 + u_shift) * e_u - ((nv_p - 1) / 2 + v_shift) * e_v
        m = np.linalg.inv(np.stack([e_u, e_v, origin - src], axis=1))
        out.append(np.concatenate([m, (-m @ src)[:, None]], axis=1).reshape(-1))
    return np.concatenate(out)


def run_fbpv2_case(name, cfg, RV2, rng):
    cfg = _clean(cfg)
    with tempfile.TemporaryDirectory() as d, _chdir(d):
        os.makedirs("sgm")
        cfg.update(InputDir=d + "/sgm", OutputDir=d + "/rec")
        sgm = rng.uniform(0.0, 1.0, (cfg["DetectorElementCountVertical"], cfg["Views"],
                                     cfg["DetectorElementCountHorizontal"])).astype(np.float32)
        sgm.tofile("sgm/sgm_a.raw")
        json.dump(cfg, open("config.jsonc", "w"))
        fbp = RV2.Mgfbp_v2(RV2.ReadConfigFile("config.jsonc"))
        img = fbp.MainFunction()
        return dict(config=json.dumps(cfg), input_sgm=sgm, recon=np.asarray(img, np.float64))


def run_helical_case(name, cfg, RH, rng):
    cfg = _clean(cfg)
    with tempfile.TemporaryDirectory() as d, _chdir(d):
        os.makedirs("sgm")
        cfg.update(InputDir=d + "/sgm", OutputDir=d + "/rec")
        sgm = rng.uniform(0.0, 1.0, (cfg["DetectorElementCountVertical"], cfg["Views"],
                                     cfg["DetectorElementCountHorizontal"])).astype(np.float32)
        sgm.tofile("sgm/sgm_a.raw")
        json.dump(cfg, open("config.jsonc", "w"))
        fbp = RH.Mgfbp_helical(RH.ReadConfigFile("config.jsonc"))
        img = fbp.MainFunction()
        rebinned = np.fromfile("sgm/temp/sgm_rebin.raw", dtype=np.float32)
        return dict(config=json.dumps(cfg), input_sgm=sgm, recon=np.asarray(img, np.float64),
                    rebinned=rebinned.reshape(len(fbp.array_z_pos), fbp.view_count, -1).astype(np.float64),
                    z_pos=np.asarray(fbp.array_z_pos, np.float64))


def run_admm_case(name, cfg, RA, R, rng):
    cfg = _clean(cfg)
    with tempfile.TemporaryDirectory() as d, _chdir(d):
        os.makedirs("sgm")
        cfg.update(InputDir=d + "/sgm", OutputDir=d + "/rec")
        n, nz = cfg["ImageDimension"], cfg["ImageDimensionZ"]
        nu, nv, nb = cfg["DetectorElementCountHorizontal"], cfg["DetectorElementCountVertical"], cfg["Views"]
        sgm = (rng.uniform(0.0, 0.4, (nv, nb, nu)) + 0.1).astype(np.float32)
        sgm.transpose(1, 0, 2).tofile("sgm/sgm_a.raw")
        prior = (rng.uniform(-200, 200, (nz, n, n))).astype(np.float32)
        prior.tofile("prior.raw")
        cfg["PriorImageFile"] = d + "/prior.raw"
        json.dump(cfg, open("config.jsonc", "w"))
        seed = R.Mgfbp(R.ReadConfigFile("config.jsonc")).MainFunction()
        obj = RA.Mgfbp_ir_piccs(R.ReadConfigFile("config.jsonc"))
        img = obj.MainFunction(np.array(seed))
        return dict(config=json.dumps(cfg), input_sgm=sgm, prior=prior, fbp_seed=np.asarray(seed, np.float64),
                    recon=np.asarray(img, np.float64), v_x=np.asarray(obj.v_x, np.float64),
                    v_y=np.asarray(obj.v_y, np.float64), p_x=np.asarray(obj.p_x, np.float64),
                    p_y=np.asarray(obj.p_y, np.float64), ptp_calls=obj.num_iter_runned,
                    emap=np.asarray(obj.img_fp_effective_map, np.float64),
                    bp_b=np.asarray(obj.img_bp_b, np.float64), u=_arr(obj.array_u_taichi),
                    v=_arr(obj.array_v_taichi), angles=_arr(obj.array_angle_taichi),
                    cz=_arr(obj.array_img_center_z_taichi).ravel())


def run_pmatrix_case(name, spec, R, rng):
    cfg, geo = spec
    cfg = _clean(cfg)
    with tempfile.TemporaryDirectory() as d, _chdir(d):
        pm = pmatrices(cfg, **geo)
        path = os.path.join(d, "pmatrix.jsonc")
        json.dump({"Value": [float(v) for v in pm]}, open(path, "w"))
        cfg = dict(cfg, PMatrixFile=path)
        out = run_fbp_case(name, cfg, R, rng)
        out["pmatrix_input"] = pm
        return out


class _MathCompat:
    """The math module with size-1 NumPy arrays accepted where scalars are expected."""

    def __getattr__(self, name):
        import math
        f = getattr(math, name)
        if not callable(f):
            return f

        def g(*a):
            return f(*[float(np.asarray(x).reshape(-1)[0]) if isinstance(x, np.ndarray) and x.size == 1 else x
                       for x in a])
        return g


# per-view side files (run_mgfpj_v3.py:131-172): ScanAngleFile (degrees; Mgfbp_ir keeps
# them, Mgfpj_v3's InitializeArrays overwrites them) and ImageCenterZFile (per-view image
# centre z, used by both projectors and the IR backprojector)
SIDE_FPJ_CASES = {
    "fpj_cone_sidefiles": _upd(BASE_FPJ, __ScanAngles=[0.0, 27.0, 61.5, 88.0, 121.0, 149.5, 183.0, 210.0, 241.5,
                                                       268.0, 302.0, 330.5],
                               __CenterZ=[0.2 + 0.15 * j for j in range(12)]),
}
SIDE_IR_CASES = {
    "ir_tv_sidefiles": _upd(BASE_IR, __ScanAngles=[3.0, 40.0, 71.0, 105.0, 139.0, 178.0, 212.0, 250.0, 288.0, 323.0],
                            __CenterZ=[0.4 - 0.2 * j for j in range(10)]),
}


def _clean(cfg):
    return {k: v for k, v in cfg.items() if v is not None}


def _side_files(cfg, out):
    """Write the case's per-view side files into the working folder, point the config
    at them and keep their values in the fixture."""
    if "__ScanAngles" in cfg:
        vals = cfg.pop("__ScanAngles")
        json.dump({"Value": vals}, open("scan_angle.jsonc", "w"))
        cfg["ScanAngleFile"] = os.path.abspath("scan_angle.jsonc")
        out["side_scan_angles"] = np.asarray(vals, np.float64)
    if "__CenterZ" in cfg:
        vals = cfg.pop("__CenterZ")
        json.dump({"Value": vals}, open("center_z.jsonc", "w"))
        cfg["ImageCenterZFile"] = os.path.abspath("center_z.jsonc")
        out["side_center_z"] = np.asarray(vals, np.float64)


@contextlib.contextmanager
def _chdir(d):
    old = os.getcwd()
    os.chdir(d)
    try:
        yield
    finally:
        os.chdir(old)


def _arr(field):
    return np.asarray(field.to_numpy(), dtype=np.float64)


def _smooth_volume(rng, nz, n):
    """A few random blobs, so that projections are smooth and non-trivial."""
    z, y, x = np.meshgrid(np.linspace(-1, 1, nz), np.linspace(-1, 1, n), np.linspace(-1, 1, n), indexing="ij")
    v = np.zeros((nz, n, n))
    for _ in range(4):
        c = rng.uniform(-0.5, 0.5, 3)
        s = rng.uniform(0.2, 0.5)
        v += rng.uniform(0.5, 1.5) * np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / s ** 2)
    return (v * 0.02 + rng.uniform(0, 0.002, v.shape)).astype(np.float32)


def run_fbp_case(name, cfg, R, rng):
    cfg = _clean(cfg)
    with tempfile.TemporaryDirectory() as d, _chdir(d):
        os.makedirs("sgm")
        cfg.update(InputDir=d + "/sgm", OutputDir=d + "/rec")
        nu = cfg["DetectorElementCountHorizontal"]
        nv = cfg["DetectorElementCountVertical"]
        nb = cfg["Views"]
        sgm = rng.uniform(0.0, 1.0, (nv, nb, nu)).astype(np.float32)
        if cfg.get("InputFileForm") == "post_log_images":
            sgm.transpose(1, 0, 2).tofile("sgm/sgm_a.raw")
        else:
            sgm.tofile("sgm/sgm_a.raw")
        json.dump(cfg, open("config.jsonc", "w"))
        conf = R.ReadConfigFile("config.jsonc")
        fbp = R.Mgfbp(conf)
        img = fbp.MainFunction()
        out = dict(config=json.dumps(cfg), input_sgm=sgm, recon=np.asarray(img, np.float64),
                   taps=_arr(fbp.array_recon_kernel_taichi), u=_arr(fbp.array_u_taichi),
                   v=_arr(fbp.array_v_taichi), angles=_arr(fbp.array_angle_taichi),
                   weighted=np.asarray(fbp.img_sgm, np.float64), filtered=_arr(fbp.img_sgm_filtered_taichi))
        if fbp.apply_gauss_vertical:
            out["gauss_v"] = _arr(fbp.array_kernel_gauss_vertical_taichi)
        if getattr(fbp, "bool_apply_pmatrix", 0):
            out["pmatrix"] = np.asarray(fbp.array_pmatrix, np.float64)
            out["pm_params"] = np.array([fbp.source_isocenter_dis, fbp.source_det_dis, fbp.det_offset_horizontal,
                                         fbp.det_offset_vertical, fbp.total_scan_angle, fbp.img_center_z],
                                        np.float64)
        return out


def run_fpj_case(name, cfg, R3, rng):
    cfg = _clean(cfg)
    with tempfile.TemporaryDirectory() as d, _chdir(d):
        os.makedirs("img")
        cfg.update(InputDir=d + "/img", OutputDir=d + "/sgm")
        vol = _smooth_volume(rng, cfg.get("ImageDimensionZ", cfg["DetectorElementCountVertical"]),
                             cfg["ImageDimension"])
        if not cfg.get("ConeBeam", False):
            vol = _smooth_volume(rng, cfg["DetectorElementCountVertical"], cfg["ImageDimension"])
        vol.tofile("img/img_a.raw")
        side = {}
        _side_files(cfg, side)
        json.dump(cfg, open("config.jsonc", "w"))
        conf = R3.ReadConfigFile("config.jsonc")
        fpj = R3.Mgfpj_v3(conf)
        sgm = fpj.MainFunction()
        return dict(config=json.dumps(cfg), input_vol=vol, sgm=np.asarray(sgm, np.float64),
                    u=_arr(fpj.array_u_taichi), v=_arr(fpj.array_v_taichi),
                    angles=_arr(fpj.array_angle_taichi), cz=_arr(fpj.array_img_center_z_taichi).ravel(), **side)


def run_fpj_variant_case(name, cfg, module, rng):
    """Mgfpj of run_mgfpj.py (v1) or run_mgfpj_v2.py (v2)."""
    cfg = _clean(cfg)
    with tempfile.TemporaryDirectory() as d, _chdir(d):
        os.makedirs("img")
        os.makedirs("sgm")  # run_mgfpj.py does not create its output folder
        cfg.update(InputDir=d + "/img", OutputDir=d + "/sgm")
        nz = cfg.get("ImageDimensionZ") if cfg.get("ConeBeam") else cfg.get("ImageDimensionZ",
                                                                             cfg["DetectorElementCountVertical"])
        if not cfg.get("ConeBeam") and "DetectorElementVerticalReconRange" not in cfg and name.startswith("fpjv2"):
            nz = cfg["DetectorElementCountVertical"]
        vol = _smooth_volume(rng, nz, cfg["ImageDimension"])
        vol.tofile("img/img_a.raw")
        json.dump(cfg, open("config.jsonc", "w"))
        fpj = module.Mgfpj(module.ReadConfigFile("config.jsonc"))
        sgm = fpj.MainFunction()
        return dict(config=json.dumps(cfg), input_vol=vol, sgm=np.asarray(sgm, np.float64),
                    u=_arr(fpj.array_u_taichi), v=_arr(fpj.array_v_taichi), angles=_arr(fpj.array_angle_taichi))


def run_ir_case(name, cfg, RI, RP, R, rng):
    cfg = _clean(cfg)
    with tempfile.TemporaryDirectory() as d, _chdir(d):
        os.makedirs("sgm")
        cfg.update(InputDir=d + "/sgm", OutputDir=d + "/rec")
        n, nz = cfg["ImageDimension"], cfg["ImageDimensionZ"]
        nu, nv, nb = cfg["DetectorElementCountHorizontal"], cfg["DetectorElementCountVertical"], cfg["Views"]
        sgm = (rng.uniform(0.0, 0.4, (nv, nb, nu)) + 0.1).astype(np.float32)
        sgm.transpose(1, 0, 2).tofile("sgm/sgm_a.raw")  # post_log_images layout [views, rows, cols]
        out = dict(input_sgm=sgm)
        if "Alpha" in cfg:
            prior = (rng.uniform(-200, 200, (nz, n, n))).astype(np.float32)  # HU
            prior.tofile("prior.raw")
            cfg["PriorImageFile"] = d + "/prior.raw"
            out["prior"] = prior
        _side_files(cfg, out)
        json.dump(cfg, open("config.jsonc", "w"))
        conf = R.ReadConfigFile("config.jsonc")
        if "Alpha" in cfg:
            obj = RP.Mgfbp_ir_piccs(conf)
            img = obj.MainFunction()
        else:
            seed = R.Mgfbp(R.ReadConfigFile("config.jsonc")).MainFunction()
            out["fbp_seed"] = np.asarray(seed, np.float64)
            obj = RI.Mgfbp_ir(conf)
            img = obj.MainFunction(seed)
        out.update(config=json.dumps(cfg), recon=np.asarray(img, np.float64),
                   emap=np.asarray(obj.img_fp_effective_map, np.float64),
                   bp_b=np.asarray(obj.img_bp_b, np.float64),
                   u=_arr(obj.array_u_taichi), v=_arr(obj.array_v_taichi),
                   angles=_arr(obj.array_angle_taichi), cz=_arr(obj.array_img_center_z_taichi).ravel(),
                   ptp_calls=obj.num_iter_runned)
        # single-operator probes on the same object
        xt = rng.uniform(0.0, 0.03, (nz, n, n))
        out["probe_x"] = xt
        out["probe_fp"] = np.asarray(obj.ForwardProjection(xt), np.float64)
        out["probe_ptp"] = np.asarray(obj.ForwardProjectionAndBackProjection(xt), np.float64)
        wr = obj.GenerateWR(xt, cfg["BetaTV"])
        out["probe_wr"] = np.asarray(wr, np.float64)
        out["probe_dtwd"] = np.asarray(obj.Dt_W_D(xt, wr), np.float64)
        out["probe_tv"] = float(obj.TVPenaltyVal(xt))
        return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MANDOCT_REFERENCE", "")
    if not ref or not os.path.isdir(ref):
        sys.exit("usage: make_golden.py /path/to/reference [case ...]")
    only = set(sys.argv[2:])
    sys.path.insert(0, ref)
    sys.path.insert(0, os.path.join(HERE, "refshim"))
    import taichi as ti_shim  # the stand-in
    import run_mgfbp as R
    import run_mgfpj_v3 as R3
    import run_mgfbp_iterative_recon_IRN_CGLS as RI
    import run_mgfbp_iterative_recon_IRN_CGLS_piccs as RP
    import run_mgfpj as R1
    import run_mgfpj_v2 as R2
    import run_mgfbp_v2 as RV2
    import run_mgfbp_helical as RH
    import run_mgfbp_iterative_recon_ADMM_CGLS as RA
    # NumPy >= 2 no longer turns size-1 arrays into Python scalars in math.cos & co.;
    # the reference relies on that (run_mgfbp.py:738-741, on least-squares solutions of
    # shape (3, 1)), so its modules get a math whose functions convert them first, as
    # the NumPy of the reference's time did.
    for mod in (R, R3, RI, RP, R1, R2, RV2, RH, RA):
        if hasattr(mod, "math"):
            mod.math = _MathCompat()
    jobs = [(k, v, "fbp") for k, v in FBP_CASES.items()] + [(k, v, "fpj") for k, v in FPJ_CASES.items()] \
        + [(k, v, "ir") for k, v in IR_CASES.items()] + [(k, v, "v1") for k, v in FPJ_V1_CASES.items()] \
        + [(k, v, "v2") for k, v in FPJ_V2_CASES.items()] + [(k, v, "pm") for k, v in PM_CASES.items()] \
        + [(k, v, "fbpv2") for k, v in FBPV2_CASES.items()] + [(k, v, "helical") for k, v in HELICAL_CASES.items()] \
        + [(k, v, "admm") for k, v in ADMM_CASES.items()] + [(k, v, "fpj") for k, v in SIDE_FPJ_CASES.items()] \
        + [(k, v, "ir") for k, v in SIDE_IR_CASES.items()]
    for i, (name, cfg, kind) in enumerate(jobs):
        if only and name not in only:
            continue
        rng = np.random.default_rng(1000 + i)
        ti_shim.seed(1000 + i)
        t = time.time()
        with open(os.devnull, "w") as devnull, contextlib.redirect_stdout(devnull):
            if kind == "fbp":
                out = run_fbp_case(name, cfg, R, rng)
            elif kind == "fpj":
                out = run_fpj_case(name, cfg, R3, rng)
            elif kind == "pm":
                out = run_pmatrix_case(name, cfg, R, rng)
            elif kind == "fbpv2":
                out = run_fbpv2_case(name, cfg, RV2, rng)
            elif kind == "helical":
                out = run_helical_case(name, cfg, RH, rng)
            elif kind == "admm":
                out = run_admm_case(name, cfg, RA, R, rng)
            elif kind in ("v1", "v2"):
                out = run_fpj_variant_case(name, cfg, R1 if kind == "v1" else R2, rng)
            else:
                out = run_ir_case(name, cfg, RI, RP, R, rng)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(f"{name}: {time.time() - t:.1f}s")


if __name__ == "__main__":
    main()
