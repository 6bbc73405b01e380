"""Build and bind oracle/cpu_ref.c (OpenMP C restatement) -- TEST INFRASTRUCTURE.

Two builds of the same source: float32 (``prec=32``, Taichi's default precision;
bench.py's timed CPU baseline, "port") and float64 (``prec=64``; the FP64 checker of
results at benchmark sizes, pinned to the float64 NumPy restatement by
tests/test_cpu_ref.py).  Used by tests and by bench.py's CPU leg; the product never
imports it.
"""
import ctypes
import math
import os
import shutil
import subprocess
from dataclasses import dataclass, fields, replace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpu_ref.c")
OUT_DIR = os.path.join(HERE, "_build")
LIBS = {32: os.path.join(OUT_DIR, "libmandoct_cpu_ref.so"), 64: os.path.join(OUT_DIR, "libmandoct_cpu_ref64.so")}
_libs = {}


def build(force=False):
    """Compile both builds (skipped when up to date); returns their paths."""
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = shutil.which("gcc") or "cc"
    for prec, lib in LIBS.items():
        if not force and os.path.exists(lib) and os.path.getmtime(lib) >= os.path.getmtime(SRC):
            continue
        real = ["-DREAL=double"] if prec == 64 else []
        cmd = [cc, "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", *real, "-o", lib + ".tmp", SRC, "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("cpu_ref build failed:\n" + r.stdout + r.stderr)
        os.replace(lib + ".tmp", lib)
    return dict(LIBS)


def load(prec=32):
    if prec not in LIBS:
        raise ValueError("prec must be 32 or 64")
    if prec not in _libs:
        build()
        lib = ctypes.CDLL(LIBS[prec])
        lib.cpu_threads.restype = ctypes.c_int
        lib.cpu_real_bytes.restype = ctypes.c_int
        lib.cpu_fdk_bp.restype = ctypes.c_int64
        assert lib.cpu_real_bytes() == prec // 8
        _libs[prec] = lib
    return _libs[prec]


@dataclass
class CpuGeom:
    """Geometry of the C restatement, float64 on the Python side (converted to the
    build's precision inside, as Taichi converts its Python-float fields)."""
    nu: int = 1
    nv: int = 1
    views: int = 1
    nx: int = 1
    nz: int = 1
    cone: bool = True
    curved: bool = False
    short_scan: bool = False
    fp_steps: int = 0
    du: float = 1.0
    dv: float = 1.0
    u0: float = 0.0
    u_step: float = 1.0
    v0: float = 0.0
    v_step: float = 1.0
    px: float = 1.0
    pz: float = 1.0
    cx: float = 0.0
    cy: float = 0.0
    cz: float = 0.0
    sid: float = 1.0
    sdd: float = 1.0
    img_rot: float = 0.0
    total_scan_angle: float = 2 * 3.1415926536
    fp_step: float = 0.2

    _INT = ("nu", "nv", "views", "nx", "nz", "cone", "curved", "short_scan", "fp_steps")

    def arrays(self):
        gi = np.array([int(getattr(self, k)) for k in self._INT], dtype=np.int64)
        gd = np.array([float(getattr(self, f.name)) for f in fields(self) if f.name not in self._INT],
                      dtype=np.float64)
        return gi, gd

    def copy(self, **kw):
        return replace(self, **kw)


def geom_from_config(o, u, v, fp_steps=0):
    """CpuGeom of a parsed config (attributes of config.parse_fbp / parse_fpj) with
    the detector position arrays u, v of the operator to run (FBP arrays for the
    weighting, filter and backprojection; the ray arrays are passed to fp())."""
    u = np.asarray(u, dtype=np.float64)
    v = np.asarray(v, dtype=np.float64)
    return CpuGeom(nu=len(u), nv=len(v), views=o.view_num, nx=o.img_dim, nz=o.img_dim_z, cone=bool(o.cone_beam),
                   curved=bool(o.curved_dect), short_scan=bool(o.short_scan), fp_steps=int(fp_steps),
                   du=o.det_elem_width, dv=o.det_elem_height, u0=u[0], u_step=(u[1] - u[0]) if len(u) > 1 else 1.0,
                   v0=v[0], v_step=(v[1] - v[0]) if len(v) > 1 else 1.0, px=o.img_pix_size, pz=o.img_voxel_height,
                   cx=o.img_center_x, cy=o.img_center_y, cz=o.img_center_z, sid=o.source_isocenter_dis,
                   sdd=o.source_det_dis, img_rot=o.img_rot, total_scan_angle=o.total_scan_angle,
                   fp_step=getattr(o, "fpj_step_size", 0.2))


def _p(a, prec):
    want = np.float64 if prec == 64 else np.float32
    if a.dtype != want or not a.flags.c_contiguous:
        raise TypeError(f"array must be C-contiguous {np.dtype(want).name} for the {prec}-bit build")
    return a.ctypes.data_as(ctypes.c_void_p)


def _g(geom):
    gi, gd = geom.arrays()
    return gi, gd, gi.ctypes.data_as(ctypes.c_void_p), gd.ctypes.data_as(ctypes.c_void_p)


def threads():
    return int(load().cpu_threads())


def weight(geom, sgm, prec=32):
    gi, gd, pi, pd = _g(geom)
    load(prec).cpu_weight(pi, pd, _p(sgm, prec))


def filter_rows(geom, x, taps, y, r0, r1, prec=32):
    gi, gd, pi, pd = _g(geom)
    load(prec).cpu_filter(pi, pd, _p(x, prec), _p(taps, prec), _p(y, prec), ctypes.c_int64(r0), ctypes.c_int64(r1))


def fdk_bp(geom, angles, F, vol, alive, v0, v1, prec=32, z0=0, z1=None, f_row0=0):
    """vol [z1-z0, nx, nx] += views [v0, v1) of the filtered sinogram block F (detector
    rows [f_row0, f_row0 + F.shape[0])); returns the number of updates whose rows lie
    outside the block (0 when it covers the slab)."""
    z1 = geom.nz if z1 is None else z1
    assert vol.shape == (z1 - z0, geom.nx, geom.nx) and alive.shape == vol.shape and alive.dtype == np.uint8
    assert F.ndim == 3 and F.shape[1:] == (geom.views, geom.nu)
    gi, gd, pi, pd = _g(geom)
    n = int(load(prec).cpu_fdk_bp(pi, pd, _p(angles, prec), _p(F, prec), ctypes.c_int(f_row0),
                                     ctypes.c_int(F.shape[0]), _p(vol, prec), alive.ctypes.data_as(ctypes.c_void_p),
                                     ctypes.c_int(z0), ctypes.c_int(z1), ctypes.c_int(v0), ctypes.c_int(v1)))
    if n < 0:
        raise MemoryError("cpu_fdk_bp: out of host memory")
    return n


def fp(geom, angles, u, v, vol, out, v0, v1, prec=32):
    gi, gd, pi, pd = _g(geom)
    load(prec).cpu_fp(pi, pd, _p(angles, prec), _p(u, prec), _p(v, prec), _p(vol, prec), _p(out, prec),
                      ctypes.c_int(v0), ctypes.c_int(v1))


# ---------------------------------------------------------------- FP64 checks at size

def slab_rows(geom, z0, z1):
    """Detector rows [r0, r1) that the axial FDK backprojection of slices [z0, z1)
    can read (flat or curved cone beam), with a row of margin on each side."""
    if not geom.cone:
        return z0, z1
    half = (geom.nx - 1) / 2.0 * geom.px
    rmax = math.hypot(half + abs(geom.cx), half + abs(geom.cy))
    zs = [((iz - (geom.nz - 1) / 2.0) * geom.pz + geom.cz) for iz in (z0, z1 - 1)]
    ls = [geom.sid - rmax, geom.sid + rmax]
    if ls[0] <= 0:
        return 0, geom.nv
    sgn = 1.0 if geom.v_step > 0 else -1.0
    vals = [(geom.sdd / L * z - geom.v0) / geom.dv * sgn for L in ls for z in zs]
    r0 = max(0, int(math.floor(min(vals))) - 1)
    r1 = min(geom.nv, int(math.floor(max(vals))) + 3)
    return r0, max(r0 + 1, r1)


def fdk_slab_f64(geom, angles, sgm, taps, z0, z1):
    """Float64 FDK (flat/curved cosine weighting of a full scan, direct Toeplitz row
    filter, axial pixel-driven backprojection with the break-to-zero rule) of slices
    [z0, z1) from the raw sinogram sgm [nv, views, nu].  Only the detector rows the slab
    reads are weighted and filtered.  Returns (slab [z1-z0, nx, nx] float64, (r0, r1))."""
    r0, r1 = slab_rows(geom, z0, z1)
    sub = geom.copy(nv=r1 - r0, v0=geom.v0 + r0 * geom.v_step)
    # weighted in place: a copy; sgm may be any array-like that slices by detector row
    block = np.array(sgm[r0:r1], dtype=np.float64, order="C", copy=True)
    weight(sub, block, 64)
    filt = np.empty_like(block)
    filter_rows(sub, block.reshape(-1, geom.nu), np.ascontiguousarray(taps, dtype=np.float64),
                filt.reshape(-1, geom.nu), 0, (r1 - r0) * geom.views, 64)
    vol = np.zeros((z1 - z0, geom.nx, geom.nx), np.float64)
    alive = np.ones(vol.shape, np.uint8)
    ang = np.ascontiguousarray(angles, dtype=np.float64)
    misses = fdk_bp(geom, ang, filt, vol, alive, 0, geom.views, 64, z0, z1, r0)
    if misses:
        raise RuntimeError(f"row block [{r0}, {r1}) does not cover slices [{z0}, {z1}): {misses} misses")
    return vol, (r0, r1)


def fp_views_f64(geom, angles, u, v, vol, views):
    """Float64 forward projection (run_mgfpj_v3 ray march, flat detector, circular) of
    vol [nz, nx, nx] for the listed views; returns [nv, len(views), nu] float64."""
    out = np.zeros((geom.nv, geom.views, geom.nu), np.float64)
    ang = np.ascontiguousarray(angles, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    vol = np.ascontiguousarray(vol, dtype=np.float64)
    for j in views:
        fp(geom, ang, u, v, vol, out, int(j), int(j) + 1, 64)
    return out[:, list(views), :]


def errors(got, want, mask=None):
    """rel-L2 and max-abs of got against want (float64), optionally on a mask."""
    g = np.asarray(got, dtype=np.float64)
    w = np.asarray(want, dtype=np.float64)
    if mask is not None:
        g, w = g[mask], w[mask]
    d = g - w
    return {"rel_l2": float(np.linalg.norm(d) / max(np.linalg.norm(w), 1e-300)),
            "max_abs": float(np.abs(d).max()) if d.size else 0.0,
            "max_abs_rel_to_peak": float(np.abs(d).max() / max(np.abs(w).max(), 1e-300)) if d.size else 0.0}


def bp_unmatched_slab_f64(geom, angles, cz_views, sgm, z0, z1):
    """Float64 IR backprojector (the reference's per-view "P^T" with its u-truncation
    flag) of slices [z0, z1) from sgm [nv, views, nu]; only the detector rows the slab
    reads are passed.  Returns (slab float64 [z1-z0, nx, nx], (r0, r1))."""
    lo, hi = [], []
    for c in (min(cz_views), max(cz_views)):
        r = slab_rows(geom.copy(cz=float(c)), z0, z1)
        lo.append(r[0])
        hi.append(r[1])
    r0, r1 = min(lo), max(hi)
    block = np.ascontiguousarray(sgm[r0:r1], dtype=np.float64)
    vol = np.zeros((z1 - z0, geom.nx, geom.nx), np.float64)
    flag = np.ones(vol.shape, np.uint8)
    gi, gd, pi, pd = _g(geom)
    lib = load(64)
    lib.cpu_bp_unmatched.restype = ctypes.c_int64
    misses = lib.cpu_bp_unmatched(pi, pd, _p(np.ascontiguousarray(angles, dtype=np.float64), 64),
                                  _p(np.ascontiguousarray(cz_views, dtype=np.float64), 64), _p(block, 64),
                                  ctypes.c_int(r0), ctypes.c_int(r1 - r0), _p(vol, 64),
                                  flag.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(z0), ctypes.c_int(z1),
                                  ctypes.c_int(0), ctypes.c_int(geom.views))
    if misses < 0:
        raise MemoryError("cpu_bp_unmatched: out of host memory")
    if misses:
        raise RuntimeError(f"row block [{r0}, {r1}) does not cover slices [{z0}, {z1}): {misses} misses")
    return vol * flag, (r0, r1)
