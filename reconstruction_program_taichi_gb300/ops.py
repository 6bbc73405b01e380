"""Device operators over torch CUDA tensors, each a thin call into the C ABI
(include/mandoct_gb300.h) on the current CUDA stream.

Tensors are float32 and C-contiguous.  Sinograms are [rows, views, cols] and volumes
[z, y, x], the reference's layouts; the filtered sinogram handed from the filter to
the backprojector is view-major [views, rows, cols] and is then packed into the
backprojector's gather layout.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import MCT_BF16, MCT_CONE, MCT_F16, MCT_F32, Geom, Tables


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


_VEC = {torch.float32: MCT_F32, torch.bfloat16: MCT_BF16}


def _vec_dtype(t, name, shape=None):
    """MCT_F32 / MCT_BF16 of a float32 or bf16 volume (bf16 CG iterates)."""
    if not isinstance(t, torch.Tensor) or t.dtype not in _VEC:
        raise TypeError(f"{name} must be a float32 or bfloat16 CUDA tensor")
    _check(t, name, shape, dtype=t.dtype)
    return _VEC[t.dtype]


def _check(t, name, shape=None, dtype=torch.float32):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {tuple(shape)}")


class DeviceGeometry:
    """An mct_geom plus its device tables (angles, u, v, per-view z centre, matrices)."""

    def __init__(self, geom, angles, u=None, v=None, cz=None, pmatrix=None, pmat_a=None, pmat_xs=None,
                 device=None):
        self.geom = geom
        dev = torch.device(device or "cuda")
        self._keep = {}

        def up(name, arr):
            if arr is None:
                return None
            t = torch.as_tensor(np.ascontiguousarray(np.asarray(arr, dtype=np.float64)).astype(np.float32),
                                device=dev).contiguous()
            self._keep[name] = t
            return t.data_ptr()

        self.tables = Tables(angles=up("angles", angles), u=up("u", u), v=up("v", v), cz=up("cz", cz),
                             pmatrix=up("pmatrix", pmatrix), pmat_a=up("pmat_a", pmat_a),
                             pmat_xs=up("pmat_xs", pmat_xs))
        self.device = dev

    @property
    def sgm_shape(self):
        g = self.geom
        return (g.nv, g.views, g.nu)

    @property
    def vol_shape(self):
        g = self.geom
        return (g.nz, g.nx, g.nx)

    def g(self):
        return ctypes.byref(self.geom)

    def t(self):
        return ctypes.byref(self.tables)


class ViewChunk:
    """Views [view_begin, view_begin + views) of a DeviceGeometry for view-chunked FBP:
    the whole scan's device tables with a geometry whose views / view_begin /
    views_total select the range (mct_weight, mct_filter, mct_pack and mct_fdk_bp
    accept it; accumulate=True adds the backprojection to the volume)."""

    def __init__(self, dg, view_begin, views, accumulate=False):
        g = dg.geom
        if not (0 <= view_begin and views >= 1 and view_begin + views <= g.views):
            raise ValueError("view chunk outside the scan")
        self.geom = g.copy(views=views, view_begin=view_begin, views_total=g.views,
                           flags=g.flags | (_lib.MCT_ACCUMULATE if accumulate else 0))
        self.tables = dg.tables
        self.device = dg.device
        self._parent = dg  # keeps the tables alive

    sgm_shape = DeviceGeometry.sgm_shape
    vol_shape = DeviceGeometry.vol_shape
    g = DeviceGeometry.g
    t = DeviceGeometry.t


def fdk_bp_finish(dg, vol):
    """Write the voxels that left the detector in some chunk as 0 (after the last
    chunk of a view-chunked FBP)."""
    _check(vol, "vol", dg.vol_shape)
    _lib.call("mct_fdk_bp_finish", dg.g(), _ptr(vol), _stream())
    return vol


# ---------------------------------------------------------------- FBP / FDK

def strided_extent(nv, views, nu, row_stride, view_stride):
    """Elements a strided sinogram must hold: element (row, view, col) sits at
    row*row_stride + view*view_stride + col.  Raises on negative strides."""
    row_stride, view_stride = int(row_stride), int(view_stride)
    if row_stride < 0 or view_stride < 0:
        raise ValueError("sinogram strides must be non-negative")
    return (nv - 1) * row_stride + (views - 1) * view_stride + nu


def _check_strided(sgm, g, row_stride, view_stride):
    """The strided sinogram must lie inside sgm: the kernels read every element."""
    _check(sgm, "sgm")
    last = strided_extent(g.nv, g.views, g.nu, row_stride, view_stride)
    if last > sgm.numel():
        raise ValueError(f"sgm holds {sgm.numel()} elements; strides ({row_stride}, {view_stride}) over "
                         f"{g.nv} rows x {g.views} views x {g.nu} columns address {last}")
    return int(row_stride), int(view_stride)


def weight(dg, sgm, row_stride, view_stride, bh=None, out=None):
    """BH polynomial + cosine (+ Parker) weighting into [nv, views, nu]."""
    row_stride, view_stride = _check_strided(sgm, dg.geom, row_stride, view_stride)
    if out is None:
        out = torch.empty(dg.sgm_shape, dtype=torch.float32, device=sgm.device)
    _check(out, "out", dg.sgm_shape)
    n_bh = 0
    if bh is not None:
        _check(bh, "bh")
        n_bh = bh.numel()
    _lib.call("mct_weight", dg.g(), dg.t(), _ptr(sgm), row_stride, view_stride, _ptr(bh), n_bh, _ptr(out), _stream())
    return out


def vgauss(dg, weighted, taps, out=None):
    _check(weighted, "weighted", dg.sgm_shape)
    _check(taps, "taps", (2 * dg.geom.nv - 1,))
    if out is None:
        out = torch.empty_like(weighted)
    _lib.call("mct_vgauss", dg.g(), _ptr(weighted), _ptr(taps), _ptr(out), _stream())
    return out


def filter_rows(dg, weighted, taps, out=None):
    """Toeplitz row filter; returns the view-major filtered sinogram [views, nv, nu]."""
    g = dg.geom
    _check(weighted, "weighted", dg.sgm_shape)
    _check(taps, "taps", (2 * g.nu - 1,))
    if out is None:
        out = torch.empty((g.views, g.nv, g.nu), dtype=torch.float32, device=weighted.device)
    _check(out, "out", (g.views, g.nv, g.nu))
    _lib.call("mct_filter", dg.g(), _ptr(weighted), _ptr(taps), _ptr(out), _stream())
    return out


class TcFilter:
    """Tensor-core row filter for one geometry and one set of taps: owns the tiled
    operand workspace (A and B^T part tiles, 1 KiB aligned).  dtype MCT_F32: three bf16
    parts (~1e-6); MCT_BF16: two parts (~1e-5)."""

    def __init__(self, dg, taps, dtype=MCT_BF16):
        g = dg.geom
        _check(taps, "taps", (2 * g.nu - 1,))
        self.dtype = int(dtype)
        n = int(_lib.load().mct_filter_tc_workspace_size(dg.g(), self.dtype))
        self.dg = dg
        self._buf = torch.empty(n + 1024, dtype=torch.uint8, device=dg.device)
        off = (-self._buf.data_ptr()) % 1024
        self.ws = ctypes.c_void_p(self._buf.data_ptr() + off)
        _lib.call("mct_filter_tc_prepare", dg.g(), _ptr(taps), self.dtype, self.ws, _stream())

    def __call__(self, weighted, out=None):
        g = self.dg.geom
        _check(weighted, "weighted", self.dg.sgm_shape)
        if out is None:
            out = torch.empty((g.views, g.nv, g.nu), dtype=torch.float32, device=weighted.device)
        _check(out, "out", (g.views, g.nv, g.nu))
        _lib.call("mct_filter_tc", self.dg.g(), _ptr(weighted), self.dtype, self.ws, _ptr(out), _stream())
        return out

    def weight_filter(self, sgm, row_stride, view_stride, bh=None, out=None, dg=None):
        """Weighting (BH, cosine, Parker) and this filter in one pass over the sinogram:
        the weighting runs while the operand is split, the weighted float32 sinogram is
        never written (mct_weight_filter).  Same result as weight() then __call__.  dg:
        the geometry to weight for, when it is another view chunk of the same size as
        the one this filter was built for (the weights depend on the chunk's views)."""
        dg = self.dg if dg is None else dg
        g = dg.geom
        if (g.nv, g.views, g.nu) != (self.dg.geom.nv, self.dg.geom.views, self.dg.geom.nu):
            raise ValueError("the geometry's sinogram size differs from this filter's")
        row_stride, view_stride = _check_strided(sgm, g, row_stride, view_stride)
        if out is None:
            out = torch.empty((g.views, g.nv, g.nu), dtype=torch.float32, device=sgm.device)
        _check(out, "out", (g.views, g.nv, g.nu))
        n_bh = 0
        if bh is not None:
            _check(bh, "bh")
            n_bh = bh.numel()
        _lib.call("mct_weight_filter", dg.g(), dg.t(), _ptr(sgm), int(row_stride), int(view_stride),
                  _ptr(bh), n_bh, self.dtype, self.ws, _ptr(out), _stream())
        return out

    def status(self):
        """Raise if a bounded pipeline wait of an earlier launch timed out (syncs)."""
        _lib.call("mct_filter_tc_status", self.dg.g(), self.dtype, self.ws, _stream())


def packed_bytes(dg, dtype=MCT_F32):
    return int(_lib.load().mct_packed_size(dg.g(), dtype))


def pack(dg, filtered, dtype=MCT_F32, out=None):
    g = dg.geom
    _check(filtered, "filtered", (g.views, g.nv, g.nu))
    nbytes = packed_bytes(dg, dtype)
    if out is None:
        out = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=filtered.device)
    if out.numel() < nbytes:
        raise ValueError("packed buffer too small")
    _lib.call("mct_pack", dg.g(), _ptr(filtered), _ptr(out), dtype, _stream())
    return out


def pack_sinogram(dg, sgm, dtype=MCT_F32, out=None):
    """Pack a [nv, views, nu] sinogram into the one-gather stencil layout."""
    g = dg.geom
    _check(sgm, "sgm", dg.sgm_shape)
    nbytes = packed_bytes(dg, dtype)
    if out is None:
        out = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=sgm.device)
    if out.numel() < nbytes:
        raise ValueError("packed buffer too small")
    _lib.call("mct_pack_strided", dg.g(), _ptr(sgm), g.views * g.nu, g.nu, _ptr(out), dtype, _stream())
    return out


def bp_unmatched_packed(dg, packed, dtype=MCT_F32, out=None):
    """The IR driver's backprojector of a packed sinogram; out may be bf16 (axial cone
    beam), rounded from the float32 sums."""
    if out is None:
        out = torch.empty(dg.vol_shape, dtype=torch.float32, device=packed.device)
    odt = _vec_dtype(out, "out", dg.vol_shape)
    if odt == MCT_F32:
        _lib.call("mct_bp_ref_unmatched_packed", dg.g(), dg.t(), _ptr(packed), dtype, _ptr(out), _stream())
    else:
        _lib.call("mct_bp_ref_unmatched_packed_out", dg.g(), dg.t(), _ptr(packed), dtype, _ptr(out), odt, _stream())
    return out


def fdk_bp(dg, packed, dtype=MCT_F32, out=None):
    if out is None:
        out = torch.empty(dg.vol_shape, dtype=torch.float32, device=packed.device)
    _check(out, "out", dg.vol_shape)
    _lib.call("mct_fdk_bp", dg.g(), dg.t(), _ptr(packed), dtype, _ptr(out), _stream())
    return out


# ---------------------------------------------------------------- forward projection

def fp_workspace(dg, dtype=MCT_F32):
    """Per-geometry workspace of fp() (the gather copies of the volume), cached per
    storage type.  It belongs to the geometry object: calls that share one geometry
    must be ordered on one stream, or pass workspaces of their own."""
    cache = dg.__dict__.setdefault("_fp_ws", {})
    ws = cache.get(int(dtype))
    if ws is None:
        n = int(_lib.load().mct_fp_storage_workspace_size(dg.g(), int(dtype)))
        if n == 0:
            raise ValueError("this storage type needs a cone-beam geometry")
        ws = torch.empty(max(n // 4, 1), dtype=torch.float32, device=dg.device)
        cache[int(dtype)] = ws
    return ws


def fp(dg, vol, mask=None, out=None, workspace=True, dtype=MCT_F32):
    """P vol.  workspace=True uses the geometry's cached gather-copy buffer (coalesced
    gathers for every view); None runs without it.  dtype=MCT_BF16 or MCT_F16 (cone
    beam) stores the gather copies as 16-bit cells (mct_fp_storage).  vol may be bf16
    (bf16 iterates; cone beam with the workspace)."""
    vdt = _vec_dtype(vol, "vol", dg.vol_shape)
    if mask is not None:
        _check(mask, "mask", dg.sgm_shape)
    if out is None:
        out = torch.empty(dg.sgm_shape, dtype=torch.float32, device=vol.device)
    _check(out, "out", dg.sgm_shape)
    ws = fp_workspace(dg, dtype) if workspace is True else workspace
    if vdt != MCT_F32:
        _lib.call("mct_fp_storage_in", dg.g(), dg.t(), _ptr(vol), vdt, _ptr(mask), _ptr(out), _ptr(ws), int(dtype),
                  _stream())
    elif dtype == MCT_F32:
        _lib.call("mct_fp", dg.g(), dg.t(), _ptr(vol), _ptr(mask), _ptr(out), _ptr(ws), _stream())
    else:
        _lib.call("mct_fp_storage", dg.g(), dg.t(), _ptr(vol), _ptr(mask), _ptr(out), _ptr(ws), int(dtype), _stream())
    return out


def fp_adjoint_workspace(dg):
    """Per-geometry cell-space buffer of fp_adjoint() (cached; like fp_workspace() it
    belongs to the geometry object, so calls sharing a geometry stay on one stream)."""
    ws = dg.__dict__.get("_adj_ws")
    if ws is None:
        n = int(_lib.load().mct_fp_adjoint_workspace_size(dg.g()))
        ws = torch.empty(max(n // 4, 4), dtype=torch.float32, device=dg.device)
        dg.__dict__["_adj_ws"] = ws
    return ws


def fp_adjoint(dg, sgm, mask=None, out=None, accumulate=False, workspace=True):
    """P^T sgm, the exact transpose of fp().  workspace=True scatters through the
    geometry's cached cell-space buffer (mct_fp_adjoint_cells); None scatters the 8
    corner weights straight into the volume (mct_fp_adjoint)."""
    _check(sgm, "sgm", dg.sgm_shape)
    if mask is not None:
        _check(mask, "mask", dg.sgm_shape)
    if out is None:
        out = torch.zeros(dg.vol_shape, dtype=torch.float32, device=sgm.device)
    elif not accumulate:
        out.zero_()
    _check(out, "out", dg.vol_shape)
    ws = fp_adjoint_workspace(dg) if workspace is True else workspace
    if ws is None:
        _lib.call("mct_fp_adjoint", dg.g(), dg.t(), _ptr(sgm), _ptr(mask), _ptr(out), _stream())
    else:
        _lib.call("mct_fp_adjoint_cells", dg.g(), dg.t(), _ptr(sgm), _ptr(mask), _ptr(out), _ptr(ws), _stream())
    return out


def fp_count_samples(dg, mask=None):
    """Number of in-volume trilinear samples of fp() (int)."""
    out = torch.zeros(1, dtype=torch.int64, device=dg.device)
    _lib.call("mct_fp_count_samples", dg.g(), dg.t(), _ptr(mask), _ptr(out), _stream())
    return int(out.item())


def effective_map(dg, out=None):
    if out is None:
        out = torch.empty(dg.sgm_shape, dtype=torch.float32, device=dg.device)
    _check(out, "out", dg.sgm_shape)
    _lib.call("mct_effective_map", dg.g(), dg.t(), _ptr(out), _stream())
    return out


def bin_noise(dg, sgm_large, bin_size, photons=0.0, seed=0, out=None):
    """[nv, views, nu*bin] -> [nv, views, nu] with optional photon noise."""
    g = dg.geom
    _check(sgm_large, "sgm_large", (g.nv, g.views, g.nu * bin_size))
    if out is None:
        out = torch.empty((g.nv, g.views, g.nu), dtype=torch.float32, device=sgm_large.device)
    _check(out, "out", (g.nv, g.views, g.nu))
    _lib.call("mct_bin_noise", dg.g(), _ptr(sgm_large), bin_size, float(photons), int(seed) & (2 ** 64 - 1),
              _ptr(out), _stream())
    return out


def project_ellipsoids(dg, ell, out=None):
    """Analytic line integrals of ellipsoids ([n, 10] rows) along the projector's rays."""
    ell = torch.as_tensor(np.asarray(ell, dtype=np.float32), device=dg.device).contiguous()
    if out is None:
        out = torch.empty(dg.sgm_shape, dtype=torch.float32, device=dg.device)
    _check(out, "out", dg.sgm_shape)
    _lib.call("mct_project_ellipsoids", dg.g(), dg.t(), _ptr(ell), int(ell.shape[0]), _ptr(out), _stream())
    return out


# ---------------------------------------------------------------- iterative reconstruction

def bp_unmatched(dg, sgm, out=None):
    _check(sgm, "sgm", dg.sgm_shape)
    if out is None:
        out = torch.empty(dg.vol_shape, dtype=torch.float32, device=sgm.device)
    _check(out, "out", dg.vol_shape)
    _lib.call("mct_bp_ref_unmatched", dg.g(), dg.t(), _ptr(sgm), _ptr(out), _stream())
    return out


def bp_unmatched_packed_cg(dg, packed, dtype, d, terms, q, dq_out):
    """One CG operator application with the vector work in the backprojector's
    epilogue: q = P^T p + sum_t s_t D^T W_t D d (terms: up to two (s, W) pairs, added in
    order) and dq_out = <d, q> (float64 device scalar) over the stored q.  Axial view
    mode, cone beam; d and q both float32 or both bf16, each W float32."""
    vdt = _vec_dtype(d, "d", dg.vol_shape)
    if _vec_dtype(q, "q", dg.vol_shape) != vdt:
        raise TypeError("q must have the dtype of d")
    if len(terms) > 2:
        raise ValueError("at most two D^T W D terms")
    ws = [None, None]
    ss = [0.0, 0.0]
    for k, (sk, wk) in enumerate(terms):
        _check(wk, "W", dg.vol_shape)
        ws[k], ss[k] = wk, float(sk)
    part = dg.__dict__.get("_cg_partials")
    if part is None:
        n = int(_lib.load().mct_bp_cg_partials_size(dg.g())) // 8
        part = torch.empty(max(n, 1), dtype=torch.float64, device=dg.device)
        dg.__dict__["_cg_partials"] = part
    _lib.call("mct_bp_ref_unmatched_packed_cg", dg.g(), dg.t(), _ptr(packed), int(dtype), _ptr(d), _ptr(ws[0]), ss[0],
              _ptr(ws[1]), ss[1], _ptr(q), vdt, _ptr(part), _ptr(dq_out), _stream())
    return q


def tv_weights(dg, x, beta, out=None):
    """WR = 1/sqrt(|D x|^2 + beta) as float32; x float32 or bf16."""
    xdt = _vec_dtype(x, "x", dg.vol_shape)
    if out is None:
        out = torch.empty(dg.vol_shape, dtype=torch.float32, device=x.device)
    _check(out, "out", dg.vol_shape)
    if xdt == MCT_F32:
        _lib.call("mct_tv_weights", dg.g(), _ptr(x), float(beta), _ptr(out), _stream())
    else:
        _lib.call("mct_tv_weights_t", dg.g(), _ptr(x), xdt, float(beta), _ptr(out), _stream())
    return out


def dtwd(dg, x, wr, s=1.0, out_in=None, a=0.0, out=None):
    """out = a*out_in + s * D^T W D x (x, out_in, out all float32 or all bf16; wr float32)."""
    xdt = _vec_dtype(x, "x", dg.vol_shape)
    _check(wr, "wr", dg.vol_shape)
    if out is None:
        out = torch.empty_like(x)
    if xdt == MCT_F32:
        _lib.call("mct_dtwd", dg.g(), _ptr(x), _ptr(wr), float(s), _ptr(out_in), float(a), _ptr(out), _stream())
    else:
        for t, n in ((out, "out"), (out_in, "out_in")):
            if t is not None and _vec_dtype(t, n, dg.vol_shape) != xdt:
                raise TypeError(f"{n} must have the dtype of x")
        _lib.call("mct_dtwd_t", dg.g(), _ptr(x), _ptr(wr), float(s), _ptr(out_in), float(a), _ptr(out), xdt, None,
                  None, _stream())
    return out


def dtwd_dot(dg, x, wr, s, acc, dot_out):
    """acc += s * D^T W D x (in place) and dot_out = <x, acc> (float64 device scalar),
    in one pass (x and acc float32 or both bf16)."""
    xdt = _vec_dtype(x, "x", dg.vol_shape)
    _check(wr, "wr", dg.vol_shape)
    if _vec_dtype(acc, "acc", dg.vol_shape) != xdt:
        raise TypeError("acc must have the dtype of x")
    if xdt == MCT_F32:
        _lib.call("mct_dtwd_dot", dg.g(), _ptr(x), _ptr(wr), float(s), _ptr(acc), 1.0, _ptr(acc),
                  _ptr(reduce_scratch(x.device)), _ptr(dot_out), _stream())
    else:
        _lib.call("mct_dtwd_t", dg.g(), _ptr(x), _ptr(wr), float(s), _ptr(acc), 1.0, _ptr(acc), xdt,
                  _ptr(reduce_scratch(x.device)), _ptr(dot_out), _stream())
    return dot_out


_scratch = {}


def reduce_scratch(device):
    key = (str(device), torch.cuda.current_stream(device).cuda_stream)
    t = _scratch.get(key)
    if t is None:
        n = int(_lib.load().mct_reduce_scratch_size()) // 8
        t = torch.empty(n, dtype=torch.float64, device=device)
        _scratch[key] = t
    return t


def tv_penalty(dg, x, beta, out=None):
    """sum sqrt(|D x|^2 + beta) as a float64 device scalar."""
    _check(x, "x", dg.vol_shape)
    if out is None:
        out = torch.empty((), dtype=torch.float64, device=x.device)
    _lib.call("mct_tv_penalty", dg.g(), _ptr(x), float(beta), _ptr(reduce_scratch(x.device)), _ptr(out), _stream())
    return out


def dot(a, b, out=None):
    """float64 inner product of two float32 (or two bf16) tensors, as a device scalar."""
    adt = _vec_dtype(a, "a")
    if _vec_dtype(b, "b", tuple(a.shape)) != adt:
        raise TypeError("a and b must have the same dtype")
    if out is None:
        out = torch.empty((), dtype=torch.float64, device=a.device)
    if adt == MCT_F32:
        _lib.call("mct_dot_f64", _ptr(a), _ptr(b), a.numel(), _ptr(reduce_scratch(a.device)), _ptr(out), _stream())
    else:
        _lib.call("mct_dot_f64_t", _ptr(a), _ptr(b), a.numel(), adt, _ptr(reduce_scratch(a.device)), _ptr(out),
                  _stream())
    return out


def _same_vec_dtype(*ts):
    dts = {_vec_dtype(t, "vector") for t in ts}
    if len(dts) != 1:
        raise TypeError("CG vectors must share one dtype (float32 or bfloat16)")
    return dts.pop()


def cgls_update(rr, dq, x, r, d, q, rr_new):
    """alpha = rr/dq; x += alpha d; r -= alpha q; rr_new = |r|^2 (device scalars)."""
    vdt = _same_vec_dtype(x, r, d, q)
    if vdt == MCT_F32:
        _lib.call("mct_cgls_update", x.numel(), _ptr(rr), _ptr(dq), _ptr(x), _ptr(r), _ptr(d), _ptr(q),
                  _ptr(reduce_scratch(x.device)), _ptr(rr_new), _stream())
    else:
        _lib.call("mct_cgls_update_t", x.numel(), vdt, _ptr(rr), _ptr(dq), _ptr(x), _ptr(r), _ptr(d), _ptr(q),
                  _ptr(reduce_scratch(x.device)), _ptr(rr_new), _stream())


def cgls_direction(rr, rr_new, r, d):
    """d = r + (rr_new/rr) d."""
    vdt = _same_vec_dtype(r, d)
    if vdt == MCT_F32:
        _lib.call("mct_cgls_direction", d.numel(), _ptr(rr), _ptr(rr_new), _ptr(r), _ptr(d), _stream())
    else:
        _lib.call("mct_cgls_direction_t", d.numel(), vdt, _ptr(rr), _ptr(rr_new), _ptr(r), _ptr(d), _stream())
