"""Host-side geometry: detector coordinate arrays, angle arrays, filter taps and
step counts (float64), and the mct_geom / device-table bundles built from a parsed
configuration for the FBP, forward-projection and iterative-reconstruction paths.

The array-building order reproduces each reference driver, including the places
where a later call overwrites an earlier one (see fpj_geometry).
"""
import math

import numpy as np

from ._lib import MCT_CONE, MCT_CURVED, MCT_PMATRIX, MCT_SHORT_SCAN, Geom
from .config import PI, ConfigError


def angle_array(views, img_rot, scan):
    """beta_j = scan/views*j + img_rot (run_mgfbp.py:930-934)."""
    return scan / views * np.arange(views, dtype=np.float64) + img_rot


def det_positions(n_total, n_actual, d, offset, begin=0):
    """(i + begin - (n_total-1)/2)*d + offset for i < n_actual (run_mgfbp.py:937-944)."""
    return (np.arange(n_actual, dtype=np.float64) + begin - (n_total - 1) / 2.0) * d + offset


def det_positions_fpj(n, d, offset):
    """(i - (n-1)/2)*d + offset (run_mgfpj_v2.py:229-233)."""
    return (np.arange(n, dtype=np.float64) - (n - 1) / 2.0) * d + offset


def hamming_taps(nu, du, t, sdd=1.0, curved=False, dbt=False):
    """Ramp x (t + (1-t)cos) taps for n = -(nu-1)..nu-1 (run_mgfbp.py:877-914)."""
    n = np.arange(2 * nu - 1, dtype=np.int64) - (nu - 1)
    h = np.zeros(n.shape)
    odd = n % 2 != 0
    h[n == 0] = t / (4.0 * du * du)
    nf = n[odd].astype(np.float64)
    if curved:
        tv = nf * du / sdd
        h[odd] = -t / (PI * PI * sdd ** 2 * (tv - tv ** 3 / 6.0 + tv ** 5 / 120.0) ** 2)
    else:
        h[odd] = -t / (PI * PI * nf ** 2 * du ** 2)
    sgn = np.where(n % 2 == 0, 1.0, -1.0)
    p = 1.0 / (1.0 + 2.0 * n)
    q = 1.0 / (1.0 - 2.0 * n)
    h = h + (1.0 - t) * (sgn / (2 * PI * du * du) * (p + q) - (p * p + q * q) / (PI * PI * du * du))
    if dbt:
        kt = 0.02 / (2 * du)
        zero = n == 0
        h[zero] += kt ** 2
        arg = n[~zero] * du * kt * PI
        h[~zero] += (np.sin(arg) / arg) ** 2 * kt ** 2
    return h


def gaussian_taps(n_elem, d, delta):
    """exp(-n^2/(2 delta^2)) normalised to unit sum, / d (run_mgfbp.py:917-927)."""
    n = np.arange(2 * n_elem - 1, dtype=np.float64) - (n_elem - 1)
    g = np.exp(-n * n / 2.0 / delta / delta)
    with np.errstate(divide="ignore", invalid="ignore"):
        return g / g.sum() / d


def gaussian_ramp_taps(nu, du, delta, sdd, curved, dbt):
    """Gaussian-apodised ramp = du * (gauss (*) ramp) (run_mgfbp.py:1048-1060, :1265-1275)."""
    g = gaussian_taps(nu, du, delta)
    ramp = hamming_taps(nu, du, 1.0, sdd, curved, dbt)
    full = np.convolve(g, ramp)  # index i+j; the reference keeps i in [0, 2nu-2] shifted by nu-1
    return full[nu - 1:nu - 1 + 2 * nu - 1] * du


def recon_taps(obj):
    """The reconstruction kernel selected by the config (run_mgfbp.py:1261-1280)."""
    nu, du = obj.det_elem_count_horizontal, obj.det_elem_width
    if obj.kernel_name == "HammingFilter":
        return hamming_taps(nu, du, obj.kernel_param, obj.source_det_dis, obj.curved_dect, obj.dbt_or_not == 1)
    if obj.kernel_name == "GaussianApodizedRamp":
        return gaussian_ramp_taps(nu, du, obj.kernel_param, obj.source_det_dis, obj.curved_dect, obj.dbt_or_not == 1)
    raise ConfigError("ERROR: no reconstruction kernel (HammingFilter, GaussianApodizedRamp or None) in the config!")


def count_steps_v3(nx, nz, px, pz, step):
    """floor(D / (step*vd)), run_mgfpj_v3.py:252."""
    d = math.sqrt(2 * (nx * px) ** 2 + (nz * pz) ** 2)
    return int(math.floor(d / (step * math.sqrt(2 * px ** 2 + pz ** 2))))


def count_steps_ir(nx, nz, px, pz, step, sid):
    """floor((l_max - l_min) / (step*vd)), run_mgfbp_iterative_recon_IRN_CGLS.py:561-563."""
    d = (2 * (nx * px) ** 2 + (nz * pz) ** 2) ** 0.5
    l_min = sid - d / 2.0
    l_max = sid + d / 2.0
    return int(math.floor((l_max - l_min) / (step * (2 * px ** 2 + pz ** 2) ** 0.5)))


def helical_z_per_view(angles, v_arr, nv_total, pitch, sid, sdd):
    """Gantry advance per view, run_mgfpj_v3.py:242-249."""
    nb = len(angles)
    total = abs(angles[nb - 1] - angles[0]) / (nb - 1) * nb
    laps = total / (PI * 2)
    return pitch * (laps / nb) * (abs(v_arr[1] - v_arr[0]) * nv_total) / (sdd / sid)


def _flags(obj, pmatrix=False):
    f = 0
    if obj.cone_beam:
        f |= MCT_CONE
    if obj.curved_dect:
        f |= MCT_CURVED
    if obj.short_scan:
        f |= MCT_SHORT_SCAN
    if pmatrix:
        f |= MCT_PMATRIX
    return f


def _base_geom(obj):
    g = Geom()
    g.nx, g.nz = obj.img_dim, obj.img_dim_z
    g.du, g.dv = obj.det_elem_width, obj.det_elem_height
    g.px, g.pz = obj.img_pix_size, obj.img_voxel_height
    g.cx, g.cy, g.cz = obj.img_center_x, obj.img_center_y, obj.img_center_z
    g.sid, g.sdd = obj.source_isocenter_dis, obj.source_det_dis
    g.img_rot, g.total_scan_angle = obj.img_rot, obj.total_scan_angle
    g.view_mode = obj.recon_view_mode
    g.views = obj.view_num
    g.nv_total = obj.det_elem_count_vertical
    g.row_begin = obj.det_elem_vertical_recon_range_begin
    return g


def _steps(arr):
    a = np.asarray(arr, dtype=np.float64)
    return float(a[0]), float(a[1] - a[0]) if a.size > 1 else 0.0


def fbp_arrays(obj):
    """u, v and angle arrays of Mgfbp.InitializeArrays (run_mgfbp.py:1244-1259)."""
    u = det_positions(obj.det_elem_count_horizontal, obj.det_elem_count_horizontal,
                      obj.positive_u_is_positive_y * obj.det_elem_width, (-1) * obj.det_offset_horizontal, 0)
    if obj.cone_beam:
        v = det_positions(obj.det_elem_count_vertical, obj.det_elem_count_vertical_actual,
                          obj.positive_v_is_positive_z * obj.det_elem_height, obj.det_offset_vertical,
                          obj.det_elem_vertical_recon_range_begin)
    else:
        v = np.zeros(obj.det_elem_count_vertical_actual)
    angles = angle_array(obj.view_num, obj.img_rot, obj.total_scan_angle)
    return u, v, angles


def fbp_geometry(obj, device=None):
    """Geometry of the FBP/FDK path (weighting, filter, backprojection)."""
    from .ops import DeviceGeometry
    u, v, angles = fbp_arrays(obj)
    g = _base_geom(obj)
    g.nu, g.nv = obj.det_elem_count_horizontal, obj.det_elem_count_vertical_actual
    g.flags = _flags(obj, obj.bool_apply_pmatrix)
    g.u0, g.u_step = _steps(u)
    g.v0, g.v_step = _steps(v)
    pm = np.asarray(obj.array_pmatrix, dtype=np.float64) if obj.bool_apply_pmatrix else None
    dg = DeviceGeometry(g, angles, u=u, v=v, pmatrix=pm, device=device)
    dg.host = dict(u=u, v=v, angles=angles)
    return dg


def fpj_arrays(obj):
    """u, v and angle arrays as Mgfpj_v3.MainFunction leaves them (run_mgfpj_v3.py:84-91):
    the FPJ-convention arrays are written first, then Mgfbp.InitializeArrays
    overwrites the first nu entries of u, the first rows of v and the angles."""
    os_ = obj.oversample_size
    v = det_positions_fpj(obj.det_elem_count_vertical, -obj.det_elem_height, obj.det_offset_vertical)
    u = det_positions_fpj(obj.det_elem_count_horizontal * os_, -obj.det_elem_width / os_, -obj.det_offset_horizontal)
    u_fbp, v_fbp, angles = fbp_arrays(obj)
    u[:obj.det_elem_count_horizontal] = u_fbp
    v[:obj.det_elem_count_vertical_actual] = v_fbp
    return u, v, angles


def fpj_geometry(obj, device=None):
    """Geometry of the forward projector of Mgfpj_v3 (rows = actual rows, cols = nu*os)."""
    from .ops import DeviceGeometry
    u, v, angles = fpj_arrays(obj)
    g = _base_geom(obj)
    g.nu = obj.det_elem_count_horizontal * obj.oversample_size
    g.nv = obj.det_elem_count_vertical_actual
    g.flags = _flags(obj, obj.bool_apply_pmatrix)
    g.fp_steps = count_steps_v3(obj.img_dim, obj.img_dim_z, obj.img_pix_size, obj.img_voxel_height, obj.fpj_step_size)
    g.fp_step = obj.fpj_step_size
    g.fp_z_per_view = helical_z_per_view(angles, v, obj.det_elem_count_vertical, obj.helical_pitch,
                                         obj.source_isocenter_dis, obj.source_det_dis) if obj.helical_scan else 0.0
    pa = pxs = None
    if obj.bool_apply_pmatrix:
        pa, pxs = obj.matrix_A_each_view, obj.x_s_each_view
    dg = DeviceGeometry(g, angles, u=u, v=v[:obj.det_elem_count_vertical_actual], cz=obj.array_img_center_z,
                        pmat_a=pa, pmat_xs=pxs, device=device)
    dg.host = dict(u=u, v=v, angles=angles)
    return dg


def ir_arrays(obj):
    """Arrays of Mgfbp_ir.MainFunction (run_mgfbp_iterative_recon_IRN_CGLS.py:140-145):
    FPJ convention (row 0 = top, +u along -y), no later overwrite."""
    if obj.bool_uneven_scan_angle:
        angles = np.asarray(obj.array_angle, dtype=np.float64)
    else:
        angles = angle_array(obj.view_num, obj.img_rot, obj.total_scan_angle)
    v = det_positions_fpj(obj.det_elem_count_vertical, -obj.det_elem_height, obj.det_offset_vertical)
    u = det_positions_fpj(obj.det_elem_count_horizontal * obj.oversample_size,
                          -obj.det_elem_width / obj.oversample_size, -obj.det_offset_horizontal)
    return u, v, angles


def ir_geometry(obj, device=None):
    """Geometry shared by the IR forward projector, effective map and backprojectors."""
    from .ops import DeviceGeometry
    if obj.det_elem_count_vertical_actual != obj.det_elem_count_vertical:
        raise ConfigError("ERROR: DetectorElementVerticalReconRange is not supported by iterative reconstruction "
                          "(the reference's per-view buffers assume the full detector)")
    if obj.bool_apply_pmatrix:
        raise ConfigError("ERROR: PMatrixFile is not supported by iterative reconstruction")
    u, v, angles = ir_arrays(obj)
    g = _base_geom(obj)
    g.nu = obj.det_elem_count_horizontal
    g.nv = obj.det_elem_count_vertical_actual
    g.flags = _flags(obj, False)
    g.fp_steps = count_steps_ir(obj.img_dim, obj.img_dim_z, obj.img_pix_size, obj.img_voxel_height,
                                obj.fpj_step_size, obj.source_isocenter_dis)
    g.fp_step = obj.fpj_step_size
    g.fp_z_per_view = helical_z_per_view(angles, v, obj.det_elem_count_vertical, obj.helical_pitch,
                                         obj.source_isocenter_dis, obj.source_det_dis) if obj.helical_scan else 0.0
    g.u0, g.u_step = _steps(u)
    g.v0, g.v_step = _steps(v)
    dg = DeviceGeometry(g, angles, u=u[:obj.det_elem_count_horizontal], v=v[:g.nv], cz=obj.array_img_center_z,
                        device=device)
    dg.host = dict(u=u, v=v, angles=angles)
    return dg


def fpj_v2_arrays(obj):
    """Mgfpj.MainFunction (run_mgfpj_v2.py:70-110) only runs Mgfbp.InitializeArrays:
    the first nu entries of the (nu*oversample)-long u table hold the FBP u array,
    the rest stay 0; v and the angles are the FBP arrays."""
    u_fbp, v, angles = fbp_arrays(obj)
    u = np.zeros(obj.det_elem_count_horizontal * obj.oversample_size)
    u[:obj.det_elem_count_horizontal] = u_fbp
    return u, v, angles


def fpj_v1_arrays(obj):
    """Mgfpj.MainFunction of run_mgfpj.py:57-66: FPJ-convention u and v (row 0 =
    top) and angles from StartAngle."""
    angles = angle_array(obj.view_num, obj.start_angle, obj.scan_angle)
    v = det_positions_fpj(obj.det_elem_count_vertical, -obj.det_elem_height, obj.det_offset_vertical)
    u = det_positions_fpj(obj.det_elem_count_horizontal * obj.oversample_size,
                          -obj.det_elem_width / obj.oversample_size, -obj.det_offset_horizontal)
    return u, v, angles


def fpj_variant_geometry(obj, version, device=None):
    """Forward-projector geometry of run_mgfpj.py (version 1) or run_mgfpj_v2.py
    (version 2): step count (l_max - l_min)/(step*vd) and one image centre z."""
    from .ops import DeviceGeometry
    u, v, angles = fpj_v1_arrays(obj) if version == 1 else fpj_v2_arrays(obj)
    g = _base_geom(obj)
    g.nu = obj.det_elem_count_horizontal * obj.oversample_size
    g.nv = obj.det_elem_count_vertical_actual
    g.flags = _flags(obj, obj.bool_apply_pmatrix)
    g.fp_steps = count_steps_ir(obj.img_dim, obj.img_dim_z, obj.img_pix_size, obj.img_voxel_height,
                                obj.fpj_step_size, obj.source_isocenter_dis)
    g.fp_step = obj.fpj_step_size
    g.fp_z_per_view = helical_z_per_view(angles, v, obj.det_elem_count_vertical, obj.helical_pitch,
                                         obj.source_isocenter_dis, obj.source_det_dis) if obj.helical_scan else 0.0
    pa = pxs = None
    if obj.bool_apply_pmatrix:
        pa, pxs = obj.matrix_A_each_view, obj.x_s_each_view
    dg = DeviceGeometry(g, angles, u=u, v=v[:g.nv], pmat_a=pa, pmat_xs=pxs, device=device)
    dg.host = dict(u=u, v=v, angles=angles)
    return dg
