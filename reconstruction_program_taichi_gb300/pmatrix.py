"""Projection-matrix (PMatrixFile) geometry: reading, normalisation to the standard
circular trajectory, pixel-size and row-range adjustment, and the per-view
(A = inv(P[:, :3]), source position) pairs used by the forward projector.

Host-side float64 math following run_mgfbp.py:549-627 and :721-874 and
run_mgfpj_v2.py:218-227.  The 3x4 matrices map (x, y, z, 1) to homogeneous
detector coordinates (u, v, 1) in pixel units.
"""
import math

import numpy as np

from .config import PI, ConfigError, load_jsonc, save_jsonc


def _lstsq(B, y):
    """x = (B^T B)^-1 B^T y, run_mgfbp.py:1351-1355."""
    return np.linalg.inv(B.T @ B) @ B.T @ y


def apply_pmatrix_config(self, cfg):
    """PMatrixFile branch of the cone-beam configuration, run_mgfbp.py:549-627."""
    d = load_jsonc(cfg["PMatrixFile"])
    if "Value" not in d:
        raise ConfigError("ERROR: PMatrixFile has no member named 'Value'!")
    pm = d["Value"]
    if not isinstance(pm, list):
        raise ConfigError("ERROR: PMatrixFile.Value is not an array")
    if len(pm) != self.view_num * 12:
        raise ConfigError(f"ERROR: view number is {self.view_num:d} while pmatrix has {len(pm):d} elements!")
    # float32 storage, as the reference keeps it (updates round to float32)
    self.array_pmatrix = np.array(pm, dtype=np.float32)
    self.bool_apply_pmatrix = True
    mod = cfg.get("ModifyPMatrixToStandardForm", False)
    if not isinstance(mod, bool):
        raise ConfigError("ERROR: ModifyPMatrixToStandardForm must be True or False!")
    self.modify_pmatrix_to_standard_form = mod
    for key, attr, base in (("PMatrixDetectorElementWidth", "pmatrix_elem_width", self.det_elem_width),
                            ("PMatrixDetectorElementHeight", "pmatrix_elem_height", self.det_elem_height)):
        if key in cfg:
            val = cfg[key]
            if not isinstance(val, (float, int)):
                raise ConfigError(f"ERROR: {key} must be a number!")
            if val <= 0:
                raise ConfigError(f"ERROR: {key} must be positive!")
            setattr(self, attr, val)
        else:
            setattr(self, attr, base)
    change_source_trajectory(self)
    cfg["SourceIsocenterDistance"] = self.source_isocenter_dis
    cfg["SourceDetectorDistance"] = self.source_det_dis
    cfg["DetectorOffsetHorizontal"] = self.det_offset_horizontal
    cfg["DetectorOffsetVertical"] = self.det_offset_vertical
    cfg["TotalScanAngle"] = self.total_scan_angle / PI * 180.0
    change_pixel_size(self)
    change_vertical_recon_range(self)


def _views(pm, n):
    for j in range(n):
        yield j, pm[12 * j:12 * j + 12].reshape(3, 4)


def change_source_trajectory(self):
    """Fit the source circle, optionally rotate it to the standard form, and derive
    SID, SDD, offsets and the scan angle; run_mgfbp.py:721-839."""
    n = self.view_num
    xs = np.zeros((3, n))
    for j, P in _views(self.array_pmatrix, n):
        A = np.linalg.inv(P[:, :3])
        xs[:, j] = -(A @ P[:, 3])
    sol = _lstsq(xs.T, np.ones((n, 1)))
    ang_y = float(np.arctan(sol[0] / sol[2])[0])
    ang_x = float((np.arctan(sol[1] / np.sqrt(sol[0] ** 2 + sol[2] ** 2)) * np.sign(sol[2]))[0])
    Ry = np.array([[math.cos(ang_y), 0, -math.sin(ang_y)], [0, 1, 0], [math.sin(ang_y), 0, math.cos(ang_y)]])
    Rx = np.array([[1, 0, 0], [0, math.cos(ang_x), -math.sin(ang_x)], [0, math.sin(ang_x), math.cos(ang_x)]])
    xs_rot = Rx @ (Ry @ xs)
    zc = np.mean(xs_rot[2, :])
    xy = xs_rot[0:2, :]
    B = np.concatenate((-xy.T, np.ones((n, 1))), axis=1)
    sol2 = _lstsq(B, -np.sum(xy ** 2, axis=0))
    shifted = xs_rot - np.array([[sol2[0] / 2], [sol2[1] / 2], [zc]])
    ang_z = math.atan2(shifted[1, 0], shifted[0, 0])
    Rz = np.array([[math.cos(ang_z), math.sin(ang_z), 0], [-math.sin(ang_z), math.cos(ang_z), 0], [0, 0, 1]])
    xs_final = Rz @ shifted
    R_total = Rz @ (Rx @ Ry)
    if not self.modify_pmatrix_to_standard_form:
        R_total = np.eye(3)
        xs_final = xs
    v_center = np.zeros((n, 1))
    u_center = np.zeros((n, 1))
    scan_sum = 0.0
    self.scan_angle_each_view = np.zeros((n, 1))
    xd_c = np.zeros((3, n))
    for j, P in _views(self.array_pmatrix, n):
        A = np.linalg.inv(P[:, :3])
        ratio = (self.pmatrix_elem_width / np.linalg.norm(A[:, 0]) + self.pmatrix_elem_height / np.linalg.norm(A[:, 1])) * 0.5
        P = P / ratio
        A = np.linalg.inv(P[:, :3])
        x_s = xs_final[:, j:j + 1]
        if j <= n - 2:
            nxt = xs_final[:, j + 1:j + 2]
            da = math.atan2(nxt[1, 0], nxt[0, 0]) - math.atan2(x_s[1, 0], x_s[0, 0])
            if abs(da) > PI:
                da = da - 2 * PI * np.sign(da)
            scan_sum = scan_sum + da
            self.scan_angle_each_view[j + 1, 0] = scan_sum / PI * 180.0
        e_v = R_total @ A[:, 1]
        e_u = R_total @ A[:, 0]
        if j == 0:
            self.positive_u_is_positive_y = np.sign(e_u[1])
            self.positive_v_is_positive_z = np.sign(e_v[2])
        xdo = R_total @ A[:, 2]
        A2 = np.stack([e_u, e_v, xdo], axis=1)
        Ainv = np.linalg.inv(A2)
        Pn = np.append(Ainv, -(Ainv @ x_s), axis=1)
        u_center[j, 0] = Pn[0, 3] / Pn[2, 3]
        v_center[j, 0] = -np.dot(xdo, e_v) / (self.pmatrix_elem_height ** 2)
        xd_c[:, j:j + 1] = xdo.reshape(3, 1) + u_center[j, 0] * e_u.reshape(3, 1) + v_center[j, 0] * e_v.reshape(3, 1)
        self.array_pmatrix[12 * j:12 * j + 12] = Pn.reshape(12)
    self.det_offset_vertical_each_view = self.positive_v_is_positive_z * (
        (self.det_elem_count_vertical * self.det_elem_height / self.pmatrix_elem_height - 1) / 2.0 - v_center) \
        * self.pmatrix_elem_height
    self.det_offset_horizontal_each_view = -self.positive_u_is_positive_y * (
        (self.det_elem_count_horizontal * self.det_elem_width / self.pmatrix_elem_width - 1) / 2.0 - u_center) \
        * self.pmatrix_elem_width
    self.det_offset_vertical = float(np.squeeze(np.mean(self.det_offset_vertical_each_view, axis=0)))
    self.det_offset_horizontal = float(np.squeeze(np.mean(self.det_offset_horizontal_each_view, axis=0)))
    self.source_isocenter_dis_each_view = np.sqrt(np.sum(xs_final * xs_final, axis=0))
    self.source_det_dis_each_view = np.sqrt(np.sum(xd_c * xd_c, axis=0))
    self.source_isocenter_dis = float(np.mean(self.source_isocenter_dis_each_view))
    self.source_det_dis = float(np.mean(self.source_det_dis_each_view))
    if self.short_scan:
        self.total_scan_angle = scan_sum / (n - 1) * n


def change_pixel_size(self):
    """Rescale matrices to the scan's detector pixel size, run_mgfbp.py:841-858
    (including its use of e_v_0 in the u correction term)."""
    for j, P in _views(self.array_pmatrix, self.view_num):
        A = np.linalg.inv(P[:, :3])
        x_s = -(A @ P[:, 3]).reshape(3, 1)
        e_v0, e_u0 = A[:, 1].copy(), A[:, 0].copy()
        e_v = e_v0 * self.det_elem_height / self.pmatrix_elem_height
        e_u = e_u0 * self.det_elem_width / self.pmatrix_elem_width
        xdo = A[:, 2] + 0.5 * (e_v - e_v0) + 0.5 * (e_u - e_v0)
        A2 = np.stack([e_u, e_v, xdo], axis=1)
        Ainv = np.linalg.inv(A2)
        self.array_pmatrix[12 * j:12 * j + 12] = np.append(Ainv, -(Ainv @ x_s), axis=1).reshape(12)


def change_vertical_recon_range(self):
    """Shift the detector origin to the first reconstructed row, run_mgfbp.py:860-874."""
    for j, P in _views(self.array_pmatrix, self.view_num):
        A = np.linalg.inv(P[:, :3])
        x_s = -(A @ P[:, 3]).reshape(3, 1)
        A[:, 2] = A[:, 2] + self.det_elem_vertical_recon_range_begin * A[:, 1]
        Ainv = np.linalg.inv(A)
        self.array_pmatrix[12 * j:12 * j + 12] = np.append(Ainv, -(Ainv @ x_s), axis=1).reshape(12)


def matrix_a_from_pmatrix(pm, n):
    """Per-view A = inv(P[:, :3]) (row-major 9) and source x_s = -A P[:, 3],
    run_mgfpj_v2.py:218-227."""
    A_all = np.zeros(9 * n)
    xs_all = np.zeros(3 * n)
    for j, P in _views(np.asarray(pm, dtype=np.float64), n):
        A = np.linalg.inv(P[:, :3])
        A_all[9 * j:9 * j + 9] = A.reshape(9)
        xs_all[3 * j:3 * j + 3] = -(A @ P[:, 3])
    return A_all, xs_all


def save_pmatrix_side_files(self, folder):
    """Side files written with SaveModifiedConfigFolder, run_mgfbp.py:700-716."""
    save_jsonc(folder + "/pmatrix_file.jsonc", {"Value": self.array_pmatrix.tolist()})
    save_jsonc(folder + "/sid_file.jsonc", {"Value": self.source_isocenter_dis_each_view.tolist()})
    save_jsonc(folder + "/sdd_file.jsonc", {"Value": self.source_det_dis_each_view.tolist()})
    save_jsonc(folder + "/det_offset_horizontal_file.jsonc",
               {"Value": np.squeeze(self.det_offset_horizontal_each_view).tolist()})
    save_jsonc(folder + "/det_offset_vertical_file.jsonc",
               {"Value": np.squeeze(self.det_offset_vertical_each_view).tolist()})
    save_jsonc(folder + "/scan_angle_file.jsonc", {"Value": np.squeeze(self.scan_angle_each_view).tolist()})
