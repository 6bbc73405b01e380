"""Float64 NumPy restatement of the IRN-CGLS-TV / PICCS operators.

run_mgfbp_iterative_recon_IRN_CGLS.py (per-view "P^T" backprojector, TV
reweighting, D^T W D, CGLS Tikhonov solves) and
run_mgfbp_iterative_recon_IRN_CGLS_piccs.py.  Test infrastructure (see
oracle/__init__.py).
"""
import math

import numpy as np

from .fbp_ops import voxel_coords
from .fpj_ops import march


def bp_unmatched(sgm, angles, u_arr, v_arr, cz_views, *, nx, nz, px, pz, cx, cy, sid, sdd, dv,
                 img_rot, cone_beam, curved=False, view_mode=1, pmatrix=None):
    """Sum over views of the per-view bilinear-gather backprojector, then zero
    every voxel whose u fell outside [0, nu-1) in any view.

    run_mgfbp_iterative_recon_IRN_CGLS.py:372-474 (BackProjectionPixelDrivenPerView)
    driven view by view as in :319-336, and SetTruncatedRegionToZero :477-481.
    ``sgm`` is [rows, views, cols]; rows outside [0, nv-1) in v only skip.
    """
    S = np.asarray(sgm, dtype=np.float64)
    nv, nb, nu = S.shape
    acc = np.zeros((nz, nx, nx), dtype=np.float64)
    flag = np.ones((nz, nx, nx), dtype=np.float64)
    u0 = u_arr[0]
    dus = u_arr[1] - u_arr[0]
    if cone_beam and pmatrix is None:
        v0 = v_arr[0]
        vs = abs(v_arr[1] - v_arr[0]) / (v_arr[1] - v_arr[0])
    iz = np.broadcast_to(np.arange(nz)[:, None, None], acc.shape)
    for j in range(nb):
        x, y, z = voxel_coords(nx, nz, px, pz, cx, cy, cz_views[j], img_rot, view_mode)
        b = angles[j] - img_rot
        cb, sb = math.cos(b), math.sin(b)
        L = sid - x * cb - y * sb
        ax = np.abs(x - sid * cb)
        ay = np.abs(y - sid * sb)
        dflag = ax > ay
        dfac = np.sqrt((x - sid * cb) ** 2 + (y - sid * sb) ** 2 + z ** 2) / (ax * dflag + ay * (1 - dflag))
        if pmatrix is None:
            mag = sdd / L
            t = -x * sb + y * cb
            u = sdd * np.arctan2(t, L) if curved else mag * t
            uidx = (u - u0) / dus
        else:
            P = pmatrix[12 * j:12 * j + 12]
            mag = 1.0 / (P[8] * x + P[9] * y + P[10] * z + P[11])
            uidx = (P[0] * x + P[1] * y + P[2] * z + P[3]) * mag
        out_u = (uidx < 0) | (uidx + 1 > nu - 1)
        flag[out_u] = 0.0
        ufl_f = np.floor(uidx)
        ufl = np.clip(ufl_f, 0, nu - 2).astype(np.int64)
        ru = uidx - ufl_f
        if cone_beam:
            if pmatrix is None:
                vidx = (mag * z - v0) / dv * vs
            else:
                vidx = (P[4] * x + P[5] * y + P[6] * z + P[7]) * mag
            vfl_f = np.floor(vidx)
            out_v = (vfl_f < 0) | (vfl_f + 1 > nv - 1)
            vfl = np.clip(vfl_f, 0, nv - 2).astype(np.int64)
            rv = vidx - vfl_f
            p0 = S[vfl, j, ufl] * (1 - ru) + S[vfl, j, ufl + 1] * ru
            p1 = S[vfl + 1, j, ufl] * (1 - ru) + S[vfl + 1, j, ufl + 1] * ru
            val = ((1 - rv) * p0 + rv * p1) * dfac * px
            acc += np.where(out_u | out_v, 0.0, val)
        else:
            val = ((1 - ru) * S[iz, j, ufl] + ru * S[iz, j, ufl + 1]) * dfac * px
            acc += np.where(out_u, 0.0, val)
    return acc * flag


def forward_diffs(x):
    """(ux along y, uy along x, uz along z if nz > 2), zero at the last index.

    run_mgfbp_iterative_recon_IRN_CGLS.py:235-241 (same in :246-252, :268-274).
    """
    ux = np.zeros_like(x)
    uy = np.zeros_like(x)
    uz = np.zeros_like(x)
    ux[:, 0:-1, :] = x[:, 1:, :] - x[:, :-1, :]
    uy[:, :, 0:-1] = x[:, :, 1:] - x[:, :, :-1]
    if x.shape[0] > 2:
        uz[0:-1, :, :] = x[1:, :, :] - x[:-1, :, :]
    return ux, uy, uz


def generate_wr(x, beta_tv):
    """WR = 1/sqrt(|grad x|^2 + beta), IRN_CGLS.py:234-243."""
    ux, uy, uz = forward_diffs(np.asarray(x, dtype=np.float64))
    return 1.0 / np.sqrt(ux ** 2 + uy ** 2 + uz ** 2 + beta_tv)


def tv_penalty(x, beta_tv):
    """sum sqrt(|grad x|^2 + beta), IRN_CGLS.py:245-254."""
    ux, uy, uz = forward_diffs(np.asarray(x, dtype=np.float64))
    return float(np.sum(np.sqrt(ux * ux + uy * uy + uz * uz + beta_tv)))


def dtwd(x, wr):
    """D^T W D x with interior-only backward differences, IRN_CGLS.py:267-286."""
    x = np.asarray(x, dtype=np.float64)
    ux, uy, uz = forward_diffs(x)
    ux = wr * ux
    uy = wr * uy
    uz = wr * uz
    uxx = np.zeros_like(x)
    uyy = np.zeros_like(x)
    uzz = np.zeros_like(x)
    uxx[:, 1:-1, :] = ux[:, 1:-1, :] - ux[:, 0:-2, :]
    uyy[:, :, 1:-1] = uy[:, :, 1:-1] - uy[:, :, 0:-2]
    if x.shape[0] > 2:
        uzz[1:-1, :, :] = uz[1:-1, :, :] - uz[0:-2, :, :]
    return -uxx - uyy - uzz


class IrOperators:
    """Masked FP (IRN_CGLS.py:354-370, 494-676), unmatched BP (:319-336, 372-481)
    and their composition P^T P (:288-316), for one fixed geometry."""

    def __init__(self, g):
        self.g = g  # dict of geometry (see tests/golden/make_golden.py for keys)
        self.calls = 0

    def emap(self):
        g = self.g
        out = np.zeros((g["rows"], g["views"], g["nu"]))
        for j in range(g["views"]):
            out[:, j, :] = march(None, j, g["angles"], g["u"], g["v"], nx=g["nx"], nz=g["nz"], px=g["px"],
                                 pz=g["pz"], cx=g["cx"], cy=g["cy"], cz_view=g["cz"][j], sid=g["sid"],
                                 sdd=g["sdd"], step=g["step"], cone_beam=g["cone"], curved=g["curved"],
                                 zpv=g["zpv"], rows=g["rows"], K=g["K"], mode="emap")
        return out

    def fp(self, x, mask):
        g = self.g
        out = np.zeros((g["rows"], g["views"], g["nu"]))
        for j in range(g["views"]):
            out[:, j, :] = march(x, j, g["angles"], g["u"], g["v"], nx=g["nx"], nz=g["nz"], px=g["px"],
                                 pz=g["pz"], cx=g["cx"], cy=g["cy"], cz_view=g["cz"][j], sid=g["sid"],
                                 sdd=g["sdd"], step=g["step"], cone_beam=g["cone"], curved=g["curved"],
                                 zpv=g["zpv"], rows=g["rows"], K=g["K"], mask=mask[:, j, :])
        return out

    def bp(self, sgm):
        g = self.g
        return bp_unmatched(sgm, g["angles"], g["u"], g["v"], g["cz"], nx=g["nx"], nz=g["nz"], px=g["px"],
                            pz=g["pz"], cx=g["cx"], cy=g["cy"], sid=g["sid"], sdd=g["sdd"], dv=g["dv"],
                            img_rot=g["img_rot"], cone_beam=g["cone"], curved=g["curved"],
                            view_mode=g.get("view_mode", 1))

    def ptp(self, x, mask):
        self.calls += 1
        return self.bp(self.fp(x, mask))


def tikhonov_tv(ops, mask, bp_b, x_seed, wr, lam, ratio, n_iter):
    """CGLS on (P^T P + lam*ratio*D^T W D) x = P^T b, IRN_CGLS.py:188-232."""
    bpfpx = ops.ptp(x_seed, mask)
    out = x_seed
    d = bp_b - bpfpx - lam * dtwd(x_seed, wr) * ratio
    r = d
    for _ in range(n_iter):
        q = ops.ptp(d, mask) + lam * dtwd(d, wr) * ratio
        rr = np.sum(r * r)
        alpha = rr / np.sum(d * q)
        out = out + alpha * d
        r = r - alpha * q
        beta = np.sum(r * r) / rr
        d = r + beta * d
    return out


def irn_tv(ops, sgm, x_seed, lam, beta_tv, n_irn, n_iter):
    """IRN-CGLS-TV driver, IRN_CGLS.py:138-176 (returns the attenuation image)."""
    g = ops.g
    mask = ops.emap()
    bp_b = ops.bp(sgm * mask)
    ratio = float(g["rows"] * g["views"] * g["nu"] / (g["nz"] * g["nx"] * g["nx"]))
    x = tikhonov_tv(ops, mask, bp_b, x_seed, np.ones_like(x_seed), lam, ratio, n_iter)
    for _ in range(n_irn):
        wr = generate_wr(x, beta_tv)
        x = tikhonov_tv(ops, mask, bp_b, x, wr, lam, ratio, n_iter)
    return x


def tikhonov_piccs(ops, mask, bp_b, x_seed, prior, wr, wrp, lam, alpha, ratio, n_iter):
    """PICCS CGLS, run_mgfbp_iterative_recon_IRN_CGLS_piccs.py:112-150."""

    def fx(x):
        return (ops.ptp(x, mask) + lam * (1 - alpha) * dtwd(x, wr) * ratio
                + lam * alpha * dtwd(x, wrp) * ratio)

    out = x_seed
    d = bp_b + lam * alpha * ratio * dtwd(prior, wrp) - fx(x_seed)
    r = d
    for _ in range(n_iter):
        q = fx(d)
        rr = np.sum(r * r)
        a = rr / np.sum(d * q)
        out = out + a * d
        r = r - a * q
        beta = np.sum(r * r) / rr
        d = r + beta * d
    return out


def irn_piccs(ops, sgm, prior, lam, alpha, beta_tv, n_irn, n_iter):
    """IRN-CGLS-PICCS driver, run_mgfbp_iterative_recon_IRN_CGLS_piccs.py:70-110."""
    g = ops.g
    mask = ops.emap()
    bp_b = ops.bp(sgm * mask)
    ratio = float(g["rows"] * g["views"] * g["nu"] / (g["nz"] * g["nx"] * g["nx"]))
    x = prior
    ones = np.ones_like(prior)
    x = tikhonov_piccs(ops, mask, bp_b, x, prior, ones, ones, lam, alpha, ratio, n_iter)
    for _ in range(n_irn):
        wr = generate_wr(x, beta_tv)
        wrp = generate_wr(x - prior, beta_tv)
        x = tikhonov_piccs(ops, mask, bp_b, x, prior, wr, wrp, lam, alpha, ratio, n_iter)
    return x


def _diff(x, axis):
    """Forward difference with 0 at the last index (ADMM script Diff, :185-193)."""
    out = np.zeros_like(x)
    sl_a = [slice(None)] * 3
    sl_b = [slice(None)] * 3
    sl_a[axis], sl_b[axis] = slice(1, None), slice(None, -1)
    out[tuple(sl_b)] = x[tuple(sl_a)] - x[tuple(sl_b)]
    return out


def _diff_t(x, axis):
    """out[i] = x[i-1] - x[i] on interior indices (ADMM script DiffT, :195-203)."""
    out = np.zeros_like(x)
    sl_o = [slice(None)] * 3
    sl_p = [slice(None)] * 3
    sl_o[axis], sl_p[axis] = slice(1, -1), slice(0, -2)
    out[tuple(sl_o)] = x[tuple(sl_p)] - x[tuple(sl_o)]
    return out


def admm_tv(ops, sgm, x_seed, lam, n_outer, n_iter, rho=0.1):
    """ADMM-TV driver of run_mgfbp_iterative_recon_ADMM_CGLS.py:79-162 (float64):
    x-step CGLS on (P^T P + rho D^T D) x = P^T b + rho Dt v - Dt p; hard-threshold
    v-step; dual ascent.  Returns (x, v_y, v_x, p_y, p_x) with y = axis 1, x = axis 2."""
    g = ops.g
    mask = ops.emap()
    bp_b = ops.bp(sgm * mask)
    ratio = float(g["rows"] * g["views"] * g["nu"] / (g["nz"] * g["nx"] * g["nx"]))
    ones = np.ones_like(x_seed)
    x = x_seed
    vy, vx = _diff(x, 1), _diff(x, 2)
    py, px = np.zeros_like(x), np.zeros_like(x)
    for _ in range(n_outer):
        rhs = bp_b + rho * (_diff_t(vy, 1) + _diff_t(vx, 2)) - (_diff_t(py, 1) + _diff_t(px, 2))

        def fx(a):
            return ops.ptp(a, mask) + rho * dtwd(a, ones)

        out = x
        d = rhs - fx(x)
        r = d
        for _ in range(n_iter):
            q = fx(d)
            rr = np.sum(r * r)
            alpha = rr / np.sum(d * q)
            out = out + alpha * d
            r = r - alpha * q
            d = r + np.sum(r * r) / rr * d
        x = out
        wy = _diff(x, 1) + py / rho
        wx = _diff(x, 2) + px / rho
        t = np.sqrt(wy * wy + wx * wx)
        keep = ((t - lam * ratio / rho) > 0) & (t != 0)
        vy, vx = np.where(keep, wy, 0.0), np.where(keep, wx, 0.0)
        py = py + rho * (_diff(x, 1) - vy)
        px = px + rho * (_diff(x, 2) - vx)
    return x, vy, vx, py, px
