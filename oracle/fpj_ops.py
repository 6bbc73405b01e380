"""Float64 NumPy restatement of the ray-driven forward projector.

run_mgfpj_v3.py:184-366 (ForwardProjectionBilinear, one view per launch), its
masked copy in run_mgfbp_iterative_recon_IRN_CGLS.py:494-676 and the
effective-ray-map agent :679-833.  Test infrastructure (see oracle/__init__.py).
"""
import math

import numpy as np

from . import PI


def helical_z_per_view(angles, v_arr, nv_total, pitch, sid, sdd):
    """Gantry z advance per view, run_mgfpj_v3.py:242-249."""
    nb = angles.size
    total = abs(angles[nb - 1] - angles[0]) / (nb - 1) * nb
    laps = total / (PI * 2)
    return pitch * (laps / nb) * (abs(v_arr[1] - v_arr[0]) * nv_total) / (sdd / sid)


def count_steps(nx, nz, px, pz, step):
    """Number of ray-march steps K = floor(D / (step*vd)), run_mgfpj_v3.py:252."""
    img_dimension = nx * px
    image_dimension_z = nz * pz
    vd = (2 * (px ** 2) + (pz ** 2)) ** 0.5
    D = (2 * img_dimension ** 2 + image_dimension_z ** 2) ** 0.5
    return int(math.floor(D / (step * vd)))


def count_steps_ir(nx, nz, px, pz, step, sid):
    """K = floor((l_max - l_min) / (step*vd)), IRN_CGLS.py:562-563 and :746-747."""
    img_dimension = nx * px
    image_dimension_z = nz * pz
    vd = (2 * (px ** 2) + (pz ** 2)) ** 0.5
    l_min = sid - (2 * img_dimension ** 2 + image_dimension_z ** 2) ** 0.5 / 2.0
    l_max = sid + (2 * img_dimension ** 2 + image_dimension_z ** 2) ** 0.5 / 2.0
    return int(math.floor((l_max - l_min) / (step * vd)))


def _ray_dirs(u_arr, v_arr, rows, sid, sdd, curved, zpv, view_idx):
    """Source position and unit direction of every (row, col) ray of one view.

    run_mgfpj_v3.py:258-278.
    """
    uu = np.asarray(u_arr, dtype=np.float64)[None, :]
    vv = np.asarray(v_arr, dtype=np.float64)[:rows, None]
    if curved:
        g = (-uu) / sdd
        dx = -sdd * np.cos(g) + sid
        dy = -sdd * np.sin(g)
    else:
        dx = -(sdd - sid) + 0.0 * uu
        dy = uu
    dz = vv + zpv * view_idx
    sz = zpv * view_idx
    dx, dy, dz = np.broadcast_arrays(dx, dy, dz)
    dist = ((dx - sid) ** 2 + (dy - 0.0) ** 2 + (dz - sz) ** 2) ** 0.5
    return sz, (dx - sid) / dist, (dy - 0.0) / dist, (dz - sz) / dist, dist


def march(vol, view_idx, angles, u_arr, v_arr, *, nx, nz, px, pz, cx, cy, cz_view, sid, sdd,
          step, cone_beam, curved=False, zpv=0.0, rows=None, K=None, mask=None,
          pmat_A=None, pmat_xs=None, mode="fp", ray_values=None, out=None):
    """One view of the ray-driven projector over rows x cols rays.

    mode 'fp'     : trilinear Riemann sum (run_mgfpj_v3.py:283-363); rays with
                    mask == 0 give 0 (IRN_CGLS.py:567).  Returns [rows, cols].
    mode 'emap'   : effective-map value (IRN_CGLS.py:750, 824-833).  Returns [rows, cols].
    mode 'adjoint': the exact transpose of 'fp' (no reference counterpart): every sample
                    that 'fp' sums adds ray_values[row, col] x its trilinear weights x
                    the step length to the volume `out` [nz, nx, nx] (float64, in place;
                    rays with mask != 1 add nothing).  Returns out.
    """
    nu = len(u_arr)
    rows = len(v_arr) if rows is None else rows
    vd = (2 * (px ** 2) + (pz ** 2)) ** 0.5
    img_dimension = nx * px
    image_dimension_z = nz * pz
    l_min = sid - (2 * img_dimension ** 2 + image_dimension_z ** 2) ** 0.5 / 2.0
    x0 = -(nx - 1.0) / 2.0 * px + cx
    y0 = -(nx - 1.0) / 2.0 * (-px) + cy
    z0 = -(nz - 1.0) / 2.0 * pz + cz_view
    sz, ux, uy, uz, dist = _ray_dirs(u_arr, v_arr, rows, sid, sdd, curved, zpv, view_idx)
    cb, sb = math.cos(angles[view_idx]), math.sin(angles[view_idx])
    c0, s0 = math.cos(angles[0]), math.sin(angles[0])
    use_p = pmat_A is not None
    if use_p:
        A = pmat_A[view_idx * 9:view_idx * 9 + 9]
        xs = pmat_xs[view_idx * 3:view_idx * 3 + 3]
        ui = np.arange(nu, dtype=np.float64)[None, :]
        vi = np.arange(rows, dtype=np.float64)[:, None]
        ax = A[0] * ui + A[1] * vi + A[2]
        ay = A[3] * ui + A[4] * vi + A[5]
        az = A[6] * ui + A[7] * vi + A[8]
    acc = np.zeros((rows, nu), dtype=np.float64)
    emap = np.ones((rows, nu), dtype=np.float64)
    V = None if vol is None else np.asarray(vol, dtype=np.float64)
    if mode == "adjoint":
        Y = np.asarray(ray_values, dtype=np.float64)[:rows]
        if mask is not None:
            Y = np.where(np.asarray(mask)[:rows] == 1, Y, 0.0)
    rowz = np.broadcast_to(np.arange(rows)[:, None], (rows, nu))
    for k in range(K):
        lk = k * step * vd + l_min
        if use_p:
            om = lk / dist
            xp = om * ax + xs[0]
            yp = om * ay + xs[1]
            zp = om * az + xs[2] + zpv * view_idx
            xr = xp * c0 - yp * s0
            yr = yp * c0 + xp * s0
            zr = zp
        else:
            x = sid + ux * lk
            y = 0.0 + uy * lk
            z = sz + uz * lk
            xr = x * cb - y * sb
            yr = y * cb + x * sb
            zr = z
        xi = np.floor((xr - x0) / px)
        yi = np.floor((yr - y0) / (-px))
        ok = (xi >= 0) & (xi + 1 < nx) & (yi >= 0) & (yi + 1 < nx)
        if mode == "emap":
            if cone_beam:
                zi = np.floor((zr - z0) / pz)
                inc = ((xi - nx / 2.0) ** 2 + (yi - nx / 2.0) ** 2) < (nx / 2.0) ** 2
                bad = ok & inc & ((zi < 0) | (zi + 1 >= nz))
                emap[bad] = 0.0
            continue
        xw = (xr - (xi * px + x0)) / px
        yw = (yr - (yi * (-px) + y0)) / (-px)
        xa = np.clip(xi, 0, nx - 2).astype(np.int64)
        ya = np.clip(yi, 0, nx - 2).astype(np.int64)
        if mode == "adjoint":
            if cone_beam:
                zi = np.floor((zr - z0) / pz)
                okz = ok & (zi >= 0) & (zi + 1 < nz)
                za = np.clip(zi, 0, nz - 2).astype(np.int64)
                zw = (zr - (zi * pz + z0)) / pz
            else:
                okz, za, zw = ok, rowz, np.zeros_like(xw)
            w = np.where(okz, Y * step * vd, 0.0)
            for dz in ((0, 1) if cone_beam else (0,)):
                wz = zw if dz else 1.0 - zw
                for dy in (0, 1):
                    wy = yw if dy else 1.0 - yw
                    for dx in (0, 1):
                        wx = xw if dx else 1.0 - xw
                        np.add.at(out, (za + dz, ya + dy, xa + dx), w * wz * wy * wx)
            continue
        if cone_beam:
            zi = np.floor((zr - z0) / pz)
            okz = ok & (zi >= 0) & (zi + 1 < nz)
            za = np.clip(zi, 0, nz - 2).astype(np.int64)
            zw = (zr - (zi * pz + z0)) / pz
            lo = ((1.0 - xw) * (1.0 - yw) * V[za, ya, xa] + xw * (1.0 - yw) * V[za, ya, xa + 1]
                  + (1.0 - xw) * yw * V[za, ya + 1, xa] + xw * yw * V[za, ya + 1, xa + 1])
            hi = ((1.0 - xw) * (1.0 - yw) * V[za + 1, ya, xa] + xw * (1.0 - yw) * V[za + 1, ya, xa + 1]
                  + (1.0 - xw) * yw * V[za + 1, ya + 1, xa] + xw * yw * V[za + 1, ya + 1, xa + 1])
            val = ((1.0 - zw) * lo + zw * hi) * step * vd
            acc += np.where(okz, val, 0.0)
        else:
            zz = rowz
            val = ((1 - xw) * (1 - yw) * V[zz, ya, xa] + xw * (1 - yw) * V[zz, ya, xa + 1]
                   + (1 - xw) * yw * V[zz, ya + 1, xa] + xw * yw * V[zz, ya + 1, xa + 1])
            acc += np.where(ok, val * step * vd, 0.0)
    if mode == "emap":
        return emap
    if mode == "adjoint":
        return out
    if mask is not None:
        acc = np.where(np.asarray(mask)[:rows] == 1, acc, 0.0)
    return acc


def bin_sinogram(sgm_large, bin_size):
    """Mean over oversampled sub-columns, run_mgfpj_v3.py:368-375."""
    a = np.asarray(sgm_large, dtype=np.float64)
    r, c = a.shape[0], a.shape[-1] // bin_size
    return a[..., :c * bin_size].reshape(a.shape[:-1] + (c, bin_size)).sum(-1) / bin_size
