"""Float64 NumPy restatement of the FBP/FDK operators of run_mgfbp.py.

Test infrastructure (see ``oracle/__init__.py``).  Arrays follow the reference
layouts: sinogram ``[rows, views, cols]``, volume ``[z, y, x]``.
"""
import math

import numpy as np

from . import PI


def hamming_taps(nu, du, t, sdd=1.0, curved=False, dbt=False):
    """Spatial filter taps h[i], i in [0, 2*nu-1), n = i-(nu-1).

    run_mgfbp.py:877-914 (GenerateHammingKernel): ramp part scaled by t plus a
    cosine part scaled by (1-t); Taylor-series sine for the curved detector;
    optional DBT term.
    """
    n = np.arange(2 * nu - 1, dtype=np.int64) - (nu - 1)
    h = np.zeros(n.shape, dtype=np.float64)
    odd = (n % 2) != 0
    h[n == 0] = t / (4.0 * du * du)
    nf = n[odd].astype(np.float64)
    if curved:
        tv = nf * du / sdd
        s = tv - tv ** 3 / 3 / 2 / 1 + tv ** 5 / 5 / 4 / 3 / 2 / 1
        h[odd] = -t / (PI * PI * (sdd ** 2) * s ** 2)
    else:
        h[odd] = -t / (PI * PI * nf ** 2 * du ** 2)
    sgn = np.where(n % 2 == 0, 1.0, -1.0)
    a = 1.0 / (1.0 + 2.0 * n)
    b = 1.0 / (1.0 - 2.0 * n)
    h += (1.0 - t) * (sgn / (2 * PI * du * du) * (a + b) - 1.0 / (PI * PI * du * du) * (a * a + b * b))
    if dbt:
        kt = 0.02 / (2 * du)
        nz = n != 0
        h[~nz] += kt ** 2
        tv = n[nz] * du * kt * PI
        h[nz] += np.sin(tv) ** 2 / tv ** 2 * kt ** 2
    return h


def gaussian_taps(n_elem, d, delta):
    """Normalised Gaussian taps exp(-n^2/2/delta^2)/sum/d, run_mgfbp.py:917-927."""
    n = np.arange(2 * n_elem - 1, dtype=np.float64) - (n_elem - 1)
    g = np.exp(-n * n / 2.0 / delta / delta)
    with np.errstate(divide="ignore", invalid="ignore"):
        return g / g.sum() / d


def gaussian_apodized_ramp_taps(nu, du, delta, sdd=1.0, curved=False, dbt=False):
    """Ramp (t=1) convolved with the Gaussian, times du.

    run_mgfbp.py:1048-1060 (ConvolveKernelAndKernel) fed by :1265-1275.
    """
    g = gaussian_taps(nu, du, delta)
    ramp = hamming_taps(nu, du, 1.0, sdd, curved, dbt)
    m = 2 * nu - 1
    out = np.zeros(m, dtype=np.float64)
    for i in range(m):
        j = np.arange(m)
        k = i - (j - (nu - 1))
        ok = (k >= 0) & (k <= m - 1)
        out[i] = np.sum(g[j[ok]] * ramp[k[ok]]) * du
    return out


def angle_array(views, img_rot, scan):
    """beta_j = scan/views*j + img_rot, run_mgfbp.py:930-934."""
    return scan / views * np.arange(views, dtype=np.float64) + img_rot


def det_positions(n_total, n_actual, d, offset, begin=0):
    """(i + begin - (n_total-1)/2) * d + offset, run_mgfbp.py:937-944."""
    i = np.arange(n_actual, dtype=np.float64)
    return (i + begin - (n_total - 1) / 2.0) * d + offset


def det_positions_fpj(n, d, offset):
    """(i - (n-1)/2) * d + offset, run_mgfpj_v2.py:229-233."""
    i = np.arange(n, dtype=np.float64)
    return (i - (n - 1) / 2.0) * d + offset


def bh_correct(sgm, coeffs):
    """sum_t c_t * p^(t+1), run_mgfbp.py:946-954."""
    p = np.asarray(sgm, dtype=np.float64)
    out = np.zeros_like(p)
    for t, c in enumerate(coeffs):
        out += c * p ** (t + 1)
    return out


def parker_weights(u, angles, sdd, scan, curved):
    """Short-scan (Parker / over-scan) weights [views, cols], run_mgfbp.py:971-1011."""
    num_rounds = math.floor(abs(scan) / (PI * 2))
    remain = abs(scan) - num_rounds * PI * 2
    beta = np.abs(angles - angles[0])[:, None]
    rot_dir = abs(scan) / scan
    if curved:
        gamma = ((-1) * u / sdd) * rot_dir
    else:
        gamma = np.arctan2((-1) * u, sdd) * rot_dir
    gamma = np.broadcast_to(gamma[None, :], (angles.size, u.size))
    beta = np.broadcast_to(beta, gamma.shape)
    gmax = remain - PI
    w = np.zeros(gamma.shape, dtype=np.float64)
    if remain <= PI and num_rounds == 0:
        w[...] = 1.0
    elif remain <= PI and num_rounds >= 1:
        c1 = (0 <= beta) & (beta < remain)
        c2 = (remain <= beta) & (beta < 2 * PI * num_rounds)
        c3 = (2 * PI * num_rounds <= beta) & (beta <= 2 * PI * num_rounds + remain)
        w = np.where(c1, beta / remain, np.where(c2, 1.0, np.where(c3, (2 * PI * num_rounds + remain - beta) / remain, 0.0)))
    elif PI < remain <= 2 * PI:
        a = gmax - 2 * gamma
        b = PI * (2 * num_rounds + 1) - 2 * gamma
        c = PI * (2 * num_rounds + 1) + gmax
        with np.errstate(divide="ignore", invalid="ignore"):
            w1 = np.sin(PI / 2 * beta / a) ** 2
            w3 = np.sin(PI / 2 * (PI + gmax - (beta - PI * 2 * num_rounds)) / (gmax + 2 * gamma)) ** 2
        c1 = (0 <= beta) & (beta < a)
        c2 = (a <= beta) & (beta < b)
        c3 = (b <= beta) & (beta <= c)
        w = np.where(c1, w1, np.where(c2, 1.0, np.where(c3, w3, 0.0)))
    else:
        w[...] = 1.0
    return w


def weight_sgm(sgm, u, v, angles, sdd, curved=False, short_scan=False, scan=2 * PI):
    """Cosine (+ Parker) weighting of a [rows, views, cols] sinogram.

    run_mgfbp.py:956-1011 (WeightSgm).
    """
    p = np.asarray(sgm, dtype=np.float64)
    uu = u[None, None, :]
    vv = v[:, None, None]
    if curved:
        w = sdd * np.cos((-1) * uu / sdd) * sdd / np.sqrt(sdd ** 2 + vv ** 2)
    else:
        w = sdd * sdd / np.sqrt(sdd ** 2 + uu ** 2 + vv ** 2)
    out = p * w
    if short_scan:
        out = out * parker_weights(u, angles, sdd, scan, curved)[None, :, :]
    return out


def toeplitz_matrix(taps, nu):
    """T[m, k] = taps[k - m + nu - 1] so that y = x @ T (run_mgfbp.py:1043-1045)."""
    m = np.arange(nu)[:, None]
    k = np.arange(nu)[None, :]
    return taps[k - m + nu - 1]


def filter_rows(sgm, taps, du, gauss_v=None, dv=0.0):
    """Row convolution y = du * sum_m x[m] h[k-m+nu-1], optional +-10-row vertical
    Gaussian first.  run_mgfbp.py:1013-1046 (ConvolveSgmAndKernel).
    """
    p = np.asarray(sgm, dtype=np.float64)
    nv, nb, nu = p.shape
    if gauss_v is not None:
        inter = np.zeros_like(p)
        for i in range(nv):
            for n in range(max(0, i - 10), min(nv, i + 11)):
                inter[i] += p[n] * gauss_v[i + (nv - 1) - n]
        p = inter * dv
    T = toeplitz_matrix(np.asarray(taps, dtype=np.float64), nu)
    return (p.reshape(-1, nu) @ T).reshape(nv, nb, nu) * du


def div_factor(total_scan_angle, short_scan):
    """Redundancy factor of the backprojection, run_mgfbp.py:1072-1084."""
    num_rounds = float(math.floor(abs(total_scan_angle) / (PI * 2)))
    div = 1.0
    if short_scan:
        remain = abs(total_scan_angle) - num_rounds * 2 * PI
        if abs(total_scan_angle) < 2 * PI:
            div = 1.0
        elif remain < PI:
            div = 1.0 / (num_rounds * 2.0)
        elif PI < remain < 2 * PI:
            div = 1.0 / (num_rounds * 2.0 + 1.0)
    else:
        div = 1.0 / (num_rounds * 2.0)
    return div


def voxel_coords(nx, nz, px, pz, cx, cy, cz, img_rot, view_mode=1):
    """Rotated voxel-centre coordinates (x, y, z) as [nz, ny, nx] arrays.

    run_mgfbp.py:1090-1104 (axial / coronal / sagittal view modes).
    """
    iz, iy, ix = np.meshgrid(np.arange(nz, dtype=np.float64), np.arange(nx, dtype=np.float64),
                             np.arange(nx, dtype=np.float64), indexing="ij")
    if view_mode == 1:
        xa = px * (ix - (nx - 1) / 2.0) + cx
        ya = -px * (iy - (nx - 1) / 2.0) + cy
        z = (iz - (nz - 1) / 2.0) * pz + cz
    elif view_mode == 2:
        xa = px * (ix - (nx - 1) / 2.0) + cx
        z = -px * (iy - (nx - 1) / 2.0) + cz
        ya = -(iz - (nz - 1) / 2.0) * pz + cy
    else:
        z = -px * (iy - (nx - 1) / 2.0) + cz
        ya = -px * (ix - (nx - 1) / 2.0) + cy
        xa = (iz - (nz - 1) / 2.0) * pz + cx
    x = xa * math.cos(img_rot) + ya * math.sin(img_rot)
    y = -xa * math.sin(img_rot) + ya * math.cos(img_rot)
    return x, y, z


def _gather_bilinear(F, j, vfl, ufl, rv, ru):
    p0 = F[vfl, j, ufl] * (1 - ru) + F[vfl, j, ufl + 1] * ru
    p1 = F[vfl + 1, j, ufl] * (1 - ru) + F[vfl + 1, j, ufl + 1] * ru
    return (1 - rv) * p0 + rv * p1


def fdk_bp(F, angles, u_arr, v_arr, *, nx, nz, px, pz, cx, cy, cz, sid, sdd, dv, img_rot,
           total_scan_angle, short_scan, cone_beam, curved=False, view_mode=1, pmatrix=None):
    """Pixel-driven FDK backprojection of a filtered sinogram F [rows, views, cols].

    run_mgfbp.py:1062-1187 (BackProjectionPixelDriven), including its quirk: a
    voxel that projects outside u in [0, nu-1) or whose floor(v) is outside
    [0, nv-2] in ANY view is set to zero (the view loop breaks).
    """
    F = np.asarray(F, dtype=np.float64)
    nv, nb, nu = F.shape
    div = div_factor(total_scan_angle, short_scan)
    x, y, z = voxel_coords(nx, nz, px, pz, cx, cy, cz, img_rot, view_mode)
    acc = np.zeros(x.shape, dtype=np.float64)
    dead = np.zeros(x.shape, dtype=bool)
    iz = np.broadcast_to(np.arange(nz)[:, None, None], x.shape)
    u0 = u_arr[0]
    dus = u_arr[1] - u_arr[0]
    if cone_beam and pmatrix is None:
        v0 = v_arr[0]
        vs = abs(v_arr[1] - v_arr[0]) / (v_arr[1] - v_arr[0])
    for j in range(nb):
        if j == nb - 1:
            dbeta = abs(angles[nb - 1] - angles[0]) / (nb - 1)
        else:
            dbeta = abs(angles[j + 1] - angles[j])
        b = angles[j] - img_rot
        cb, sb = math.cos(b), math.sin(b)
        L = sid - x * cb - y * sb
        if pmatrix is None:
            mag = sdd / L
            t = -x * sb + y * cb
            if curved:
                u = sdd * np.arctan2(t, L)
            else:
                u = mag * t
            uidx = (u - u0) / dus
        else:
            P = pmatrix[12 * j:12 * j + 12]
            mag = 1.0 / (P[8] * x + P[9] * y + P[10] * z + P[11])
            uidx = (P[0] * x + P[1] * y + P[2] * z + P[3]) * mag
        du_dead = (uidx < 0) | (uidx + 1 > nu - 1)
        ufl = np.clip(np.floor(uidx), 0, nu - 2).astype(np.int64)
        ru = uidx - np.floor(uidx)
        if curved:
            dw = 1.0 / (L * L + (x * sb - y * cb) * (x * sb - y * cb))
        else:
            dw = 1.0 / (L * L)
        if cone_beam:
            if pmatrix is None:
                vidx = (mag * z - v0) / dv * vs
            else:
                vidx = (P[4] * x + P[5] * y + P[6] * z + P[7]) * mag
            vfl_f = np.floor(vidx)
            dv_dead = (vfl_f < 0) | (vfl_f + 1 > nv - 1)
            vfl = np.clip(vfl_f, 0, nv - 2).astype(np.int64)
            rv = vidx - vfl_f
            val = _gather_bilinear(F, j, vfl, ufl, rv, ru)
            dead_now = du_dead | dv_dead
        else:
            val = F[iz, j, ufl] * (1 - ru) + F[iz, j, ufl + 1] * ru
            dead_now = du_dead
        dead |= dead_now
        term = (sid * dw) * val * dbeta * div
        acc += np.where(dead, 0.0, term)
    return np.where(dead, 0.0, acc)


def helical_rebin(sgm, z_pos, *, view_count, dis_per_view, mag, det_offset_vertical, dv, sdd):
    """Per-slice fan sinograms from a helical sinogram sgm [rows, views, cols]:
    out [slices, view_count, cols].  Mgfbp_helical.SinogramRebinning,
    run_mgfbp_helical.py:178-205 (float64 here)."""
    sgm = np.asarray(sgm, dtype=np.float64)
    nv, nb, nu = sgm.shape
    out = np.zeros((len(z_pos), view_count, nu))
    for s, z in enumerate(np.asarray(z_pos, dtype=np.float64)):
        v0 = (z - det_offset_vertical / mag) / dis_per_view
        begin = math.floor(v0 - 0.5 * view_count + 0.5)
        for i in range(view_count):
            vi = begin + i
            if not (0 <= vi <= nb - 2):
                continue
            v_pos = (z - vi * dis_per_view) * mag - det_offset_vertical
            v_idx = -v_pos / dv + (nv - 1.0) / 2.0
            if v_idx >= nv - 1:
                row = sgm[nv - 1, int(vi)]
            elif v_idx <= 0:
                row = sgm[0, int(vi)]
            else:
                f = math.floor(v_idx)
                w = v_idx - f
                row = sgm[f, int(vi)] * (1 - w) + sgm[f + 1, int(vi)] * w
            out[s, i] = row * sdd / math.sqrt(sdd ** 2 + v_pos ** 2)
    return out
