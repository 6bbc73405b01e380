"""Differentiation through the projector pair: dot-product adjointness, central
finite differences, a torch-autograd reference gradient on a 64^2 grid, and the
TV / PICCS objectives."""
import math

import numpy as np
import pytest

from test_gpu_parity import _cone_obj

pytestmark = pytest.mark.gpu


def _torch_fp_reference(vol, dg):
    """Pure-torch (float64, autograd) restatement of the ray-driven trilinear
    projector (run_mgfpj_v3.py:255-365) for small grids."""
    import torch
    g = dg.geom
    u = torch.tensor(dg.host["u"][:g.nu], dtype=torch.float64)
    v = torch.tensor(dg.host["v"][:g.nv], dtype=torch.float64)
    ang = torch.tensor(dg.host["angles"], dtype=torch.float64)
    nx, nz = g.nx, g.nz
    px, pz = float(g.px), float(g.pz)
    vd = math.sqrt(2 * px * px + pz * pz)
    lmin = g.sid - math.sqrt(2 * (nx * px) ** 2 + (nz * pz) ** 2) / 2.0
    x0 = -(nx - 1) / 2 * px + g.cx
    y0 = (nx - 1) / 2 * px + g.cy
    z0 = -(nz - 1) / 2 * pz + g.cz
    dx = -(g.sdd - g.sid)
    dy = u[None, :].expand(g.nv, g.nu)
    dz = v[:, None].expand(g.nv, g.nu)
    ex, ey, ez = dx - g.sid, dy, dz
    dist = torch.sqrt(ex * ex + ey * ey + ez * ez)
    ux, uy, uz = ex / dist, ey / dist, ez / dist
    k = torch.arange(g.fp_steps, dtype=torch.float64)
    lk = k * g.fp_step * vd + lmin
    flat = vol.reshape(-1)
    out = []
    for j in range(g.views):
        cb, sb = torch.cos(ang[j]), torch.sin(ang[j])
        x = g.sid + ux[..., None] * lk
        y = uy[..., None] * lk
        z = uz[..., None] * lk
        xr, yr = x * cb - y * sb, y * cb + x * sb
        fx, fy, fz = (xr - x0) / px, (yr - y0) / (-px), (z - z0) / pz
        xi, yi, zi = torch.floor(fx), torch.floor(fy), torch.floor(fz)
        ok = (xi >= 0) & (xi + 1 < nx) & (yi >= 0) & (yi + 1 < nx) & (zi >= 0) & (zi + 1 < nz)
        xw, yw, zw = fx - xi, fy - yi, fz - zi
        xi = xi.clamp(0, nx - 2).long()
        yi = yi.clamp(0, nx - 2).long()
        zi = zi.clamp(0, nz - 2).long()
        val = 0
        for a in (0, 1):
            for b in (0, 1):
                for c in (0, 1):
                    w = (xw if c else 1 - xw) * (yw if b else 1 - yw) * (zw if a else 1 - zw)
                    val = val + w * flat[((zi + a) * nx + (yi + b)) * nx + (xi + c)]
        out.append((val * ok).sum(-1) * g.fp_step * vd)
    return torch.stack(out, dim=1)


def test_gradient_matches_torch_autograd_reference(cuda):
    import torch
    from reconstruction_program_taichi_gb300 import geometry
    from reconstruction_program_taichi_gb300.autograd import forward_project
    # 16 slices: every ray stays well inside the volume in z, so no ray grazes a
    # boundary voxel-centre plane (where float32 vs float64 rounding would decide
    # whole rays); zero border in x, y for the same reason.
    o = _cone_obj(n=64, nz=16, nu=80, nv=6, views=8)
    dg = geometry.fpj_geometry(o)
    rng = np.random.default_rng(2)
    x = np.zeros(dg.vol_shape)
    x[:, 2:-2, 2:-2] = rng.uniform(0, 0.02, (16, 60, 60))
    b = rng.uniform(0, 1, dg.sgm_shape)
    xt = torch.tensor(x, dtype=torch.float64, requires_grad=True)
    ref_sgm = _torch_fp_reference(xt, dg)
    loss_ref = 0.5 * ((ref_sgm - torch.tensor(b)) ** 2).sum()
    loss_ref.backward()
    xg = torch.tensor(x, dtype=torch.float32, device="cuda", requires_grad=True)
    sgm = forward_project(xg, dg)
    assert torch.linalg.vector_norm(sgm.double().cpu() - ref_sgm.detach()) / torch.linalg.vector_norm(ref_sgm) < 1e-4
    loss = 0.5 * ((sgm - torch.tensor(b, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()
    g_ours = xg.grad.double().cpu()
    rel = torch.linalg.vector_norm(g_ours - xt.grad) / torch.linalg.vector_norm(xt.grad)
    assert rel < 1e-4


def test_central_finite_differences(cuda):
    import torch
    from reconstruction_program_taichi_gb300 import geometry
    from reconstruction_program_taichi_gb300.autograd import forward_project
    o = _cone_obj(n=32, nz=12, nu=48, nv=16, views=12)
    dg = geometry.fpj_geometry(o)
    gen = torch.Generator(device="cuda").manual_seed(4)
    x = torch.rand(dg.vol_shape, device="cuda", generator=gen) * 0.02
    b = torch.rand(dg.sgm_shape, device="cuda", generator=gen)
    d = torch.randn(dg.vol_shape, device="cuda", generator=gen)

    def loss(v):
        r = forward_project(v, dg) - b
        return 0.5 * (r.double() ** 2).sum()

    xg = x.clone().requires_grad_(True)
    loss(xg).backward()
    analytic = float((xg.grad.double() * d.double()).sum())
    eps = 1e-3
    with torch.no_grad():
        fd = (float(loss(x + eps * d)) - float(loss(x - eps * d))) / (2 * eps)
    assert abs(fd - analytic) / abs(analytic) < 1e-3


def test_tv_and_piccs_objectives_differentiate(cuda):
    import torch
    from reconstruction_program_taichi_gb300 import geometry
    from reconstruction_program_taichi_gb300.autograd import Projector, tv_isotropic
    o = _cone_obj(n=32, nz=8, nu=48, nv=12, views=10)
    proj = Projector(geometry.fpj_geometry(o))
    gen = torch.Generator(device="cuda").manual_seed(5)
    truth = torch.rand(proj.dg.vol_shape, device="cuda", generator=gen) * 0.02
    b = proj(truth).detach()
    prior = truth * 0.9
    x = torch.zeros_like(truth, requires_grad=True)
    opt = torch.optim.Adam([x], lr=2e-3)
    first = None
    for _ in range(30):
        opt.zero_grad()
        lam, alpha = 1e-4, 0.5
        loss = 0.5 * ((proj(x) - b) ** 2).sum() + lam * (1 - alpha) * tv_isotropic(x, 1e-6) \
            + lam * alpha * tv_isotropic(x - prior, 1e-6)
        loss.backward()
        first = first if first is not None else float(loss)
        opt.step()
    assert float(loss) < 0.2 * first
    assert torch.isfinite(x.grad).all()
