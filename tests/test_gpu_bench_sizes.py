"""Parity at the benchmark configurations' full sizes against float64 restatements of
the same discrete operators.

* 2D fan-beam FBP (256^2, 720 views, 512 bins): the whole image against the float64
  NumPy oracle (oracle/fbp_ops.py).
* Cone-beam FDK at 512x512x256 / 1080 views / 1024x256 detector: a central slab and a
  slab near the volume's end (where the reference's break-to-zero rule clears voxels
  that leave the detector), every view and every detector row the slab reads, against
  the float64 C restatement (oracle/cpu_ref.c, pinned to the NumPy oracle to 1e-12 by
  tests/test_cpu_ref.py); the forward projection of the FDK volume on 4 evenly spaced
  views, every ray.
* The iterative drivers' operators at 512x512x64 / 360 views and 512x512x128 / 90 views:
  the masked projector (4 views) and the driver's backprojector (8-slice slab).

The plain float32 path must match within 1e-4 relative L2 with the same zero pattern;
each 16-bit storage variant has its own stated bound (measured values in the
docstrings)."""
import numpy as np
import pytest

import bench
from conftest import rel_l2
from oracle import cpu_ref
from oracle import fbp_ops as F

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _sino(dg, w):
    from reconstruction_program_taichi_gb300 import ops
    return bench.noisy(ops.project_ellipsoids(dg, bench.ellipsoids(w)), w["photons"], w["seed"])


def _max_rel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / np.abs(b).max())


def test_c1_fan_fbp_whole_image_vs_float64_oracle(cuda):
    """Plain: tensor-core filter with three bf16 parts and float32 backprojection
    coefficients.  Mixed: two parts and bf16 coefficients (bound 2e-3)."""
    from reconstruction_program_taichi_gb300 import fbp, geometry
    w = bench.C1
    o = bench.parse(w)
    taps = bench.hann_from_ramp(geometry.recon_taps(o))
    ref = None
    for storage, impl, tol in (("f32", "tc3", TOL), ("f32", "simt", TOL), ("bf16", "tc", 2e-3)):
        pipe = fbp.FdkPipeline(o, storage=storage, filter_impl=impl)
        pipe.set_taps(taps)
        sgm = _sino(pipe.dg, w)
        got = pipe.run(sgm).cpu().numpy()
        if ref is None:
            u, v, ang = geometry.fbp_arrays(o)
            s64 = sgm.cpu().numpy().astype(np.float64)
            wtd = F.weight_sgm(s64, u, v, ang, o.source_det_dis)
            filt = F.filter_rows(wtd, taps, o.det_elem_width)
            ref = F.fdk_bp(filt, ang, u, v, nx=o.img_dim, nz=o.img_dim_z, px=o.img_pix_size, pz=o.img_voxel_height,
                           cx=o.img_center_x, cy=o.img_center_y, cz=o.img_center_z, sid=o.source_isocenter_dis,
                           sdd=o.source_det_dis, dv=o.det_elem_height, img_rot=o.img_rot,
                           total_scan_angle=o.total_scan_angle, short_scan=o.short_scan, cone_beam=False)
        err = rel_l2(got, ref)
        print(f"c1 fbp {storage}/{impl}: rel-L2 {err:.3g}, max-abs/peak {_max_rel(got, ref):.3g}, "
              f"zero mismatches {int(np.sum((got == 0) != (ref == 0)))}")
        assert np.array_equal(got == 0, ref == 0), (storage, impl)
        assert err < tol, (storage, impl, err, _max_rel(got, ref))


def test_c1_two_part_filter_error_at_full_width(cuda):
    """The mixed path's two-part split-bf16 filter at 512 columns, 720 views: 6.7e-5
    relative to the float32 SIMT filter on the benchmark's noisy sinogram (bound 1e-4;
    the 28-column case of test_tc_filter_matches_simt_filter loses ~1.2e-4 to the ramp's
    cancellation); three parts below 5e-6."""
    import torch
    from reconstruction_program_taichi_gb300 import geometry, ops
    from reconstruction_program_taichi_gb300._lib import MCT_BF16, MCT_F32
    o = bench.parse(bench.C1)
    dg = geometry.fbp_geometry(o)
    taps = torch.tensor(bench.hann_from_ramp(geometry.recon_taps(o)), dtype=torch.float32, device="cuda")
    wtd = ops.weight(dg, _sino(dg, bench.C1), dg.geom.views * dg.geom.nu, dg.geom.nu)
    ref = ops.filter_rows(dg, wtd, taps)
    for dtype, tol in ((MCT_BF16, 1e-4), (MCT_F32, 5e-6)):
        tc = ops.TcFilter(dg, taps, dtype)
        got = tc(wtd)
        tc.status()
        err = float(torch.linalg.vector_norm(got - ref) / torch.linalg.vector_norm(ref))
        print(f"c1 tc filter parts={3 if dtype == MCT_F32 else 2}: rel-L2 {err:.3g}")
        assert err < tol, (dtype, err)


@pytest.fixture(scope="module")
def c2(cuda):
    """The benchmark's sinogram (20 seeded ellipsoids, exact line integrals, Poisson
    noise at 1e5 photons) on the device and on the host."""
    from reconstruction_program_taichi_gb300 import geometry
    w = bench.WORKLOAD
    o = bench.parse(w)
    dg = geometry.fbp_geometry(o)
    sgm = _sino(dg, w)
    return dict(w=w, o=o, sgm=sgm, host=sgm.cpu().numpy(), taps=bench.hann_from_ramp(geometry.recon_taps(o)))


# (storage, filter) variants of the FDK and the relative-L2 bound each must meet on
# both slabs
# (measured, central / near-end slab: tc3 2.4e-6 / 5.3e-5, simt 2.0e-6 / 5.3e-5, two-part
# filter 1.5e-5 / 5.5e-5, bf16 1.1e-4 / 3.1e-3; the near-end slab holds less of the
# phantom, so errors of the size of the sinogram's rounding weigh more there)
FDK_VARIANTS = [("f32", "tc3", TOL), ("f32", "simt", TOL), ("f32", "tc", 2e-4), ("bf16", "tc", 5e-3),
                ("f16", "tc", 2e-3)]


def test_c2_fdk_slabs_vs_float64(c2):
    import torch
    from reconstruction_program_taichi_gb300 import fbp, geometry
    o = c2["o"]
    u, v, ang = geometry.fbp_arrays(o)
    g = cpu_ref.geom_from_config(o, u, v)
    nz = o.img_dim_z
    slabs = [(nz // 2 - 4, nz // 2 + 4), (20, 24)]
    refs = [cpu_ref.fdk_slab_f64(g, ang, c2["host"], c2["taps"], z0, z1)[0] for z0, z1 in slabs]
    # the near-end slab holds voxels cleared by the break-to-zero rule, the central none
    assert (refs[1] == 0).any() and not (refs[0] == 0).any()
    for storage, impl, tol in FDK_VARIANTS:
        pipe = fbp.FdkPipeline(o, storage=storage, filter_impl=impl)
        pipe.set_taps(c2["taps"])
        vol = pipe.run(c2["sgm"])
        for (z0, z1), ref in zip(slabs, refs):
            got = vol[z0:z1].cpu().numpy()
            mism = int(np.sum((got == 0) != (ref == 0)))
            err = rel_l2(got, ref)
            print(f"c2 fdk {storage}/{impl} slices {z0}-{z1 - 1}: rel-L2 {err:.3g}, "
                  f"max-abs/peak {_max_rel(got, ref):.3g}, zero mismatches {mism}")
            assert mism == 0, (storage, impl, z0, mism)
            assert err < tol, (storage, impl, z0, err, _max_rel(got, ref))
        del pipe, vol
        torch.cuda.empty_cache()


def test_c2_forward_projection_views_vs_float64(c2):
    """The projection of the benchmark's FDK volume on 4 evenly spaced views: float32
    quad copies and direct reads within 1e-4; bf16 cells 2e-3, float16 cells 3e-4."""
    import torch
    from reconstruction_program_taichi_gb300 import fbp, geometry, ops
    from reconstruction_program_taichi_gb300._lib import MCT_BF16, MCT_F16, MCT_F32
    o = c2["o"]
    pipe = fbp.FdkPipeline(o)
    pipe.set_taps(c2["taps"])
    vol = pipe.run(c2["sgm"]).clone()
    del pipe
    dg = geometry.fpj_geometry(o)
    u, v, ang = geometry.fpj_arrays(o)
    g = cpu_ref.geom_from_config(o, u, v, dg.geom.fp_steps).copy(nv=dg.geom.nv)
    views = bench.spread(o.view_num, 4)
    ref = cpu_ref.fp_views_f64(g, ang, u, v, vol.cpu().numpy(), views)
    for dtype, ws, tol in ((MCT_F32, True, TOL), (MCT_F32, None, TOL), (MCT_BF16, True, 2e-3),
                           (MCT_F16, True, 3e-4)):
        got = ops.fp(dg, vol, workspace=ws, dtype=dtype)[:, views].cpu().numpy()
        err = rel_l2(got, ref)
        print(f"c2 fp dtype={dtype} workspace={ws}: rel-L2 {err:.3g}, max-abs/peak {_max_rel(got, ref):.3g}")
        assert np.array_equal(got == 0, ref == 0), (dtype, ws)
        assert err < tol, (dtype, ws, err, _max_rel(got, ref))
        torch.cuda.empty_cache()


@pytest.mark.parametrize("which", ["c3", "c4"])
def test_iterative_operators_at_benchmark_size_vs_float64(which, cuda):
    """The IR drivers' operators at their benchmark geometries, for each storage
    precision: the masked projector of the phantom on 4 views (float32 within 1e-4,
    16-bit cells as above) and the driver's backprojector of the masked sinogram on an
    8-slice central slab (float32 within 1e-4, bf16 operand 5e-3, float16 1e-3)."""
    import torch
    from reconstruction_program_taichi_gb300 import geometry
    from reconstruction_program_taichi_gb300.ir import Mgfbp_ir
    w = bench.C3 if which == "c3" else bench.C4
    fp_tol = {"float32": TOL, "bfloat16": 2e-3, "float16": 3e-4}
    bp_tol = {"float32": TOL, "bfloat16": 5e-3, "float16": 1e-3}
    ph = bench.phantom(w, torch.device("cuda"))
    refs = None
    for storage in ("float32", "bfloat16", "float16"):
        cfg = bench.make_config(w)
        cfg.update({"Lambda": 1e-3, "StoragePrecision": storage})
        ir = Mgfbp_ir(cfg, verbose=False)
        sy = ir.system
        g = sy.dg.geom
        views = bench.spread(g.views, 4)
        zc = g.nz // 2
        sgm = (_sino(sy.dg, w) * sy.mask).contiguous()
        if refs is None:
            u, v, ang = geometry.ir_arrays(ir)
            cz = np.asarray(ir.array_img_center_z)
            gf = cpu_ref.geom_from_config(ir, u, v, g.fp_steps).copy(nv=g.nv, cz=float(cz[0]))
            mask = sy.mask[:, views].cpu().numpy()
            fp_ref = np.where(mask == 1, cpu_ref.fp_views_f64(gf, ang, u, v, ph.cpu().numpy(), views), 0.0)
            gb = cpu_ref.geom_from_config(ir, u, v)
            bp_ref = cpu_ref.bp_unmatched_slab_f64(gb, ang, cz, sgm.cpu().numpy(), zc - 4, zc + 4)[0]
            refs = (fp_ref, bp_ref)
        got_fp = sy.fp(ph)[:, views].cpu().numpy()
        err = rel_l2(got_fp, refs[0])
        print(f"{which} ir fp {storage}: rel-L2 {err:.3g}, max-abs/peak {_max_rel(got_fp, refs[0]):.3g}")
        assert np.array_equal(got_fp == 0, refs[0] == 0), storage
        assert err < fp_tol[storage], ("fp", storage, err, _max_rel(got_fp, refs[0]))
        got_bp = sy.bp(sgm)[zc - 4:zc + 4].cpu().numpy()
        err = rel_l2(got_bp, refs[1])
        print(f"{which} ir bp {storage}: rel-L2 {err:.3g}, max-abs/peak {_max_rel(got_bp, refs[1]):.3g}, "
              f"zero mismatches {int(np.sum((got_bp == 0) != (refs[1] == 0)))}")
        assert np.array_equal(got_bp == 0, refs[1] == 0), storage
        assert err < bp_tol[storage], ("bp", storage, err, _max_rel(got_bp, refs[1]))
        del ir, sy, sgm
        torch.cuda.empty_cache()
