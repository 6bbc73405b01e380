"""Benchmark of the MandoCT hot path on GB300: cone-beam FDK + forward projection.

Workload (one step): FDK reconstruction (cosine weighting, Toeplitz ramp/Hann
filter, packing, backprojection) of a resident 1024x256x1080 sinogram into a
512x512x256 volume, then the trilinear ray-driven forward projection of that volume
back to 1080 views.  Synthetic data: 20 seeded random ellipsoids, exact line
integrals, Poisson noise at 1e5 photons.  Metric: GUPS = (voxel x view updates of
the backprojection + voxel x view equivalents of the forward projection) / s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--storage f32|bf16]
  python bench.py --impl reference ...   # the CPU implementation (OpenMP C port)
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(nu=1024, nv=256, views=1080, nx=512, nz=256, du=0.8, dv=0.8, px=0.4, pz=0.4, sid=600.0,
                sdd=1100.0, step=0.2, n_ell=20, photons=1e5, seed=2024)
SMALL = dict(WORKLOAD, nu=256, nv=64, views=270, nx=128, nz=64, du=3.2, dv=3.2, px=1.6, pz=1.6)
# profiling case for ncu: the full detector and a volume larger than L2 (168 MB), 36 views
PROF = dict(WORKLOAD, views=36, nz=160)
# the same with 180 views: enough views per detector-row tile for the projector's L2
# reuse to resemble the benchmark's (about 3.5 GB on the device)
PROF180 = dict(PROF, views=180)
# 270 views: scans of 256 views or more take the projector's 16-view ray tiles, as at
# 1080 views (about 4 GB on the device)
PROF270 = dict(PROF, views=270)
# 180 views of a 256-slice volume: the float32 backprojector's geometry-sharing kernel
# needs depths that are multiples of 128 slices, as at the benchmark (about 1.4 GB)
PROF180Z = dict(PROF180, nz=256)
WORKLOADS = {"c2": WORKLOAD, "small": SMALL, "prof": PROF, "prof180": PROF180, "prof270": PROF270,
             "prof180z": PROF180Z}


def make_config(w):
    return {"InputDir": "/tmp", "OutputDir": "/tmp/mandoct_bench", "InputFiles": "none", "OutputFilePrefix": "",
            "OutputFileReplace": ["sgm", "rec"], "DetectorElementCountHorizontal": w["nu"],
            "DetectorElementWidth": w["du"], "DetectorOffsetHorizontal": 0.0,
            "DetectorElementCountVertical": w["nv"], "DetectorElementHeight": w["dv"],
            "DetectorOffsetVertical": 0.0, "Views": w["views"], "TotalScanAngle": 360,
            "SourceIsocenterDistance": w["sid"], "SourceDetectorDistance": w["sdd"], "ImageDimension": w["nx"],
            "PixelSize": w["px"], "ImageDimensionZ": w["nz"], "VoxelHeight": w["pz"], "ConeBeam": w.get("cone", True),
            "HammingFilter": 1, "ForwardProjectionStepSize": w["step"]}


def hann_from_ramp(ramp):
    """Ramp x Hann window in the spatial domain: h = r/2 + (r[n-1] + r[n+1])/4."""
    h = 0.5 * ramp.copy()
    h[1:] += 0.25 * ramp[:-1]
    h[:-1] += 0.25 * ramp[1:]
    return h


def ellipsoids(w):
    if not w.get("cone", True):
        return ellipses(w)
    rng = np.random.default_rng(w["seed"])
    fov = w["nx"] * w["px"] / 2
    zext = w["nz"] * w["pz"] / 2
    out = []
    for _ in range(w["n_ell"]):
        r, a = 0.6 * fov * math.sqrt(rng.uniform()), rng.uniform(0, 2 * math.pi)
        ax, ay = rng.uniform(0.05, 0.4, 2) * fov
        az = rng.uniform(0.05, 0.4) * zext
        out.append([r * math.cos(a), r * math.sin(a), rng.uniform(-0.4, 0.4) * zext, ax, ay, az,
                    rng.uniform(0, math.pi), 0.0, 0.0, rng.uniform(0.01, 0.05)])
    return np.asarray(out, dtype=np.float32)


def ellipses(w):
    """2D phantom as ellipsoids infinitely long in z: centres uniform in a 50 mm disc,
    semi-axes U(5, 40) mm, angles U(0, pi), attenuation U(0.01, 0.05) /mm."""
    rng = np.random.default_rng(w["seed"])
    out = []
    for _ in range(w["n_ell"]):
        r, a = 50.0 * math.sqrt(rng.uniform()), rng.uniform(0, 2 * math.pi)
        ax, ay = rng.uniform(5.0, 40.0, 2)
        out.append([r * math.cos(a), r * math.sin(a), 0.0, ax, ay, 1e7, rng.uniform(0, math.pi), 0.0, 0.0,
                    rng.uniform(0.01, 0.05)])
    return np.asarray(out, dtype=np.float32)


def phantom(w, dev):
    """The ellipsoids of ellipsoids(w) sampled at the voxel centres of the
    reconstruction grid ([z][y][x], row 0 = +y, slice 0 = -z), float32 on dev."""
    return phantom_from(ellipsoids(w), w, dev)


def phantom_from(ell, w, dev):
    import torch
    nx, nz, px, pz = w["nx"], w["nz"], w["px"], w["pz"]
    f64 = dict(device=dev, dtype=torch.float64)
    x = ((torch.arange(nx, **f64) - (nx - 1) / 2) * px)[None, None, :]
    y = (((nx - 1) / 2 - torch.arange(nx, **f64)) * px)[None, :, None]
    z = ((torch.arange(nz, **f64) - (nz - 1) / 2) * pz)[:, None, None]
    vol = torch.zeros(nz, nx, nx, device=dev, dtype=torch.float32)
    for e in np.asarray(ell, dtype=np.float64):
        c, s_ = math.cos(e[6]), math.sin(e[6])
        qx, qy = x - e[0], y - e[1]
        r = ((qx * c + qy * s_) / e[3]) ** 2 + ((-qx * s_ + qy * c) / e[4]) ** 2 + ((z - e[2]) / e[5]) ** 2
        vol += (r <= 1.0).float() * float(e[9])
    return vol


def rmse(a, b, mask):
    import torch
    return float(torch.sqrt(((a - b)[mask].double() ** 2).mean()))


def noisy(line, photons, seed):
    """Poisson counts at `photons` incident photons, back to line integrals."""
    import torch
    gen = torch.Generator(device=line.device).manual_seed(seed)
    counts = torch.poisson(photons * torch.exp(-line.double()), generator=gen).clamp_(min=1.0)
    return torch.log(photons / counts).float().contiguous()


class Obj:
    verbose = False


def parse(w):
    from reconstruction_program_taichi_gb300 import config
    o = Obj()
    cfg = make_config(w)
    config.parse_fbp(o, cfg)
    config.parse_fpj(o, cfg)
    config.parse_fpj_v3(o, cfg)
    return o


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(value, device):
    """The largest value over all ranks (the job's time is its slowest replica's);
    the value itself when not distributed."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


# ---------------------------------------------------------------- GPU arm

def run_gpu(args, w):
    import torch
    from reconstruction_program_taichi_gb300 import _lib, fbp, geometry, ops
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    o = parse(w)
    pipe = fbp.FdkPipeline(o, device=dev, storage=args.storage)
    pipe.set_taps(hann_from_ramp(geometry.recon_taps(o)))
    fpg = geometry.fpj_geometry(o, device=dev)
    # synthetic data (not timed)
    ell = ellipsoids(w)
    sgm = noisy(ops.project_ellipsoids(pipe.dg, ell), w["photons"], w["seed"])
    fp_out = torch.empty(fpg.sgm_shape, dtype=torch.float32, device=dev)
    fp_dtype = {"f32": ops.MCT_F32, "bf16": ops.MCT_BF16, "f16": ops.MCT_F16}[args.storage]
    stream = torch.cuda.current_stream(dev)

    def step(evs=None):
        if evs:
            evs[0].record(stream)
        filt = pipe.filter(sgm)
        if evs:
            evs[1].record(stream)
        packed = ops.pack(pipe.dg, filt, pipe.dtype, out=pipe.packed)
        if evs:
            evs[2].record(stream)
        vol = ops.fdk_bp(pipe.dg, packed, pipe.dtype, out=pipe.vol)
        if evs:
            evs[3].record(stream)
        ops.fp(fpg, vol, out=fp_out, dtype=fp_dtype)
        if evs:
            evs[4].record(stream)
        return vol

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(args.warmup):
        step()
    barrier()
    nstage = 5
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(nstage)] for _ in range(args.steps)]
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = _lib.launch_count()
    with ClockSampler(local) as clk:
        barrier()
        t_start.record(stream)
        for k in range(args.steps):
            step(evs[k])
        t_end.record(stream)
        barrier()
    launches = _lib.launch_count() - launches0
    total_ms = t_start.elapsed_time(t_end)
    total_ms = max_over_ranks(total_ms, dev)
    ms = total_ms / args.steps
    stage = np.array([[evs[k][i].elapsed_time(evs[k][i + 1]) for i in range(nstage - 1)] for k in range(args.steps)])
    st = stage.mean(axis=0)  # filter, pack, bp, fp
    nvox = w["nx"] * w["nx"] * w["nz"]
    units = 2.0 * nvox * w["views"] * world
    value = units / (ms / 1e3) / 1e9

    # rooflines of the two gather kernels.  "achieved" counts the compulsory bytes of a
    # launch (its operand read once, its output written once) against the measured HBM
    # copy bandwidth; "dram" the DRAM bytes ncu measured per launch (a committed
    # profile, workload and scaling stated there) over this run's launch time; "on_chip"
    # the binding on-chip unit from the same profile; "gather" the bytes the kernel's
    # loads deliver (served by L1 and L2), the per-update figure of the operator.
    hbm, _, peak_kind = peaks()
    n_samples = ops.fp_count_samples(fpg)
    prof = {}
    pj = os.path.join(ROOT, "profiles", "roofline_inputs.json")
    if os.path.exists(pj):
        prof = json.load(open(pj))
    nvox = w["nx"] * w["nx"] * w["nz"]
    g_fdk = pipe.dg.geom
    cells = g_fdk.views * g_fdk.nv * (g_fdk.nu - 1)  # (nv - 1) cell rows + one NaN row per view
    bp_elem = 16 if pipe.dtype == ops.MCT_F32 else 8
    fp_rays = fpg.geom.nv * fpg.geom.views * fpg.geom.nu
    kern = {
        "fp_kernel": dict(ms=float(st[3]), compulsory=nvox * 32 + fp_rays * 4,
                          gather=n_samples * (32 if fp_dtype == ops.MCT_F32 else 16),
                          what="copies of the volume (32 B per voxel, both orientations) read once, the "
                               "projection written once; gathers: one 32-byte (16-bit: 16-byte) cell per "
                               "in-volume sample"),
        "fdk_bp_kernel": dict(ms=float(st[2]), compulsory=cells * bp_elem + nvox * 4,
                              gather=nvox * w["views"] * bp_elem,
                              what="packed operand (16 B float32 / 8 B 16-bit per detector cell) read once, the "
                                   "volume written once; gathers: one coefficient cell per voxel x view update"),
    }

    def kernel_roofline(name):
        k = kern[name]
        sec = k["ms"] / 1e3
        ach = k["compulsory"] / sec / 1e9
        out = {"kernel": name, "bound": "hbm", "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
               "frac": round(ach / hbm, 4), "traffic": None, "peak_source": peak_kind,
               "algorithmic_bytes": int(k["compulsory"]), "algorithmic": k["what"],
               "gather": {"bytes_per_launch": int(k["gather"]), "tb_per_s": round(k["gather"] / sec / 1e12, 2)}}
        pk = prof.get(name, {})
        if pk.get("dram_bytes_per_launch") and args.storage == "f32" and w is WORKLOAD:
            t = float(pk["dram_bytes_per_launch"])
            out["traffic"] = int(t)
            out["dram"] = {"gb_per_s": round(t / sec / 1e9, 1), "frac": round(t / sec / 1e9 / hbm, 4),
                           "source": pk.get("source")}
        if pk.get("on_chip"):
            out["on_chip"] = pk["on_chip"]
        return out

    dom = "fp_kernel" if st[3] >= st[2] else "fdk_bp_kernel"
    roofline = kernel_roofline(dom)
    roofline_other = kernel_roofline("fdk_bp_kernel" if dom == "fp_kernel" else "fp_kernel")

    # end to end through the public API: pinned host sinogram in, volume + projections
    # out, every step's copies inside the timed region; consecutive steps run through
    # stream.ScanStream, which overlaps step i+1's upload and step i-1's download with
    # step i's compute
    from reconstruction_program_taichi_gb300.stream import ScanStream
    host_sgm = torch.empty(sgm.shape, dtype=torch.float32, pin_memory=True)
    host_sgm.copy_(sgm.cpu())
    host_vol = torch.empty(pipe.vol.shape, dtype=torch.float32, pin_memory=True)
    host_fp = torch.empty(fp_out.shape, dtype=torch.float32, pin_memory=True)
    scans = ScanStream(pipe, fpg, fp_dtype)
    for _ in range(max(1, args.warmup // 2)):
        scans.submit(host_sgm, host_vol, host_fp)
    scans.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(scans.up)  # the first work of a step is its upload
    for _ in range(args.steps):
        scans.submit(host_sgm, host_vol, host_fp)
    e1.record(scans.down)  # the last is its download
    scans.synchronize()
    barrier()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e2e = {"value": round(units / (e2e_ms / 1e3) / 1e9, 3), "unit": "GUPS", "ms_per_step": round(e2e_ms, 3),
           "h2d_bytes_per_step": int(host_sgm.numel() * 4),
           "d2h_bytes_per_step": int(host_vol.numel() * 4 + host_fp.numel() * 4)}

    # accuracy against the float64 restatement of the same operators (evaluated in the
    # CPU leg, after every timed region): a central 8-slice slab of the FDK volume with
    # every view, and 4 evenly spaced views of the projection, for every variant
    checks = Fp64Checks() if (rank == 0 and world == 1 and not args.no_cpu) else None
    accuracy = {"fdk": {}, "fp": {}}
    ref_vol = pipe.run(sgm).clone()
    ref_fp = ops.fp(fpg, ref_vol, dtype=fp_dtype).clone()
    z0, z1 = w["nz"] // 2 - 4, w["nz"] // 2 + 4
    fp_views = spread(w["views"], 4)
    if checks is not None:
        sgm_host = sgm.cpu().numpy()
        vol_host = ref_vol.cpu().numpy()
        taps64 = hann_from_ramp(geometry.recon_taps(o))
        checks.fdk_slab(accuracy["fdk"], args.storage, o, sgm_host, taps64, z0, z1, vol_host[z0:z1])
        checks.fp_views(accuracy["fp"], args.storage, o, vol_host, fp_views, ref_fp[:, fp_views].cpu().numpy())

    # mixed precision: tensor-core split-bf16 filter, bf16 backprojection operand, bf16
    # forward-projection cells; the whole step, then FDK-only variants
    mixed = None
    # the mixed-precision, 2D, iterative and widened sections run in single-GPU runs
    # (they do not enter the metric; with several ranks they would only repeat per rank)
    if args.storage == "f32" and not args.no_mixed and world == 1:
        plain_ms = float(st[0] + st[1] + st[2])
        mixed = {"fdk_plain_ms": round(plain_ms, 3)}
        pm = fbp.FdkPipeline(o, device=dev, storage="bf16", filter_impl="tc")
        pm.set_taps(pipe.taps.cpu().numpy())
        fp_m = torch.empty_like(fp_out)

        def mixed_step():
            vol = pm.run(sgm)
            ops.fp(fpg, vol, out=fp_m, dtype=ops.MCT_BF16)
            return vol

        for _ in range(args.warmup):
            mixed_step()
        barrier()
        m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        m0.record(stream)
        for _ in range(args.steps):
            mv = mixed_step()
        m1.record(stream)
        barrier()
        pm.tc.status()
        mms = m0.elapsed_time(m1) / args.steps
        ph = phantom(w, dev)
        live = ref_vol != 0
        r_plain, r_mixed = rmse(ref_vol, ph, live), rmse(mv, ph, live)
        mixed["step"] = {
            "ms_per_step": round(mms, 3), "gups": round(units / (mms / 1e3) / 1e9, 3),
            "speedup_vs_plain": round(ms / mms, 3),
            "fdk_rmse_vs_phantom": {"plain": r_plain, "mixed": r_mixed, "ratio": round(r_mixed / r_plain, 5)},
            "fdk_rel_l2_vs_plain": float(torch.linalg.vector_norm(mv - ref_vol) / torch.linalg.vector_norm(ref_vol)),
            "fp_rel_l2_vs_plain": float(torch.linalg.vector_norm(fp_m - ref_fp) / torch.linalg.vector_norm(ref_fp)),
            "storage": "two-part split-bf16 tcgen05 row filter; bf16 backprojection coefficients; bf16 FP cells",
        }
        if checks is not None:
            checks.fdk_slab(mixed["step"], "fdk", o, sgm_host, taps64, z0, z1, mv[z0:z1].cpu().numpy())
            # the projector's own error: 16-bit cells of the plain FDK volume
            for name, dt in (("fp_bf16_cells", ops.MCT_BF16), ("fp_f16_cells", ops.MCT_F16)):
                mixed[name] = {}
                got = ops.fp(fpg, ref_vol, dtype=dt)[:, fp_views].cpu().numpy()
                checks.fp_views(mixed[name], "fp", o, vol_host, fp_views, got)
        del pm, ph, live, fp_m
        for name, storage, impl in (("simt_filter_f32", "f32", "simt"), ("tc2_filter_f32", "f32", "tc"),
                                    ("tc2_filter_bf16_bp", "bf16", "tc"), ("tc2_filter_f16_bp", "f16", "tc")):
            pm = fbp.FdkPipeline(o, device=dev, storage=storage, filter_impl=impl)
            pm.set_taps(pipe.taps.cpu().numpy())
            for _ in range(2):
                mv = pm.run(sgm)
            barrier()
            m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            m0.record(stream)
            for _ in range(args.steps):
                mv = pm.run(sgm)
            m1.record(stream)
            f0.record(stream)
            pm.filter(sgm)
            f1.record(stream)
            barrier()
            if pm.tc is not None:
                pm.tc.status()
            mms = m0.elapsed_time(m1) / args.steps
            rel = float(torch.linalg.vector_norm(mv - ref_vol) / torch.linalg.vector_norm(ref_vol))
            mixed[name] = {"fdk_ms": round(mms, 3), "weight_filter_ms": round(f0.elapsed_time(f1), 3),
                           "speedup_fdk": round(plain_ms / mms, 3), "rel_l2_vs_plain": rel}
            if checks is not None:
                checks.fdk_slab(mixed[name], "fdk", o, sgm_host, taps64, z0, z1, mv[z0:z1].cpu().numpy())
            del pm

    cgls = piccs = c1 = served = None
    if w is WORKLOAD and not args.no_mixed and world == 1:
        c1 = c1_bench(dev, stream, barrier, checks)
    widened = None
    if not args.no_cgls and w is WORKLOAD and world == 1:
        cgls = irn_bench(dev, stream, barrier, checks)
        piccs = piccs_bench(dev, stream, barrier, checks)
        widened = widen_bench(dev, stream, barrier)
    if not args.no_serve and w is WORKLOAD and world == 1:
        del pipe, fpg, sgm, fp_out, scans, host_sgm, host_vol, host_fp, ref_vol, ref_fp
        torch.cuda.empty_cache()
        served = serve_bench(dev)

    # CPU leg (after every timed region): the timed CPU baseline, then the float64
    # checks of the results collected above
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(w, o, budget_s=args.cpu_seconds)
        cpu["fp64_checks_s"] = round(checks.run(), 2)

    if rank == 0:
        line = {
            "metric": "GUPS (cone-beam FDK + forward projection, voxel x view updates per second)",
            "value": round(value, 3), "unit": "GUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.storage == "f32" else f"{args.storage}-storage/f32-compute",
            "data": "synthetic: 20 seeded ellipsoids, exact line integrals, Poisson noise at 1e5 photons",
            "config": {"workload": f"FDK+FP {w['nx']}x{w['nx']}x{w['nz']} vol @{w['px']}mm, {w['views']} views/360deg, "
                                   f"{w['nu']}x{w['nv']} flat det @{w['du']}mm, SID {w['sid']:.0f} SDD {w['sdd']:.0f}",
                       "filter": "ramp x Hann (spatial composition of the reference ramp); Toeplitz row product on "
                                 "tcgen05 tensor cores from three bf16 parts per float32 operand (~1e-6 of float32); "
                                 "the mixed step uses two parts",
                       "fp_step": w["step"], "l2": "inputs larger than L2 (sinogram 1.13 GB, volume 268 MB)",
                       "parallelism": "replicas only" if world > 1 else "single GPU"},
            "stages_ms": {"weight_filter": round(float(st[0]), 3), "pack": round(float(st[1]), 3),
                          "backproject": round(float(st[2]), 3), "forward_project": round(float(st[3]), 3)},
            "fdk_gups": round(nvox * w["views"] / ((st[0] + st[1] + st[2]) / 1e3) / 1e9, 2),
            "bp_gups": round(nvox * w["views"] / (st[2] / 1e3) / 1e9, 2),
            "fp_gups": round(nvox * w["views"] / (st[3] / 1e3) / 1e9, 2),
            "fp_samples_per_s": round(n_samples / (st[3] / 1e3), 1), "fp_in_volume_samples": n_samples,
            "roofline": roofline, "roofline_second_kernel": roofline_other, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk.summary(), "mixed": mixed, "irn_cgls_tv": cgls, "irn_cgls_piccs": piccs,
            "fbp_2d_fan": c1, "serving": served, "widened": widened, "accuracy": accuracy,
        }
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


C3 = dict(nu=1024, nv=64, views=360, nx=512, nz=64, du=0.8, dv=0.8, px=0.4, pz=0.4, sid=600.0, sdd=1100.0,
          step=0.2, n_ell=20, photons=1e5, seed=2025)
# 2D fan-beam FBP: 256x256 at 0.5 mm, 720 views, 512 bins at 0.8 mm, SID 500 / SDD 1000, 10 ellipses
C1 = dict(cone=False, nu=512, nv=1, views=720, nx=256, nz=1, du=0.8, dv=0.8, px=0.5, pz=0.5, sid=500.0,
          sdd=1000.0, step=0.2, n_ell=10, photons=1e5, seed=2023)
# IRN-CGLS-PICCS: 512x512x128 at 0.4 mm, 1024x128 detector; prior from 1440 views, target 90 views
C4 = dict(nu=1024, nv=128, views=90, nx=512, nz=128, du=0.8, dv=0.8, px=0.4, pz=0.4, sid=600.0, sdd=1100.0,
          step=0.2, n_ell=20, photons=1e5, seed=2026)


def c1_bench(dev, stream, barrier, checks=None, reps=50):
    """2D fan-beam FBP, plain and mixed: GUPS, error vs plain, RMSE vs the phantom, and
    (checks) the whole image against the float64 restatement of the same FBP."""
    import torch
    from reconstruction_program_taichi_gb300 import fbp, geometry, ops
    o = parse(C1)
    out = {"config": "2D fan FBP 256x256 @0.5mm, 720 views, 512 bins @0.8mm, SID 500 SDD 1000, ramp x Hann, "
                     "10 ellipses, Poisson 1e5"}
    ph = phantom(C1, dev)
    ref = None
    for name, storage, impl in (("plain", "f32", "tc3"), ("mixed", "bf16", "tc")):
        pipe = fbp.FdkPipeline(o, device=dev, storage=storage, filter_impl=impl)
        pipe.set_taps(hann_from_ramp(geometry.recon_taps(o)))
        sgm = noisy(ops.project_ellipsoids(pipe.dg, ellipsoids(C1)), C1["photons"], C1["seed"])
        for _ in range(5):
            vol = pipe.run(sgm)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            vol = pipe.run(sgm)
        e1.record(stream)
        barrier()
        ms = e0.elapsed_time(e1) / reps
        live = vol != 0
        r = {"ms": round(ms, 4), "gups": round(C1["nx"] ** 2 * C1["views"] / (ms / 1e3) / 1e9, 2),
             "rmse_vs_phantom": rmse(vol, ph, live)}
        if ref is None:
            ref = vol.clone()
        else:
            r["rel_l2_vs_plain"] = float(torch.linalg.vector_norm(vol - ref) / torch.linalg.vector_norm(ref))
        if checks is not None:
            checks.fdk_slab(r, "fbp", o, sgm.cpu().numpy(), hann_from_ramp(geometry.recon_taps(o)), 0, 1,
                            vol.cpu().numpy())
        out[name] = r
    return out


def ir_operator_checks(checks, target, ir, sy, sgm, ph, zc):
    """Queue the FP64 checks of one IR system's operators at its storage precision:
    the masked projector on 4 evenly spaced views of the phantom, and the driver's
    backprojector of the masked measured sinogram on an 8-slice central slab."""
    if checks is None:
        return
    g = sy.dg.geom
    views = spread(g.views, 4)
    vol = ph.cpu().numpy()
    got = sy.fp(ph)[:, views].cpu().numpy()
    checks.fp_views(target, "fp", ir, vol, views, got, mask=sy.mask[:, views].cpu().numpy(), ir=True)
    sm = (sgm * sy.mask).contiguous()
    bp = sy.bp(sm)
    checks.bp_unmatched_slab(target, "bp", ir, sm.cpu().numpy(), zc - 4, zc + 4, bp[zc - 4:zc + 4].cpu().numpy())


def irn_bench(dev, stream, barrier, checks=None):
    """IRN-CGLS-TV, 20 reweightings x 10 CG iterations (the reference driver's loop,
    run_mgfbp_iterative_recon_IRN_CGLS.py:157-172) on 512x512x64 @0.4 mm, 360 views,
    1024x64 detector, lambda 1e-3, beta_TV 1e-6, with the reference operator pair
    (masked FP + voxel-driven backprojector), from a zero start, for float32 and bf16
    gather storage: seconds per P^T P iteration and RMSE vs the phantom."""
    import torch
    from reconstruction_program_taichi_gb300 import ops
    from reconstruction_program_taichi_gb300.ir import Mgfbp_ir
    out = {"config": "512x512x64 @0.4mm, 360 views, 1024x64 det, lambda 1e-3, beta_TV 1e-6, 20 IRN x 10 CG "
                     "(231 P^T P), zero start, Poisson 1e5",
           "operator": "reference pair (masked FP + per-view BP)"}
    ph = None
    # (result key, gather storage, measured-sinogram storage); "float16_sinogram" is the
    # configuration's own precision plan: the measured sinogram stored in FP16, the
    # operator applications on 16-bit (bf16) gathers, float32 accumulation, float64 CG
    # scalars
    variants = (("float32", "float32", "float32"), ("bfloat16", "bfloat16", "float32"),
                ("float16", "float16", "float32"), ("float16_sinogram", "bfloat16", "float16"))
    for key, storage, sino in variants:
        cfg = make_config(C3)
        cfg.update({"Lambda": 1e-3, "BetaTV": 1e-6, "NumberOfIRNIterations": 20, "NumberOfIterations": 10,
                    "StoragePrecision": storage, "SinogramPrecision": sino})
        ir = Mgfbp_ir(cfg, device=dev, verbose=False)
        sy = ir.system
        sgm = noisy(ops.project_ellipsoids(sy.dg, ellipsoids(C3)), C3["photons"], C3["seed"])
        x0 = torch.zeros(sy.dg.vol_shape, dtype=torch.float32, device=dev)
        sy.bpb = sy.bp_b(sgm)
        sy.cgls(x0, [], [(1e-3, torch.ones_like(x0))], 2)  # warm-up
        barrier()
        calls0 = sy.ptp_calls
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        x = ir.solve_tv(sgm, x0)
        e1.record(stream)
        barrier()
        n = sy.ptp_calls - calls0
        sec = e0.elapsed_time(e1) / 1e3
        if ph is None:
            ph = phantom(C3, dev)
            n_ = C3["nx"]
            yy, xx = torch.meshgrid(torch.arange(n_, device=dev) - (n_ - 1) / 2,
                                    torch.arange(n_, device=dev) - (n_ - 1) / 2, indexing="ij")
            fov = (yy ** 2 + xx ** 2 <= (0.95 * n_ / 2) ** 2).expand_as(ph).contiguous()
        out[key] = {"s_total": round(sec, 3), "ptp": n, "s_per_iter": round(sec / n, 5),
                    "rmse_vs_phantom": rmse(x, ph, fov), "finite": bool(torch.isfinite(x).all()),
                    "gather_storage": storage, "sinogram_storage": sino}
        if key != "float16_sinogram":
            ir_operator_checks(checks, out[key], ir, sy, sgm, ph, C3["nz"] // 2)
        del ir, sy, sgm, x
    f = out["float32"]
    for k in ("bfloat16", "float16", "float16_sinogram"):
        out[k]["speedup"] = round(f["s_total"] / out[k]["s_total"], 3)
        out[k]["rmse_ratio"] = round(out[k]["rmse_vs_phantom"] / f["rmse_vs_phantom"], 5)
    return out


def piccs_bench(dev, stream, barrier, checks=None):
    """IRN-CGLS-PICCS (alpha 0.5, lambda 1e-3, 30 reweightings x 8 CG iterations) on
    512x512x128 @0.4 mm with a 1024x128 detector: prior = FDK of 1440 views of phantom
    A, target = 90 views of A plus 3 extra seeded ellipsoids; float32 and bf16 gather
    storage; seconds and RMSE vs the target phantom."""
    import torch
    from reconstruction_program_taichi_gb300 import fbp, geometry, io, ops
    from reconstruction_program_taichi_gb300.ir import Mgfbp_ir_piccs
    w_prior = dict(C4, views=1440)
    o = parse(w_prior)
    pipe = fbp.FdkPipeline(o, device=dev)
    pipe.set_taps(hann_from_ramp(geometry.recon_taps(o)))
    ell_a = ellipsoids(C4)
    prior = pipe.run(noisy(ops.project_ellipsoids(pipe.dg, ell_a), C4["photons"], C4["seed"])).clone()
    del pipe
    prior_file = os.path.join("/tmp", f"mandoct_bench_prior_{os.getpid()}.raw")
    io.imwriteRaw(prior.cpu().numpy(), prior_file)
    ell_t = np.concatenate([ell_a, ellipsoids(dict(C4, n_ell=3, seed=C4["seed"] + 1))])
    truth = phantom(dict(C4), dev)
    truth += phantom_from(ell_t[len(ell_a):], C4, dev)
    out = {"config": "512x512x128 @0.4mm, 1024x128 det, target 90 views, prior FDK of 1440 views, alpha 0.5, "
                     "lambda 1e-3, 30 IRN x 8 CG, Poisson 1e5",
           "prior_rmse_vs_target": None}
    n_ = C4["nx"]
    yy, xx = torch.meshgrid(torch.arange(n_, device=dev) - (n_ - 1) / 2, torch.arange(n_, device=dev) - (n_ - 1) / 2,
                            indexing="ij")
    fov = (yy ** 2 + xx ** 2 <= (0.95 * n_ / 2) ** 2).expand_as(truth).contiguous()
    out["prior_rmse_vs_target"] = rmse(prior, truth, fov)
    # (result key, gather storage, iterate storage); "bf16_iterates" is the configuration's
    # own precision plan: BF16 iterates, float64 reductions
    variants = (("float32", "float32", "float32"), ("bfloat16", "bfloat16", "float32"),
                ("float16", "float16", "float32"), ("bf16_iterates", "bfloat16", "bfloat16"))
    try:
        for key, storage, iterate in variants:
            cfg = make_config(C4)
            cfg.update({"Lambda": 1e-3, "BetaTV": 1e-6, "NumberOfIRNIterations": 30, "NumberOfIterations": 8,
                        "Alpha": 0.5, "PriorImageFile": prior_file, "StoragePrecision": storage,
                        "IterateStorage": iterate})
            ir = Mgfbp_ir_piccs(cfg, device=dev, verbose=False)
            sy = ir.system
            sgm = noisy(ops.project_ellipsoids(sy.dg, ell_t), C4["photons"], C4["seed"] + 7)
            pr = torch.from_numpy(ir.img_prior.copy()).to(dev)
            sy.bpb = sy.bp_b(sgm)
            sy.cgls(pr, [], [(1e-3, torch.ones_like(pr))], 2)  # warm-up
            barrier()
            calls0 = sy.ptp_calls
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            x = ir.solve_piccs(sgm, pr)
            e1.record(stream)
            barrier()
            n = sy.ptp_calls - calls0
            sec = e0.elapsed_time(e1) / 1e3
            out[key] = {"s_total": round(sec, 3), "ptp": n, "s_per_iter": round(sec / n, 5),
                        "rmse_vs_phantom": rmse(x, truth, fov), "finite": bool(torch.isfinite(x).all()),
                        "gather_storage": storage, "iterate_storage": iterate}
            if key != "bf16_iterates":
                ir_operator_checks(checks, out[key], ir, sy, sgm, truth, C4["nz"] // 2)
            del ir, sy, sgm, x, pr
    finally:
        os.remove(prior_file)
    f = out["float32"]
    for k in ("bfloat16", "float16", "bf16_iterates"):
        out[k]["speedup"] = round(f["s_total"] / out[k]["s_total"], 3)
        out[k]["rmse_ratio"] = round(out[k]["rmse_vs_phantom"] / f["rmse_vs_phantom"], 5)
    return out


def widen_bench(dev, stream, barrier):
    """The widened drop-ins on the benchmark geometry, timed with CUDA events on
    synthetic data (their cost does not depend on the data): the view-streaming FBP of
    the benchmark sinogram held in host memory (Mgfbp_v2, chunks of views copied while
    earlier chunks compute), the helical FBP by rebinning (Mgfbp_helical, three
    rounds at pitch 1 on a 1024 x 64 detector) and ADMM-TV (5 x 10, the C3 size)."""
    import tempfile
    import torch
    from reconstruction_program_taichi_gb300 import geometry, ops
    from reconstruction_program_taichi_gb300.admm import Mgfbp_ir_admm
    from reconstruction_program_taichi_gb300.fbp import Mgfbp_v2
    from reconstruction_program_taichi_gb300.helical import Mgfbp_helical
    rng = np.random.default_rng(5)
    out = {}

    def timed(fn):
        fn()  # warm-up
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = fn()
        e1.record(stream)
        barrier()
        return r, e0.elapsed_time(e1)

    w = WORKLOAD
    v2 = Mgfbp_v2(make_config(w), device=dev, verbose=False, views_per_chunk=120)
    v2._raw = rng.uniform(0, 1, (w["nv"], w["views"], w["nu"])).astype(np.float32)
    v2._view_stride = w["nu"]
    pipe = v2.pipeline
    pipe.set_taps(hann_from_ramp(geometry.recon_taps(v2)))
    _, ms = timed(lambda: v2._stream_file(pipe))
    nvox = w["nx"] * w["nx"] * w["nz"]
    out["fbp_view_streaming"] = {
        "config": "FDK 512x512x256 from a host sinogram (1.13 GB) in chunks of 120 views, copies inside the timing",
        "ms": round(ms, 3), "gups": round(nvox * w["views"] / (ms / 1e3) / 1e9, 2)}
    del v2, pipe
    torch.cuda.empty_cache()

    hcfg = make_config(dict(w, nv=64, views=2160))
    hcfg.update(TotalScanAngle=1080, HelicalPitch=1.0)
    hel = Mgfbp_helical(hcfg, device=dev, verbose=False)
    sgm = torch.from_numpy(rng.uniform(0, 1, (64, 2160, w["nu"])).astype(np.float32)).to(dev)
    vol, ms = timed(lambda: hel.reconstruct(sgm, save_rebinned=False))
    nz = vol.shape[0]
    out["helical_fbp"] = {
        "config": "helical, 1024x64 det @0.8mm, 3 rounds x 720 views, pitch 1.0, 512x512 slices @0.4mm",
        "slices": nz, "views_per_slice": hel.view_count, "ms": round(ms, 3), "ms_per_slice": round(ms / nz, 4),
        "gups": round(w["nx"] * w["nx"] * nz * hel.view_count / (ms / 1e3) / 1e9, 2)}
    del hel, sgm, vol
    torch.cuda.empty_cache()

    with tempfile.TemporaryDirectory() as d:
        prior = os.path.join(d, "prior.raw")
        np.zeros((C3["nz"], C3["nx"], C3["nx"]), np.float32).tofile(prior)
        cfg = make_config(C3)
        cfg.update(Lambda=1e-3, BetaTV=1e-6, NumberOfIRNIterations=5, NumberOfIterations=10, Alpha=0.5,
                   PriorImageFile=prior)
        adm = Mgfbp_ir_admm(cfg, device=dev, verbose=False)
    sy = adm.system
    sgm3 = noisy(ops.project_ellipsoids(sy.dg, ellipsoids(C3)), C3["photons"], C3["seed"])
    x0 = torch.zeros(sy.dg.vol_shape, dtype=torch.float32, device=dev)
    calls = []

    def admm():
        c0 = sy.ptp_calls
        x = adm.solve_admm(sgm3, x0)
        calls.append(sy.ptp_calls - c0)
        return x

    _, ms = timed(admm)
    out["admm_tv"] = {"config": "ADMM-TV 5 x 10 CG, 512x512x64 @0.4mm, 360 views, 1024x64 det, rho 0.1",
                      "s_total": round(ms / 1e3, 3), "ptp": calls[-1], "s_per_ptp": round(ms / 1e3 / calls[-1], 5)}
    del adm, sy, sgm3, x0
    out["fp_adjoint_pair"] = adjoint_pair_bench(dev, stream, barrier)
    torch.cuda.empty_cache()

    # FDK with the run_mgfbp options, benchmark sizes, one sinogram on the device
    from reconstruction_program_taichi_gb300 import config as mcfg
    from reconstruction_program_taichi_gb300.fbp import FdkPipeline

    class _Obj:
        verbose = False

    opts = {"curved": {"CurvedDetector": True}, "short_scan_220deg": {"TotalScanAngle": 220},
            "coronal": {"ReconViewMode": "coronal"}, "sagittal": {"ReconViewMode": "sagittal"},
            "pmatrix": {}, "pmatrix_coronal": {"ReconViewMode": "coronal"}}
    res = {}
    sgm = torch.from_numpy(rng.uniform(0, 1, (w["nv"], w["views"], w["nu"])).astype(np.float32)).to(dev)
    with tempfile.TemporaryDirectory() as d:
        for name, extra in opts.items():
            cfg = make_config(w)
            if name.startswith("pmatrix"):
                path = os.path.join(d, "pmatrix.jsonc")
                with open(path, "w") as f:
                    json.dump({"Value": [float(x) for x in circular_pmatrices(w)]}, f)
                cfg["PMatrixFile"] = path
            cfg.update(extra)
            o = _Obj()
            mcfg.parse_fbp(o, cfg)
            pipe = FdkPipeline(o, device=dev)
            _, ms = timed(lambda: pipe.run(sgm))
            res[name] = {"ms": round(ms, 3), "gups": round(nvox * w["views"] / (ms / 1e3) / 1e9, 2)}
            del pipe
            torch.cuda.empty_cache()
    out["fdk_options"] = dict(config="FDK 512x512x256, 1080 views, 1024x256 det, device-resident sinogram", **res)
    del sgm
    torch.cuda.empty_cache()
    return out


def cg_step_bench(dev, storage="float32"):
    """One TV reweighting and a 3-iteration CG solve at the C3 geometry (gathers stored
    as `storage`): the CG kernels (projector, backprojector, TV weights, stencil and
    inner product -- in the backprojector's epilogue with 16-bit gathers -- vector
    updates) launched a few times each.  Returns the solve's milliseconds."""
    import torch
    from reconstruction_program_taichi_gb300 import ops
    from reconstruction_program_taichi_gb300.ir import Mgfbp_ir
    cfg = make_config(C3)
    cfg.update({"Lambda": 1e-3, "BetaTV": 1e-6, "StoragePrecision": storage})
    ir = Mgfbp_ir(cfg, device=dev, verbose=False)
    sy = ir.system
    sgm = noisy(ops.project_ellipsoids(sy.dg, ellipsoids(C3)), C3["photons"], C3["seed"])
    x0 = phantom(C3, dev)
    sy.bpb = sy.bp_b(sgm)
    wr = ops.tv_weights(sy.dg, x0, 1e-6)
    lr = 1e-3 * ir.pixel_count_ratio
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    sy.cgls(x0, [], [(lr, wr)], 3)
    e1.record()
    torch.cuda.synchronize()
    return round(e0.elapsed_time(e1), 3)


def helical_once(dev):
    """One helical FBP by rebinning (1024x64 detector, 3 rounds x 720 views, pitch 1,
    512x512 slices); returns its milliseconds."""
    import torch
    from reconstruction_program_taichi_gb300.helical import Mgfbp_helical
    w = WORKLOAD
    hcfg = make_config(dict(w, nv=64, views=2160))
    hcfg.update(TotalScanAngle=1080, HelicalPitch=1.0)
    hel = Mgfbp_helical(hcfg, device=dev, verbose=False)
    g = torch.Generator(device=dev).manual_seed(5)
    sgm = torch.rand((64, 2160, w["nu"]), device=dev, generator=g)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    hel.reconstruct(sgm, save_rebinned=False)
    e1.record()
    torch.cuda.synchronize()
    return round(e0.elapsed_time(e1), 3)


def adjoint_pair_bench(dev, stream, barrier):
    """The autograd pair at 512x512x64, 360 views: the projector and its exact adjoint,
    which scatters through the cell-space buffer (default) or straight into the volume."""
    import torch
    from reconstruction_program_taichi_gb300 import geometry, ops
    dg = geometry.fpj_geometry(parse(C3), device=dev)
    g = torch.Generator(device=dev).manual_seed(C3["seed"])
    xs = torch.rand(dg.vol_shape, device=dev, generator=g)
    ys = torch.rand(dg.sgm_shape, device=dev, generator=g)

    def timed(fn):
        fn()  # warm-up
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        barrier()
        return e0.elapsed_time(e1)

    ms_ad = timed(lambda: ops.fp_adjoint(dg, ys))
    ms_ad_direct = timed(lambda: ops.fp_adjoint(dg, ys, workspace=None))
    ms_fp = timed(lambda: ops.fp(dg, xs))
    return {"config": "512x512x64 @0.4mm, 360 views, 1024x64 det, no mask", "fp_ms": round(ms_fp, 3),
            "adjoint_ms": round(ms_ad, 3), "adjoint_direct_scatter_ms": round(ms_ad_direct, 3)}


def circular_pmatrices(w):
    """3x4 projection matrices of the benchmark's circular scan, P_j = [e_u e_v d]^-1
    [I | -s]: source s at angle 2 pi j / views on the circle of radius SID, flat
    detector at SDD with pixel vectors e_u, e_v, centred.  Flattened, 12 per view."""
    out = []
    for j in range(w["views"]):
        b = 2 * np.pi * j / w["views"]
        c, s_ = np.cos(b), np.sin(b)
        src = np.array([w["sid"] * c, w["sid"] * s_, 0.0])
        e_u = w["du"] * np.array([s_, -c, 0.0])
        e_v = w["dv"] * np.array([0.0, 0.0, -1.0])
        origin = src - w["sdd"] * np.array([c, s_, 0.0]) - (w["nu"] - 1) / 2 * e_u - (w["nv"] - 1) / 2 * e_v
        m = np.linalg.inv(np.stack([e_u, e_v, origin - src], axis=1))
        out.append(np.concatenate([m, (-m @ src)[:, None]], axis=1).reshape(-1))
    return np.concatenate(out)


def serve_bench(dev, n_req=256, seed=7, mean_gap_ms=150.0, n_sat=96):
    """Serving stream: n_req requests with Poisson arrivals (seeded), mixing 2D fan FBP
    (256^2-1024^2, 360-1440 views), cone-beam FDK (256^3-512^3, 360-1080 views) and
    10-iteration CGLS at 256^3, under a 150 GB HBM budget; sinograms resident on the
    device (as written by an acquisition pipeline), results returned as device tensors.
    Run for the plain float32 path and the mixed-precision path (two-part tensor-core
    filter with bf16 backprojection coefficients; bf16 projector cells in CGLS): p50/p99
    latency, GUPS, and per request class the RMSE of the result against its phantom.
    Then a saturated run of each (its slots built first by one request per class, then
    n_sat requests submitted at once): the GUPS the server sustains with the GPU kept
    busy."""
    import torch
    from reconstruction_program_taichi_gb300 import config, geometry, ops
    from reconstruction_program_taichi_gb300.serve import ReconServer
    rng = np.random.default_rng(seed)
    classes = []
    for n in (256, 512, 1024):
        for v in (360, 720, 1440):
            classes.append(("fbp", dict(C1, nx=n, px=128.0 / n, nu=2 * n, du=0.8 * 256 / n, views=v, seed=seed + n + v)))
    for n, v in ((256, 360), (256, 1080), (512, 360), (512, 1080)):
        classes.append(("fbp", dict(WORKLOAD, nx=n, nz=n, px=204.8 / n, pz=204.8 / n, nu=2 * n, nv=n,
                                    du=0.8 * 512 / n, dv=0.8 * 512 / n, views=v, seed=seed + n + v)))
    classes.append(("cgls", dict(WORKLOAD, nx=256, nz=256, px=0.8, pz=0.8, nu=512, nv=256, du=1.6, dv=1.6,
                                 views=360, seed=seed + 1)))
    weights = np.array([0.4 / 9] * 9 + [0.4 / 4] * 4 + [0.2])
    # one noisy sinogram per class, made and kept on the device
    objs, sgms = [], []
    for kind, w in classes:
        o = parse(w)
        if kind == "cgls":
            config.parse_ir(o, {"Lambda": 1e-3})
            dg = geometry.ir_geometry(o, dev)
        else:
            dg = geometry.fbp_geometry(o, dev)
        sgms.append(noisy(ops.project_ellipsoids(dg, ellipsoids(w)), w["photons"], w["seed"]))
        objs.append(o)
        del dg
    torch.cuda.empty_cache()
    kinds = rng.choice(len(classes), size=n_req, p=weights / weights.sum())
    gaps = rng.exponential(mean_gap_ms / 1e3, size=n_req)
    sat_kinds = rng.choice(len(classes), size=n_sat, p=weights / weights.sum())
    x0 = {}

    def class_rmse(c, vol):
        kind, w = classes[c]
        ph = phantom(w, dev)
        if kind == "cgls":
            n_ = w["nx"]
            yy, xx = torch.meshgrid(torch.arange(n_, device=dev) - (n_ - 1) / 2,
                                    torch.arange(n_, device=dev) - (n_ - 1) / 2, indexing="ij")
            live = (yy ** 2 + xx ** 2 <= (0.95 * n_ / 2) ** 2).expand_as(ph).contiguous()
        else:
            live = vol != 0
        r = rmse(vol, ph, live)
        del ph, live
        return r

    def submit(srv, c, storage):
        kind, w = classes[c]
        if kind == "cgls":
            if c not in x0:
                x0[c] = torch.zeros((w["nz"], w["nx"], w["nx"]), dtype=torch.float32, device=dev)
            return srv.submit_cgls(objs[c], sgms[c], x0[c], 10, storage=storage)
        return srv.submit_fbp(objs[c], sgms[c], storage=storage)

    def run(storage, ks, gap_s):
        srv = ReconServer(device=dev, hbm_budget_gb=150.0, batch=4, max_slots_per_class=2)
        if gap_s is None:  # saturated: build the slots first (not timed)
            for f in [submit(srv, c, storage) for c in sorted(set(int(c) for c in ks))]:
                f.result(timeout=900)
            srv.done.clear()
        t0 = time.perf_counter()
        futs = []
        for i, c in enumerate(ks):
            if gap_s is not None:
                target = t0 + gap_s[: i + 1].sum()
                now = time.perf_counter()
                if target > now:
                    time.sleep(target - now)
            futs.append(submit(srv, c, storage))
        per_class = {}
        for i, f in enumerate(futs):
            vol = f.result(timeout=900)
            c = int(ks[i])
            if gap_s is not None and c not in per_class:
                per_class[c] = vol  # one result per class for its RMSE
            futs[i] = None  # drop the device result
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        rm = {}
        for c, vol in per_class.items():
            kind, w = classes[c]
            name = f"{kind}_{w['nx']}{'x' + str(w['nz']) if w.get('cone', True) else ''}_{w['views']}v"
            rm[name] = class_rmse(c, vol)
        del per_class
        torch.cuda.empty_cache()
        return st, wall, rm

    out = {"config": f"{n_req} requests, Poisson arrivals (mean gap {mean_gap_ms} ms), 2D FBP 256^2-1024^2 x "
                     "360-1440 views, FDK 256^3-512^3 x 360-1080 views, CGLS-10 at 256^3; HBM budget 150 GB; "
                     f"batch 4, a CUDA graph per slot member; saturated runs: slots built first, then {n_sat} "
                     "requests submitted at once",
           "mix": {"fbp_2d": int(sum(1 for c in kinds if c < 9)), "fdk": int(sum(1 for c in kinds if 9 <= c < 13)),
                   "cgls10": int(sum(1 for c in kinds if c == 13))}}
    for name, storage in (("plain", "f32"), ("mixed", "bf16")):
        st, wall, rm = run(storage, kinds, gaps)
        sat, sat_wall, _ = run(storage, sat_kinds, None)
        out[name] = {"storage": storage, "wall_s": round(wall, 3), "p50_ms": round(st["p50_ms"], 2),
                     "p99_ms": round(st["p99_ms"], 2), "mean_ms": round(st["mean_ms"], 2),
                     "queue_p50_ms": round(st["queue_p50_ms"], 2), "service_p50_ms": round(st["service_p50_ms"], 2),
                     "service_p99_ms": round(st["service_p99_ms"], 2), "gups": round(st["gups"], 2),
                     "completed": st["requests"], "slots": st["slots"], "classes": st["classes"],
                     "evictions": st["evictions"], "hbm_used_gb": round(st["hbm_used_gb"], 2),
                     "rmse_vs_phantom": rm,
                     "saturated": {"requests": sat["requests"], "wall_s": round(sat_wall, 3),
                                   "gups": round(sat["gups"], 2), "p50_ms": round(sat["p50_ms"], 2),
                                   "p99_ms": round(sat["p99_ms"], 2)}}
    p, m = out["plain"], out["mixed"]
    out["mixed_vs_plain"] = {"p50_ratio": round(m["p50_ms"] / p["p50_ms"], 3),
                             "p99_ratio": round(m["p99_ms"] / p["p99_ms"], 3),
                             "saturated_gups_ratio": round(m["saturated"]["gups"] / p["saturated"]["gups"], 3),
                             "rmse_ratio_per_class": {k: round(m["rmse_vs_phantom"][k] / v, 5)
                                                      for k, v in p["rmse_vs_phantom"].items()
                                                      if k in m["rmse_vs_phantom"] and v > 0}}
    return out


# ---------------------------------------------------------------- CPU leg: baseline and FP64 checks

def cpu_geom(w, o):
    """The C restatement's geometry of workload w (FBP arrays) and the projector's
    ray arrays."""
    from oracle import cpu_ref
    from reconstruction_program_taichi_gb300 import geometry
    u, v, ang = geometry.fbp_arrays(o)
    g = cpu_ref.geom_from_config(o, u, v, geometry.count_steps_v3(w["nx"], w["nz"], w["px"], w["pz"], w["step"]))
    fpu, fpv, _ = geometry.fpj_arrays(o)
    return g, ang, fpu, fpv


def spread(n, k):
    """k evenly spaced indices of range(n), starting at a non-special offset."""
    k = max(1, min(k, n))
    return [int((i + 0.37) * n / k) % n for i in range(k)]


def cpu_sample(w, o, bp_views, fp_views, filt_rows):
    """Time the float32 OpenMP C restatement on a bounded sample of one step: the
    direct row filter on filt_rows rows, the backprojection of bp_views views and the
    forward projection of fp_views evenly spaced views, each extrapolated linearly to
    the whole step (the cost per row and per view is uniform).  Returns (seconds for
    the full step, threads, description, parts)."""
    from oracle import cpu_ref
    g, ang, fpu, fpv = cpu_geom(w, o)
    rng = np.random.default_rng(1)
    rows = w["nv"] * w["views"]
    x = rng.uniform(0, 1, (filt_rows, w["nu"])).astype(np.float32)
    y = np.empty_like(x)
    taps = hann_from_ramp(recon_taps_of(o)).astype(np.float32)
    t0 = time.perf_counter()
    cpu_ref.filter_rows(g, x, taps, y, 0, filt_rows)
    t_f = (time.perf_counter() - t0) * rows / filt_rows
    F = rng.uniform(0, 1, (w["nv"], w["views"], w["nu"])).astype(np.float32)
    vol = np.zeros((w["nz"], w["nx"], w["nx"]), np.float32)
    alive = np.ones(vol.shape, np.uint8)
    angf = ang.astype(np.float32)
    j0 = spread(w["views"], 1)[0]
    t0 = time.perf_counter()
    cpu_ref.fdk_bp(g, angf, F, vol, alive, j0, min(w["views"], j0 + bp_views))
    t_bp = (time.perf_counter() - t0) * w["views"] / (min(w["views"], j0 + bp_views) - j0)
    out = np.zeros((w["nv"], w["views"], w["nu"]), np.float32)
    vol = rng.uniform(0, 0.02, vol.shape).astype(np.float32)
    views = spread(w["views"], fp_views)
    fpu32, fpv32 = fpu.astype(np.float32), fpv.astype(np.float32)
    t0 = time.perf_counter()
    for j in views:
        cpu_ref.fp(g, angf, fpu32, fpv32, vol, out, j, j + 1)
    t_fp = (time.perf_counter() - t0) * w["views"] / len(views)
    desc = (f"OpenMP C restatement (float32), {cpu_ref.threads()} threads: filter {filt_rows} of {rows} rows, "
            f"backprojection of views {j0}-{j0 + bp_views - 1} of {w['views']}, forward projection of "
            f"{len(views)} evenly spaced views {views}; each extrapolated linearly to the full step")
    return t_f + t_bp + t_fp, cpu_ref.threads(), desc, dict(filter_s=t_f, bp_s=t_bp, fp_s=t_fp)


def recon_taps_of(o):
    from reconstruction_program_taichi_gb300 import geometry
    return geometry.recon_taps(o)


def cpu_baseline(w, o, budget_s=20.0):
    from oracle import cpu_ref
    cpu_ref.build()
    scale = min(1.0, budget_s / 20.0)
    bp_views = max(2, int(round(48 * scale)))
    fp_views = max(1, int(round(6 * scale)))
    t, thr, desc, parts = cpu_sample(w, o, bp_views, fp_views, max(64, int(2048 * scale)))
    units = 2.0 * w["nx"] * w["nx"] * w["nz"] * w["views"]
    return {"value": round(units / t / 1e9, 4), "unit": "GUPS", "cores": thr, "kind": "port", "sample": desc,
            "extrapolated_step_s": round(t, 2), "parts_s": {k: round(v, 2) for k, v in parts.items()}}


class Fp64Checks:
    """Results collected during the GPU sections (host copies: the input sinogram, a
    slab of a volume, a few views of a projection) to be compared, after every timed
    region, with the float64 C restatement of the same discrete operator on the same
    inputs (bench.py runs it in its CPU leg).  Each check writes {"rel_l2", "max_abs",
    ...} under "vs_fp64" into the result dict it belongs to."""

    def __init__(self):
        self.items = []

    def fdk_slab(self, target, label, o, sgm, taps, z0, z1, got):
        """FDK (axial) of slices [z0, z1) from the raw sinogram sgm (host float32
        [nv, views, nu]) with filter taps; got: the GPU slab."""
        self.items.append(("fdk", target, label, dict(o=o, sgm=sgm, taps=taps, z0=z0, z1=z1, got=got)))

    def fp_views(self, target, label, o, vol, views, got, mask=None, ir=False):
        """Forward projection of vol (host float32) for the listed views; got: the GPU
        projection of those views [nv, len(views), nu]; ir: the IR driver's geometry
        (its arrays, step count and effective-map mask)."""
        self.items.append(("fp", target, label, dict(o=o, vol=vol, views=list(views), got=got, mask=mask, ir=ir)))

    def bp_unmatched_slab(self, target, label, o, sgm, z0, z1, got):
        """The IR driver's backprojector of sgm (host float32) over slices [z0, z1)."""
        self.items.append(("bpu", target, label, dict(o=o, sgm=sgm, z0=z0, z1=z1, got=got)))

    def run(self):
        """Evaluate every check (float64, all host threads); returns the seconds spent."""
        from oracle import cpu_ref
        from reconstruction_program_taichi_gb300 import geometry
        t0 = time.perf_counter()
        cache = {}
        for kind, target, label, a in self.items:
            o = a["o"]
            if kind == "fdk":
                u, v, ang = geometry.fbp_arrays(o)
                g = cpu_ref.geom_from_config(o, u, v)
                key = ("fdk", id(a["sgm"]), id(a["taps"]), a["z0"], a["z1"])
                if key not in cache:
                    cache[key] = cpu_ref.fdk_slab_f64(g, ang, a["sgm"], a["taps"], a["z0"], a["z1"])
                ref, rows = cache[key]
                e = cpu_ref.errors(a["got"], ref)
                e["zero_pattern_mismatches"] = int(np.sum((a["got"] == 0) != (ref == 0)))
                e["sample"] = (f"slices {a['z0']}-{a['z1'] - 1} of {g.nz}, every voxel of them, every view "
                               f"(detector rows {rows[0]}-{rows[1] - 1}, all that the slab reads)")
            elif kind == "fp":
                if a["ir"]:
                    u, v, ang = geometry.ir_arrays(o)
                    k = geometry.count_steps_ir(o.img_dim, o.img_dim_z, o.img_pix_size, o.img_voxel_height,
                                                o.fpj_step_size, o.source_isocenter_dis)
                    cz = np.asarray(o.array_img_center_z, dtype=np.float64)
                    assert np.all(cz == cz[0]), "per-view image centres are not checked here"
                    g = cpu_ref.geom_from_config(o, u, v, k).copy(cz=float(cz[0]))
                else:
                    u, v, ang = geometry.fpj_arrays(o)
                    k = geometry.count_steps_v3(o.img_dim, o.img_dim_z, o.img_pix_size, o.img_voxel_height,
                                                o.fpj_step_size)
                    g = cpu_ref.geom_from_config(o, u, v, k)
                g = g.copy(nv=o.det_elem_count_vertical_actual)
                key = ("fp", id(a["vol"]), a["ir"], tuple(a["views"]))
                if key not in cache:
                    cache[key] = cpu_ref.fp_views_f64(g, ang, u, v, a["vol"], a["views"])
                ref = cache[key]
                if a["mask"] is not None:
                    ref = np.where(a["mask"] == 1, ref, 0.0)
                e = cpu_ref.errors(a["got"], ref)
                e["sample"] = f"views {a['views']} of {g.views}, every ray"
            else:
                u, v, ang = geometry.ir_arrays(o)
                g = cpu_ref.geom_from_config(o, u, v)
                key = ("bpu", id(a["sgm"]), a["z0"], a["z1"])
                if key not in cache:
                    cache[key] = cpu_ref.bp_unmatched_slab_f64(g, ang, o.array_img_center_z, a["sgm"], a["z0"],
                                                               a["z1"])
                ref, rows = cache[key]
                e = cpu_ref.errors(a["got"], ref)
                e["zero_pattern_mismatches"] = int(np.sum((a["got"] == 0) != (ref == 0)))
                e["sample"] = f"slices {a['z0']}-{a['z1'] - 1} of {g.nz}, every view"
            target.setdefault("vs_fp64", {})[label] = {k_: (float(f"{v_:.4g}") if isinstance(v_, float) else v_)
                                                       for k_, v_ in e.items()}
        return time.perf_counter() - t0


def run_reference(args, w):
    """The reference arm: the reference's CPU implementation of the step (its Taichi
    kernels need Taichi, which cannot be installed here, so the OpenMP C restatement
    of those kernels, float32 like Taichi) on all host threads, each step a bounded
    sample (filter rows, a block of backprojection views, evenly spaced forward-
    projection views) extrapolated to the whole step."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    o = parse(w)
    from oracle import cpu_ref
    cpu_ref.build()
    for _ in range(args.warmup):
        cpu_sample(w, o, 2, 1, 64)
    times = []
    for _ in range(args.steps):
        t, thr, desc, parts = cpu_sample(w, o, 8, 2, 256)
        times.append(t)
    t = float(np.mean(times))
    units = 2.0 * w["nx"] * w["nx"] * w["nz"] * w["views"]
    value = units / t / 1e9
    line = {"impl": "reference", "metric": "GUPS (cone-beam FDK + forward projection, voxel x view updates per second)",
            "value": round(value, 4), "unit": "GUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(t * 1e3, 1), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (uniform random sinogram / volume; cost is data independent)",
            "config": {"workload": f"FDK+FP {w['nx']}x{w['nx']}x{w['nz']} vol, {w['views']} views, "
                                   f"{w['nu']}x{w['nv']} det; per step a bounded sample (256 filter rows, 8 "
                                   f"backprojection views, 2 evenly spaced forward-projection views), "
                                   f"extrapolated to the full step"},
            "cpu_baseline": {"value": round(value, 4), "unit": "GUPS", "cores": thr, "kind": "port", "sample": desc},
            "e2e": {"value": round(value, 4), "unit": "GUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference's Taichi kernels cannot run here (no taichi); this is the OpenMP C restatement "
                    "of the same kernels on all host threads"}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--storage", default="f32", choices=["f32", "bf16", "f16"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS),
                    help="c2: the benchmark; small: quick checks; prof, prof180, prof270, prof180z: short launches "
                         "for ncu captures")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-cgls", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--only", default=None, choices=["cgls", "piccs", "adjoint", "cg_step", "helical"],
                    help="cgls: only the IRN-CGLS-TV section; piccs: only the IRN-CGLS-PICCS section; "
                         "adjoint: only the projector / exact-adjoint "
                         "pair; cg_step: one reweighted CG solve of 3 iterations at 512x512x64 / 360 views; "
                         "helical: one helical FBP (short runs for ncu captures of their kernels)")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, w)
    elif args.only == "cgls":
        import torch
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        out = irn_bench(dev, torch.cuda.current_stream(dev), torch.cuda.synchronize)
        print(json.dumps({"irn_cgls_tv": out}))
    elif args.only == "piccs":
        import torch
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        out = piccs_bench(dev, torch.cuda.current_stream(dev), torch.cuda.synchronize)
        print(json.dumps({"irn_cgls_piccs": out}))
    elif args.only == "cg_step":
        import torch
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        storage = {"f32": "float32", "bf16": "bfloat16", "f16": "float16"}[args.storage]
        print(json.dumps({"cg_step_ms": cg_step_bench(dev, storage)}))
    elif args.only == "helical":
        import torch
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        print(json.dumps({"helical_ms": helical_once(dev)}))
    elif args.only == "adjoint":
        import torch
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        out = adjoint_pair_bench(dev, torch.cuda.current_stream(dev), torch.cuda.synchronize)
        print(json.dumps({"fp_adjoint_pair": out}))
    else:
        run_gpu(args, w)


if __name__ == "__main__":
    main()
