"""Back-to-back reconstruction of host-resident scans with the host <-> device copies
behind the compute.

One scan is: sinogram host -> device, FDK (and, optionally, the forward projection of
the reconstruction) on the device, results device -> host.  Done one scan after the
other on one stream, the copies (at 512^2 x 256 / 1080 views: 1.13 GB in, 1.40 GB out)
add to every scan.  `ScanStream` keeps two device buffer sets and three streams: while
scan i computes, scan i+1's sinogram is copied in on an upload stream and scan i-1's
results are copied out on a download stream.  Events order the reuse of each buffer
(a sinogram buffer is refilled only after the compute that read it, a result buffer
only after its download), so every scan's copies and kernels are those of the
sequential flow; only their placement in time changes.

The reference reconstructs the files of a run one after the other
(run_mgfbp.py:52-85, MainFunction); this is that loop with the transfers overlapped.
"""
import torch

from . import ops


class ScanStream:
    """Pipelined FDK (+ forward projection) of a sequence of pinned host sinograms.

    pipe: an `fbp.FdkPipeline` (its geometry fixes the shapes); fp_geom: optional
    forward-projection geometry (`geometry.fpj_geometry` / `ir_geometry`) whose
    projections of each reconstruction are returned too; fp_dtype: the projector's
    gather storage (ops.MCT_F32, MCT_BF16, MCT_F16)."""

    def __init__(self, pipe, fp_geom=None, fp_dtype=ops.MCT_F32):
        dev = pipe.device
        self.pipe = pipe
        self.fpg = fp_geom
        self.fp_dtype = fp_dtype
        self.compute = torch.cuda.Stream(device=dev)
        self.up = torch.cuda.Stream(device=dev)
        self.down = torch.cuda.Stream(device=dev)
        f32 = dict(dtype=torch.float32, device=dev)
        self.sgm = [torch.empty(pipe.dg.sgm_shape, **f32) for _ in range(2)]
        self.vol = [torch.empty(pipe.dg.vol_shape, **f32) for _ in range(2)]
        self.proj = [torch.empty(fp_geom.sgm_shape, **f32) for _ in range(2)] if fp_geom is not None else None
        self.ev_in = [torch.cuda.Event() for _ in range(2)]    # sinogram slot uploaded
        self.ev_comp = [torch.cuda.Event() for _ in range(2)]  # slot computed (its sinogram is free)
        self.ev_out = [torch.cuda.Event() for _ in range(2)]   # slot downloaded (its results are free)
        self.submitted = 0

    def submit(self, host_sgm, host_vol, host_proj=None):
        """Enqueue one scan and return at once.  host_sgm (pinned, the pipeline's
        sinogram shape) must stay unchanged, and host_vol / host_proj (pinned) unread,
        until the returned event has completed."""
        if (host_proj is None) != (self.proj is None):
            raise ValueError("host_proj is required exactly when the stream has a forward-projection geometry")
        shapes = {"host_sgm": self.sgm[0].shape, "host_vol": self.vol[0].shape,
                  "host_proj": self.proj[0].shape if self.proj is not None else None}
        for t, name in ((host_sgm, "host_sgm"), (host_vol, "host_vol"), (host_proj, "host_proj")):
            if t is None:
                continue
            if t.is_cuda or not t.is_pinned():
                raise ValueError(f"{name} must be a pinned host tensor")
            if t.dtype != torch.float32 or tuple(t.shape) != tuple(shapes[name]):
                raise ValueError(f"{name} must be float32 of shape {tuple(shapes[name])}, got {t.dtype} "
                                 f"{tuple(t.shape)}")
        s = self.submitted % 2
        reuse = self.submitted >= 2
        self.submitted += 1
        # work the caller queued on its own stream (pipeline set-up, new taps) first
        self.compute.wait_stream(torch.cuda.current_stream(self.pipe.device))
        with torch.cuda.stream(self.up):
            if reuse:
                self.up.wait_event(self.ev_comp[s])
            self.sgm[s].copy_(host_sgm, non_blocking=True)
            self.ev_in[s].record(self.up)
        with torch.cuda.stream(self.compute):
            self.compute.wait_event(self.ev_in[s])
            if reuse:
                self.compute.wait_event(self.ev_out[s])
            vol = self.pipe.run(self.sgm[s], out=self.vol[s])
            if self.fpg is not None:
                ops.fp(self.fpg, vol, out=self.proj[s], dtype=self.fp_dtype)
            self.ev_comp[s].record(self.compute)
        with torch.cuda.stream(self.down):
            self.down.wait_event(self.ev_comp[s])
            host_vol.copy_(self.vol[s], non_blocking=True)
            if host_proj is not None:
                host_proj.copy_(self.proj[s], non_blocking=True)
            self.ev_out[s].record(self.down)
        return self.ev_out[s]

    def synchronize(self):
        """Wait for every submitted scan (downloads included)."""
        for st in (self.up, self.compute, self.down):
            st.synchronize()
