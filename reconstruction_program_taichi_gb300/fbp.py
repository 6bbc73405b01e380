"""FBP / FDK drop-in: run_mgfbp(config_path) and class Mgfbp, mirroring
run_mgfbp.py:18-85 (entry point and MainFunction) on the GB300 kernels.

Every reconstruction runs as: weighting (+BH) -> [vertical Gaussian] -> Toeplitz row
filter -> packing -> backprojection, all on one CUDA stream with the sinogram,
filtered sinogram and volume resident in HBM.
"""
import gc
import os
import re
import time

import numpy as np
import torch

from . import ops
from ._lib import MCT_BF16, MCT_F16, MCT_F32
from .config import ConfigError, ReadConfigFile, parse_fbp
from .geometry import fbp_geometry, gaussian_taps, recon_taps
from .file_pipeline import run_over_files
from .io import imwriteRaw, imwriteTiff, read_sinogram_file, read_sinogram_raw_layout

STORAGE = {"f32": MCT_F32, "float32": MCT_F32, "bf16": MCT_BF16, "bfloat16": MCT_BF16, "f16": MCT_F16,
           "float16": MCT_F16}


def _device(device=None):
    if not torch.cuda.is_available():
        raise RuntimeError("a CUDA device is required (this package has no CPU fallback)")
    dev = torch.device(device or "cuda")
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    return dev


class FdkPipeline:
    """Weight -> filter -> pack -> backproject for one FBP geometry, with reusable
    device buffers.  `storage` selects the backprojection operand precision: 'f32'
    (plain), 'bf16' or 'f16' (16-bit storage).  `filter_impl` selects the row filter,
    the Toeplitz product on the tensor cores with float32 accumulation:
    'tc3' (default: bf16 hi + mid + lo parts, ~1e-6 relative) or 'tc' (hi + lo parts:
    ~1e-5 relative at benchmark sizes, up to ~1e-4 on small detectors where the ramp's
    cancellation amplifies the dropped 2^-16 terms; the mixed path) — or 'simt'
    (float32 FMA on the SIMT cores)."""

    def __init__(self, obj, device=None, storage="f32", filter_impl="tc3"):
        dev = _device(device)
        self.obj = obj
        self.dg = fbp_geometry(obj, dev)
        self.device = dev
        self.dtype = STORAGE[storage]
        self.kernel_none = obj.kernel_name == "None"
        f32 = dict(dtype=torch.float32, device=dev)
        self.taps = None if self.kernel_none else torch.tensor(recon_taps(obj), **f32)
        if filter_impl not in ("simt", "tc", "tc3"):
            raise ValueError("filter_impl must be 'tc3', 'tc' (tensor-core split bf16) or 'simt' (float32 FMA)")
        self.filter_impl = filter_impl
        self._tc_dtype = MCT_F32 if filter_impl == "tc3" else MCT_BF16
        # whether the row filter runs on the tensor cores; the filter object (its operand
        # tiles are sized by the whole sinogram) and the full-size buffers below are
        # allocated on first use, so that drivers that stream view chunks through this
        # pipeline's geometry and taps (Mgfbp_v2) hold only their chunk buffers
        self.uses_tc = filter_impl in ("tc", "tc3") and not self.kernel_none
        self._tc = None
        self.gauss_v = None
        if obj.apply_gauss_vertical:
            self.gauss_v = torch.tensor(gaussian_taps(obj.det_elem_count_vertical_actual, obj.det_elem_height,
                                                      obj.det_elem_vertical_gauss_filter_size), **f32)
        self.bh = torch.tensor(obj.array_bh_coefficients, **f32) if obj.bool_bh_correction else None
        self._weighted = None  # the weighted sinogram, allocated by the paths that write it
        self._smoothed = self._filtered = self._packed = self._vol = None

    def _buffer(self, name, make):
        t = getattr(self, name)
        if t is None:
            t = make()
            setattr(self, name, t)
        return t

    @property
    def tc(self):
        """The tensor-core row filter of this geometry and taps (None with the SIMT filter)."""
        if self._tc is None and self.uses_tc:
            self._tc = ops.TcFilter(self.dg, self.taps, self._tc_dtype)
        return self._tc

    @property
    def weighted(self):
        """Buffer of the weighted sinogram [rows, views, cols] (the tensor-core path
        without a vertical Gaussian weights while it filters and never needs it)."""
        return self._buffer("_weighted", lambda: torch.empty(self.dg.sgm_shape, dtype=torch.float32,
                                                             device=self.device))

    @property
    def smoothed(self):
        if self.gauss_v is None:
            return None
        return self._buffer("_smoothed", lambda: torch.empty(self.dg.sgm_shape, dtype=torch.float32,
                                                             device=self.device))

    @property
    def filtered(self):
        g = self.dg.geom
        return self._buffer("_filtered", lambda: torch.empty((g.views, g.nv, g.nu), dtype=torch.float32,
                                                             device=self.device))

    @property
    def packed(self):
        return self._buffer("_packed", lambda: torch.empty(max(ops.packed_bytes(self.dg, self.dtype), 16),
                                                           dtype=torch.uint8, device=self.device))

    @property
    def vol(self):
        return self._buffer("_vol", lambda: torch.empty(self.dg.vol_shape, dtype=torch.float32, device=self.device))

    def allocate(self):
        """Allocate now every buffer run() uses (callers that account device memory
        before the first run: the serving slots)."""
        fused = self.uses_tc and self.gauss_v is None
        if not fused:
            self.weighted
        self.smoothed
        self.filtered
        self.packed
        self.vol
        self.tc
        return self

    def nbytes(self):
        """Device bytes held by this pipeline's buffers (those allocated so far)."""
        ts = [self._weighted, self._smoothed, self._filtered, self._packed, self._vol]
        return sum(t.numel() * t.element_size() for t in ts if t is not None) + (
            self._tc._buf.numel() if self._tc is not None else 0)

    def filter(self, sgm, row_stride=None, view_stride=None):
        """Weighted and filtered view-major sinogram [views, rows, cols].  With the
        tensor-core filter and no vertical Gaussian, the weighting runs while the
        operand is split (one pass over the sinogram, no weighted copy)."""
        g = self.dg.geom
        if row_stride is None:
            row_stride, view_stride = g.views * g.nu, g.nu
        if self.tc is not None and self.gauss_v is None and not self.kernel_none:
            return self.tc.weight_filter(sgm, row_stride, view_stride, self.bh, out=self.filtered)
        w = ops.weight(self.dg, sgm, row_stride, view_stride, self.bh, out=self.weighted)
        if self.gauss_v is not None:
            w = ops.vgauss(self.dg, w, self.gauss_v, out=self.smoothed)
        if self.kernel_none:
            self.filtered.copy_(w.permute(1, 0, 2))
            return self.filtered
        if self.tc is not None:
            return self.tc(w, out=self.filtered)
        return ops.filter_rows(self.dg, w, self.taps, out=self.filtered)

    def set_taps(self, taps):
        """Replace the filter taps (float64/float32 array of 2*nu-1 values)."""
        self.taps.copy_(torch.as_tensor(taps, dtype=torch.float32))
        self._tc = None  # rebuilt from the new taps on first use

    def backproject(self, filtered, out=None):
        packed = ops.pack(self.dg, filtered, self.dtype, out=self.packed)
        return ops.fdk_bp(self.dg, packed, self.dtype, out=self.vol if out is None else out)

    def run(self, sgm, row_stride=None, view_stride=None, out=None):
        """Full FBP of a device sinogram (default layout [rows, views, cols])."""
        return self.backproject(self.filter(sgm, row_stride, view_stride), out)


class Mgfbp:
    """Drop-in for the reference class Mgfbp (run_mgfbp.py:50-1310)."""

    def __init__(self, config_dict, device=None, storage="f32", verbose=True):
        self.verbose = verbose
        parse_fbp(self, config_dict)
        self.img_recon = np.zeros((self.img_dim_z, self.img_dim, self.img_dim), dtype=np.float32)
        self.device = device
        self.storage = storage
        self.file_processed_count = 0
        self._pipe = None

    def _log(self, msg):
        if self.verbose:
            print(msg)

    @property
    def pipeline(self):
        if self._pipe is None:
            self._pipe = FdkPipeline(self, self.device, self.storage)
        return self._pipe

    def MainFunction(self):  # noqa: N802 - reference name
        """Reconstruct every matching input file (run_mgfbp.py:52-85)."""
        if self.kernel_name is None:
            raise ConfigError("ERROR: no reconstruction kernel (HammingFilter, GaussianApodizedRamp or None) "
                              "in the config!")
        pipe = self.pipeline
        self.file_processed_count = 0

        def compute(d):
            d.file_processed_count += 1
            d._log("Reconstructing %s ..." % d.input_path)
            dev = torch.from_numpy(d._raw).to(pipe.device, non_blocking=False)
            filtered = pipe.filter(dev, d._row_stride, d._view_stride)
            if d.save_filtered_sinogram:
                imwriteTiff(filtered.cpu().numpy(), d.output_dir + "/sgm_filtered_" + d.output_file)
            vol = pipe.backproject(filtered)
            d.img_recon = vol.cpu().numpy()
            d._log("Saving to %s !" % d.output_path)

        # the next file is read and the previous one written while this one runs
        files = [f for f in os.listdir(self.input_dir) if re.match(self.input_files_pattern, f)]
        run_over_files(self, files, lambda d, f: d.ReadSinogram(f), compute, lambda d: d.SaveReconImg())
        return self.img_recon

    def output_name(self, file):
        """Output file name from OutputFileReplace pairs (run_mgfbp.py:1190-1203)."""
        out = file
        for i in range(int(len(self.output_file_replace) / 2)):
            out = re.sub(self.output_file_replace[2 * i], self.output_file_replace[2 * i + 1], out)
        if out == file:
            raise ConfigError(f"ERROR: did not file string to replace in '{out}'")
        if self.output_file_format in ("tif", "tiff"):
            out = re.sub(".raw", ".tif", out)
        return out

    def ReadSinogram(self, file):  # noqa: N802 - reference name
        """Read one input file (run_mgfbp.py:1189-1228); keeps the file layout and
        lets the device weighting kernel read it with strides."""
        self.input_path = os.path.join(self.input_dir, file)
        self.output_file = self.output_name(file)
        self.output_path = os.path.join(self.output_dir, self.output_file_prefix + self.output_file)
        self._raw, self._row_stride, self._view_stride = read_sinogram_raw_layout(self, self.input_path)
        return True

    def read_sinogram_array(self, file):
        """[rows, views, cols] float32 of one file, as the reference's img_sgm."""
        return read_sinogram_file(self, os.path.join(self.input_dir, file))

    def SaveReconImg(self):  # noqa: N802 - reference name
        """HU conversion and file output (run_mgfbp.py:1302-1310)."""
        if self.convert_to_HU:
            self.img_recon = (self.img_recon / self.water_mu - 1) * 1000
        if self.output_file_format == "raw":
            imwriteRaw(self.img_recon, self.output_path, dtype=np.float32)
        else:
            imwriteTiff(self.img_recon, self.output_path, dtype=np.float32)


class Mgfbp_v2(Mgfbp):  # noqa: N801 - reference name
    """Drop-in for Mgfbp_v2 (run_mgfbp_v2.py:61-364), the FBP that backprojects view by
    view to bound device memory.  Here the sinogram stays on the host and streams to
    the device in chunks of `views_per_chunk` views: while chunk c is weighted,
    filtered, packed and backprojected (accumulating into the volume) on the compute
    stream, chunk c+1 is staged into pinned memory by the CPU and copied on a second
    stream.  Device memory is the volume plus two chunks, whatever the number of views.
    Voxels that leave the detector in any view are 0, as in the reference
    (SetTruncatedRegionToZero :229-233 after its per-view -10000 marks)."""

    def __init__(self, config_dict, device=None, storage="f32", verbose=True, views_per_chunk=64):
        super().__init__(config_dict, device=device, storage=storage, verbose=verbose)
        if views_per_chunk < 1:
            raise ValueError("views_per_chunk must be positive")
        self.views_per_chunk = int(views_per_chunk)

    def MainFunction(self):  # noqa: N802 - reference name
        """run_mgfbp_v2.py:62-103."""
        if self.kernel_name is None:
            raise ConfigError("ERROR: no reconstruction kernel (HammingFilter, GaussianApodizedRamp or None) "
                              "in the config!")
        pipe = self.pipeline
        self.file_processed_count = 0
        for file in os.listdir(self.input_dir):
            if re.match(self.input_files_pattern, file):
                if self.ReadSinogram(file):
                    self.file_processed_count += 1
                    self._log("Reconstructing %s ..." % self.input_path)
                    vol = self._stream_file(pipe)
                    self.img_recon = vol.cpu().numpy()
                    self._log("Saving to %s !" % self.output_path)
                    self.SaveReconImg()
        return self.img_recon

    def _stream_file(self, pipe):
        dg, dev = pipe.dg, pipe.device
        g = dg.geom
        nb, V = g.views, min(self.views_per_chunk, g.views)
        raw = self._raw
        sino_layout = self._view_stride == g.nu  # [rows][views][cols] (else [views][rows][cols])
        shape = (g.nv, V, g.nu) if sino_layout else (V, g.nv, g.nu)
        staging = [torch.empty(shape, dtype=torch.float32, pin_memory=True) for _ in range(2)]
        dev_in = [torch.empty(shape, dtype=torch.float32, device=dev) for _ in range(2)]
        copy_stream = torch.cuda.Stream(device=dev)
        compute = torch.cuda.current_stream(dev)
        copied = [torch.cuda.Event() for _ in range(2)]
        consumed = [torch.cuda.Event() for _ in range(2)]
        vol = torch.zeros(dg.vol_shape, dtype=torch.float32, device=dev)
        f32 = dict(dtype=torch.float32, device=dev)
        weighted = torch.empty((g.nv, V, g.nu), **f32)
        smoothed = torch.empty((g.nv, V, g.nu), **f32) if pipe.gauss_v is not None else None
        filtered = torch.empty((V, g.nv, g.nu), **f32)
        chunk0 = ops.ViewChunk(dg, 0, V)
        packed = torch.empty(max(ops.packed_bytes(chunk0, pipe.dtype), 16), dtype=torch.uint8, device=dev)
        chunks = [(j0, min(j0 + V, nb)) for j0 in range(0, nb, V)]

        def stage(i):
            j0, j1 = chunks[i]
            n = j1 - j0
            b = i % 2
            consumed[b].synchronize()  # the pinned buffer's previous copy has been consumed
            src = raw[:, j0:j1, :] if sino_layout else raw[j0:j1]
            dst = staging[b][:, :n, :] if sino_layout else staging[b][:n]
            dst.copy_(torch.from_numpy(src))
            with torch.cuda.stream(copy_stream):
                copy_stream.wait_event(consumed[b])
                (dev_in[b][:, :n, :] if sino_layout else dev_in[b][:n]).copy_(dst, non_blocking=True)
                copied[b].record(copy_stream)

        tcs = {}  # tensor-core filters per chunk length (the operand tiles follow the rows)

        def tc_for(cg, n):
            if not pipe.uses_tc:
                return None
            if n not in tcs:
                tcs[n] = ops.TcFilter(cg, pipe.taps, pipe._tc_dtype)
            return tcs[n]

        for e in consumed:
            e.record(compute)
        stage(0)
        for i, (j0, j1) in enumerate(chunks):
            n, b = j1 - j0, i % 2
            # chunk i's kernels are queued first, then the host stages chunk i + 1 (which
            # waits for chunk i - 1 to release its buffers), so the GPU works on chunk i
            # while the CPU copies the next one into pinned memory
            compute.wait_event(copied[b])
            cg = ops.ViewChunk(dg, j0, n, accumulate=True)
            rs, vs = (V * g.nu, g.nu) if sino_layout else (g.nu, g.nv * g.nu)
            tc = tc_for(cg, n)
            if tc is not None and smoothed is None:
                # weighting inside the tensor-core filter's operand split
                f = tc.weight_filter(dev_in[b], rs, vs, pipe.bh, out=filtered[:n], dg=cg)
            else:
                w = ops.weight(cg, dev_in[b], rs, vs, pipe.bh, out=weighted if n == V else None)
                if smoothed is not None:
                    w = ops.vgauss(cg, w, pipe.gauss_v, out=smoothed if n == V else None)
                if pipe.kernel_none:
                    f = w.permute(1, 0, 2).contiguous()
                elif tc is not None:
                    f = tc(w, out=filtered[:n])
                else:
                    f = ops.filter_rows(cg, w, pipe.taps, out=filtered[:n])
            pk = ops.pack(cg, f, pipe.dtype, out=packed)
            ops.fdk_bp(cg, pk, pipe.dtype, out=vol)
            consumed[b].record(compute)
            if i + 1 < len(chunks):
                stage(i + 1)
        ops.fdk_bp_finish(dg, vol)
        return vol


def run_mgfbp_v2(file_path, device=None, storage="f32", verbose=True, views_per_chunk=64):
    """Drop-in for run_mgfbp_v2.run_mgfbp_v2 (run_mgfbp_v2.py:26-57)."""
    if verbose:
        print("Performing FBP from MandoCT-GB300 (view-streaming) ...")
    start = time.time()
    if not os.path.exists(file_path):
        raise ConfigError(f"ERROR: Config File {file_path} does not exist!")
    fbp = Mgfbp_v2(ReadConfigFile(file_path), device=device, storage=storage, verbose=verbose,
                   views_per_chunk=views_per_chunk)
    img = fbp.MainFunction()
    if verbose:
        if fbp.file_processed_count > 0:
            print(f"\nA total of {fbp.file_processed_count:d} file(s) are reconstructed!")
            print(f"Time cost is {time.time() - start:.3} sec\n")
        else:
            print(f"\nWarning: Did not find files like {fbp.input_files_pattern:s} in {fbp.input_dir:s}.")
            print("No images are reconstructed!\n")
    del fbp
    gc.collect()
    return img


def run_mgfbp(file_path, device=None, storage="f32", verbose=True):
    """Drop-in for run_mgfbp.run_mgfbp (run_mgfbp.py:18-47): FBP of every file that
    matches the config, returning the last reconstruction [z, y, x] (HU if WaterMu)."""
    if verbose:
        print("Performing FBP from MandoCT-GB300 ...")
    start = time.time()
    if not os.path.exists(file_path):
        raise ConfigError(f"ERROR: Config File {file_path} does not exist!")
    fbp = Mgfbp(ReadConfigFile(file_path), device=device, storage=storage, verbose=verbose)
    img = fbp.MainFunction()
    if verbose:
        if fbp.file_processed_count > 0:
            print(f"\nA total of {fbp.file_processed_count:d} file(s) are reconstructed!")
            print(f"Time cost is {time.time() - start:.3} sec\n")
        else:
            print(f"\nWarning: Did not find files like {fbp.input_files_pattern:s} in {fbp.input_dir:s}.")
            print("No images are reconstructed!\n")
    del fbp
    gc.collect()
    return img
