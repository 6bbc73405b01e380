"""Forward-projection drop-in: run_mgfpj_v3(config_path) and class Mgfpj_v3,
mirroring run_mgfpj_v3.py:45-127 on the GB300 kernels.  All views of a volume are
projected in one launch; binning and noise follow in one more.
"""
import gc
import os
import re
import time

import numpy as np
import torch

from . import ops
from .config import ConfigError, ReadConfigFile, parse_fbp, parse_fpj, parse_fpj_v1, parse_fpj_v3
from .geometry import fpj_geometry, fpj_variant_geometry
from .file_pipeline import run_over_files
from .io import imwriteRaw


class FpPipeline:
    """Forward projection + binning/noise for one projector geometry.

    version 3 (Mgfpj_v3): noise on every detector row (run_mgfpj_v3.py:117-122);
    version 2 (Mgfpj of run_mgfpj_v2.py): rows outside the recon range stay 0 and
    get no noise (:84-106); version 1 (run_mgfpj.py): all rows."""

    def __init__(self, obj, device=None, version=3):
        if not torch.cuda.is_available():
            raise RuntimeError("a CUDA device is required (this package has no CPU fallback)")
        self.obj = obj
        self.version = version
        self.dg = fpj_geometry(obj, device) if version == 3 else fpj_variant_geometry(obj, version, device)
        g = self.dg.geom
        self.full_rows = obj.det_elem_count_vertical
        self.begin = obj.det_elem_vertical_recon_range_begin
        self.os = obj.oversample_size
        # geometry of the binning step: all detector rows, binned columns
        self.bin_dg = ops.DeviceGeometry(g.copy(nv=self.full_rows, nu=obj.det_elem_count_horizontal),
                                         self.dg.host["angles"], device=self.dg.device)
        self.rows_buf = torch.zeros((g.nv, g.views, g.nu), dtype=torch.float32, device=self.dg.device)
        self.full_buf = None
        if g.nv != self.full_rows:
            self.full_buf = torch.zeros((self.full_rows, g.views, g.nu), dtype=torch.float32, device=self.dg.device)

    def project(self, vol, seed=0):
        """[rows, views, cols] sinogram of a device volume, binned (and noisy if
        PhotonNumber is set), before the output-form flip."""
        obj = self.obj
        rows = ops.fp(self.dg, vol, out=self.rows_buf)
        photons = float(obj.photon_number) if obj.add_possion_noise else 0.0
        if self.version == 2 and self.full_buf is not None:
            g = self.dg.geom
            part_dg = ops.DeviceGeometry(g.copy(nu=obj.det_elem_count_horizontal), self.dg.host["angles"],
                                         device=self.dg.device)
            binned = ops.bin_noise(part_dg, rows, self.os, photons, seed)
            out = torch.zeros((self.full_rows, g.views, obj.det_elem_count_horizontal), dtype=torch.float32,
                              device=self.dg.device)
            out[self.begin:self.begin + rows.shape[0]] = binned
            return out
        if self.full_buf is not None:
            self.full_buf[self.begin:self.begin + rows.shape[0]] = rows
            rows = self.full_buf
        if self.os == 1 and photons == 0.0:
            return rows
        return ops.bin_noise(self.bin_dg, rows, self.os, photons, seed)


class Mgfpj_v3:  # noqa: N801 - reference name
    """Drop-in for the reference class Mgfpj_v3 (run_mgfpj_v3.py:80-391)."""

    VERSION = 3

    def _parse(self, config_dict):
        parse_fbp(self, config_dict)
        parse_fpj(self, config_dict)
        parse_fpj_v3(self, config_dict)

    def __init__(self, config_dict, device=None, verbose=True, noise_seed=0):
        self.verbose = verbose
        self._parse(config_dict)
        self.img_sgm = np.zeros((self.det_elem_count_vertical, self.view_num, self.det_elem_count_horizontal),
                                dtype=np.float32)
        self.device = device
        self.noise_seed = noise_seed
        self.file_processed_count = 0
        self._pipe = None

    @property
    def pipeline(self):
        if self._pipe is None:
            self._pipe = FpPipeline(self, self.device, self.VERSION)
        return self._pipe

    def ReadImage(self, file):  # noqa: N802 - reference name
        """Read one volume (run_mgfpj_v2.py:423-441)."""
        self.input_path = os.path.join(self.input_dir, file)
        self.output_file = re.sub(self.output_file_replace[0], self.output_file_replace[1], file)
        if self.output_file == file:
            raise ConfigError(f"ERROR: did not find string '{self.output_file_replace[0]}' to replace in "
                              f"'{self.output_file}'")
        self.output_path = os.path.join(self.output_dir, self.output_file_prefix + self.output_file)
        img = np.fromfile(self.input_path, dtype=np.float32).reshape(self.img_dim_z, self.img_dim, self.img_dim)
        if self.convert_to_HU:
            img = ((img + 1000.0) / 1000.0 * self.water_mu).astype(np.float32)
        self.img_image = img
        return True

    def MainFunction(self):  # noqa: N802 - reference name
        """Forward project every matching volume (run_mgfpj_v3.py:82-127)."""
        pipe = self.pipeline
        self.file_processed_count = 0

        def compute(d):
            if d.verbose:
                print("\nForward projecting %s ..." % d.input_path)
            d.file_processed_count += 1
            vol = torch.from_numpy(d.img_image).to(pipe.dg.device)
            sgm = pipe.project(vol, seed=d.noise_seed + d.file_processed_count)
            d.img_sgm = sgm.cpu().numpy()
            if d.verbose:
                print("\nSaving to %s !" % d.output_path)

        # the next volume is read and the previous sinogram written while this one runs
        files = [f for f in os.listdir(self.input_dir) if re.match(self.input_files_pattern, f)]
        run_over_files(self, files, lambda d, f: d.ReadImage(f), compute, lambda d: d.SaveSinogram())
        return self.img_sgm

    def SaveSinogram(self):  # noqa: N802 - reference name
        """Output-form conventions of run_mgfpj_v2.py:458-470."""
        if self.cone_beam:
            if self.output_file_form == "sinogram":
                self.img_sgm = np.ascontiguousarray(np.flip(self.img_sgm, axis=0))
                imwriteRaw(self.img_sgm, self.output_path, dtype=np.float32)
            else:
                imwriteRaw(self.img_sgm.transpose(1, 0, 2), self.output_path, dtype=np.float32)
        else:
            imwriteRaw(self.img_sgm, self.output_path, dtype=np.float32)


def run_mgfpj_v3(file_path, device=None, verbose=True, noise_seed=0):
    """Drop-in for run_mgfpj_v3.run_mgfpj_v3 (run_mgfpj_v3.py:45-77): returns the
    last sinogram [rows, views, cols] in the output-form convention."""
    start = time.time()
    if not os.path.exists(file_path):
        raise ConfigError(f"ERROR: Config File {file_path} does not exist!")
    fpj = Mgfpj_v3(ReadConfigFile(file_path), device=device, verbose=verbose, noise_seed=noise_seed)
    sgm = fpj.MainFunction()
    if verbose:
        if fpj.file_processed_count > 0:
            print(f"\nA total of {fpj.file_processed_count:d} files are forward projected!")
            print(f"Time cost is {time.time() - start:.3} sec\n")
        else:
            print(f"\nWarning: Did not find files like {fpj.input_files_pattern:s} in {fpj.input_dir:s}.")
    gc.collect()
    return sgm


class Mgfpj(Mgfpj_v3):
    """Drop-in for Mgfpj of run_mgfpj_v2.py:69-470 (Mgfbp-derived, row by row)."""

    VERSION = 2

    def _parse(self, config_dict):
        parse_fbp(self, config_dict)
        parse_fpj(self, config_dict)


class MgfpjOriginal(Mgfpj_v3):
    """Drop-in for the stand-alone Mgfpj of run_mgfpj.py:56-669."""

    VERSION = 1

    def _parse(self, config_dict):
        parse_fpj_v1(self, config_dict)

    def ReadImage(self, file):  # noqa: N802 - reference name
        """run_mgfpj.py:618-638 (only the first replacement pair is used)."""
        return super().ReadImage(file)


def _run(cls, file_path, device, verbose, noise_seed):
    start = time.time()
    if not os.path.exists(file_path):
        raise ConfigError(f"ERROR: Config File {file_path} does not exist!")
    fpj = cls(ReadConfigFile(file_path), device=device, verbose=verbose, noise_seed=noise_seed)
    sgm = fpj.MainFunction()
    if verbose and fpj.file_processed_count > 0:
        print(f"\nA total of {fpj.file_processed_count:d} files are forward projected!")
        print(f"Time cost is {time.time() - start:.3} sec\n")
    gc.collect()
    return sgm


def run_mgfpj(file_path, device=None, verbose=True, noise_seed=0):
    """Drop-in for run_mgfpj.run_mgfpj (run_mgfpj.py:24-53)."""
    return _run(MgfpjOriginal, file_path, device, verbose, noise_seed)


def run_mgfpj_v2(file_path, device=None, verbose=True, noise_seed=0):
    """Drop-in for run_mgfpj_v2.run_mgfpj_v2 (run_mgfpj_v2.py:35-66)."""
    return _run(Mgfpj, file_path, device, verbose, noise_seed)
