"""Helical FBP by per-slice rebinning: drop-in for Mgfbp_helical / run_mgfbp_helical
(run_mgfbp_helical.py:25-258).

The reference reconstructs one slice at a time: rebin the helical sinogram to a fan
sinogram for that slice's z, then run the 2D fan FBP with the image rotated by the
slice's angular offset.  Here every slice is processed at once:

  1. `mct_helical_rebin` builds the whole stack [slices][view_count][cols] in one
     launch;
  2. weighting and the Toeplitz row filter run over the stack as one sinogram
     (slices x views rows; the fan weighting and the short-scan weights are the same
     for every slice, as the slice offsets cancel in them);
  3. the filtered stack is packed once, slice-major, and each slice is
     backprojected with its own angle table (base angles + the slice's offset).
     Rotating the image by the offset, as the reference does, and adding the offset
     to the view angles are the same transform.
"""
import copy
import gc
import os
import re
import time

import ctypes
import numpy as np
import torch

from . import _lib, ops
from ._lib import MCT_F32, Helical, Tables
from .config import PI, ConfigError, ReadConfigFile
from .fbp import Mgfbp, FdkPipeline
from .file_pipeline import run_over_files
from .geometry import fbp_geometry, gaussian_taps
from .io import imwriteTiff


class Mgfbp_helical(Mgfbp):  # noqa: N801 - reference name
    """Drop-in for Mgfbp_helical (run_mgfbp_helical.py:57-258)."""

    def __init__(self, config_dict, device=None, storage="f32", verbose=True):
        super().__init__(config_dict, device=device, storage=storage, verbose=verbose)
        if "HelicalPitch" not in config_dict:
            raise ConfigError("ERROR: Can not find helical pitch in the config file!")
        # run_mgfbp_helical.py:61-95, in the reference's order and precision
        self.helical_pitch = config_dict["HelicalPitch"]
        self.mag_ratio_isocenter = self.source_det_dis / self.source_isocenter_dis
        self.isocenter_coverage = self.det_elem_count_vertical_actual * self.det_elem_height / self.mag_ratio_isocenter
        self.dis_per_round = self.helical_pitch * self.isocenter_coverage
        self.num_rounds = abs(self.total_scan_angle) / (2 * PI)
        self.angle_per_view = self.total_scan_angle / self.view_num
        self.dis_per_view = self.dis_per_round / (self.view_num / self.num_rounds)
        self.gamma_max = 2 * np.arctan(0.5 * self.det_elem_count_horizontal * self.det_elem_width
                                       / self.source_det_dis) / PI
        self.short_scan_range = 2 * PI / abs(self.helical_pitch)
        if self.short_scan_range < PI + self.gamma_max:
            self.short_scan_range = PI + self.gamma_max
        self.det_offset_vertical_at_isocenter = self.det_offset_vertical / self.mag_ratio_isocenter
        sgn = np.sign(self.helical_pitch)
        z_begin = self.isocenter_coverage / 2.0 * sgn + self.det_offset_vertical_at_isocenter
        z_end = self.dis_per_view * self.view_num - self.isocenter_coverage / 2.0 * sgn \
            + self.det_offset_vertical_at_isocenter
        self.array_z_pos = np.arange(z_begin, z_end, self.img_voxel_height * sgn, dtype=np.float32)
        if len(self.array_z_pos) == 0:
            raise ConfigError("ERROR: the helical scan covers no reconstruction slice!")
        self.view_count = int(np.ceil(self.short_scan_range / abs(self.angle_per_view)))
        self.short_scan_range_actual = self.view_count * abs(self.angle_per_view)
        self._log("Reconstruction Z coverage: %.1f mm to %.1f mm" % (self.array_z_pos[0], self.array_z_pos[-1]))
        self._log("Size of rebinned sinogram is %d x %d (%.1f degrees scan)"
                  % (self.det_elem_count_horizontal, self.view_count, np.rad2deg(self.short_scan_range_actual)))
        self.img_recon = np.zeros((len(self.array_z_pos), self.img_dim, self.img_dim), dtype=np.float32)

    # ------------------------------------------------------------ geometry
    def added_rotation(self):
        """img_rot_add of every slice (CalculateAddedImgRotation, :168-171)."""
        z = self.array_z_pos.astype(np.float64)
        v0 = (z - self.det_offset_vertical_at_isocenter) / self.dis_per_view
        return np.floor(v0 - 0.5 * (self.view_count - 1.0)) * self.angle_per_view

    def fan_object(self, rows):
        """The parameters ChangeReconParameterValues (:207-245) leaves: a 1-row fan
        geometry of view_count views over short_scan_range_actual (here `rows` rows,
        one per slice, which only the weighting and filter see)."""
        o = copy.copy(self)
        o.det_elem_count_vertical = o.det_elem_count_vertical_actual = rows
        o.det_elem_vertical_recon_range_begin = 0
        o.cone_beam = False
        o.total_scan_angle = self.short_scan_range_actual * np.sign(self.total_scan_angle)
        o.short_scan = 0 if abs(o.total_scan_angle % (2 * PI)) < (0.01 / 180 * PI) else 1
        o.view_num = o.sgm_height = self.view_count
        o.img_dim_z = rows
        o.bool_apply_pmatrix = False
        return o

    # ------------------------------------------------------------ driver
    def MainFunction(self):  # noqa: N802 - reference name
        """run_mgfbp_helical.py:98-166."""
        if self.kernel_name is None:
            raise ConfigError("ERROR: no reconstruction kernel (HammingFilter, GaussianApodizedRamp or None) "
                              "in the config!")
        if self.det_elem_count_vertical_actual != self.det_elem_count_vertical:
            raise ConfigError("ERROR: helical rebinning needs the full detector (no vertical recon range)!")
        self.file_processed_count = 0
        os.makedirs(os.path.join(self.input_dir, "temp"), exist_ok=True)

        def compute(d):
            d.file_processed_count += 1
            d._log("\nReconstructing %s ..." % d.input_path)
            d.img_recon = d.reconstruct(d._device_sinogram()).cpu().numpy()
            d._log("\nSaving to %s !" % d.output_path)

        # the next file is read and the previous one written while this one runs
        files = [f for f in os.listdir(self.input_dir) if re.match(self.input_files_pattern, f)]
        run_over_files(self, files, lambda d, f: d.ReadSinogram(f), compute, lambda d: d.SaveReconImg())
        return self.img_recon

    def _device_sinogram(self):
        dev = torch.device(self.device or "cuda")
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        t = torch.from_numpy(np.ascontiguousarray(self._raw)).to(dev)
        if self._view_stride != self.det_elem_count_horizontal:  # post-log stack [views][rows][cols]
            t = t.permute(1, 0, 2).contiguous()
        return t

    def reconstruct(self, sgm, save_rebinned=True):
        """All slices of one helical sinogram sgm [rows][views][cols] (device).
        save_rebinned writes the rebinned stack to InputDir/temp/sgm_rebin.raw, as the
        reference's driver does (imaddRaw)."""
        dev = sgm.device
        nz, vc, nu, n = len(self.array_z_pos), self.view_count, self.det_elem_count_horizontal, self.img_dim
        # 1. rebinning of every slice
        h = Helical(nu=nu, nv=self.det_elem_count_vertical, views=self.view_num, view_count=vc, n_slices=nz,
                    dv=self.det_elem_height, sdd=self.source_det_dis, mag=self.mag_ratio_isocenter,
                    det_offset_vertical=self.det_offset_vertical, dis_per_view=self.dis_per_view)
        z_pos = torch.from_numpy(self.array_z_pos).to(dev)
        stack = torch.empty((nz, vc, nu), dtype=torch.float32, device=dev)
        _lib.call("mct_helical_rebin", ctypes.byref(h), ops._ptr(sgm), ops._ptr(z_pos), ops._ptr(stack),
                  ops._stream())
        if save_rebinned:  # as imaddRaw leaves it
            stack.cpu().numpy().tofile(os.path.join(self.input_dir, "temp", "sgm_rebin.raw"))
        # 2. weighting + row filter over the stack (slices as rows)
        stack_obj = self.fan_object(nz)
        pipe = FdkPipeline(stack_obj, device=dev, storage="f32")
        if not self.apply_gauss_vertical and pipe.tc is not None:
            # weighting inside the tensor-core filter's operand split: [views][slices][cols]
            filt = pipe.filter(stack, vc * nu, nu)
        else:
            w = ops.weight(pipe.dg, stack, vc * nu, nu, pipe.bh, out=pipe.weighted)
            if self.apply_gauss_vertical:
                # the 1-row vertical convolution of the reference uses the first tap of the
                # full-detector Gaussian it built in __init__ (run_mgfbp.py:298-309, 1020-1029)
                g = gaussian_taps(self.det_elem_count_vertical_actual, self.det_elem_height,
                                  self.det_elem_vertical_gauss_filter_size)
                w = w * float(np.float32(g[0])) * float(np.float32(self.det_elem_height))
            if pipe.kernel_none:
                filt = w.permute(1, 0, 2)
            elif pipe.tc is not None:
                filt = pipe.tc(w, out=pipe.filtered)  # [views][slices][cols]
            else:
                filt = ops.filter_rows(pipe.dg, w, pipe.taps, out=pipe.filtered)
        if self.save_filtered_sinogram:  # the reference leaves the last slice's, as [views][1][cols]
            imwriteTiff(filt[:, nz - 1:nz, :].cpu().numpy(), self.output_dir + "/sgm_filtered_" + self.output_file)
        # 3. slice-major pack (one 1-row fan sinogram of vc views per slice) and
        #    per-slice backprojection with the slice's angles
        per_slice = filt.permute(1, 0, 2).contiguous()  # [slices][views][cols]
        fan = self.fan_object(1)
        dg1 = fbp_geometry(fan, dev)
        packed_obj = copy.copy(fan)
        packed_obj.view_num = nz * vc
        dgp = fbp_geometry(packed_obj, dev)
        packed = ops.pack(dgp, per_slice.view(nz * vc, 1, nu), MCT_F32)
        base = (fan.total_scan_angle / vc * np.arange(vc, dtype=np.float32)).astype(np.float32)
        adds = self.added_rotation()
        rots = (np.float32(self.img_rot) + adds.astype(np.float32)).astype(np.float32)
        angles = torch.from_numpy((base[None, :] + rots[:, None]).astype(np.float32)).to(dev)  # [slices][views]
        vol = torch.empty((nz, n, n), dtype=torch.float32, device=dev)
        g = dg1.geom
        slice_bytes = vc * (nu - 1) * 8
        for s in range(nz):
            gs = g.copy(img_rot=float(rots[s]))
            ts = Tables(angles=angles.data_ptr() + s * vc * 4, u=dg1.tables.u, v=dg1.tables.v)
            _lib.call("mct_fdk_bp", ctypes.byref(gs), ctypes.byref(ts), ctypes.c_void_p(packed.data_ptr() + s * slice_bytes),
                      MCT_F32, ctypes.c_void_p(vol.data_ptr() + s * n * n * 4), ops._stream())
        return vol


def run_mgfbp_helical(file_path, device=None, verbose=True):
    """Drop-in for run_mgfbp_helical.run_mgfbp_helical (run_mgfbp_helical.py:25-54)."""
    start = time.time()
    if verbose:
        print("Performing Helical Rebin and FBP from MandoCT-GB300 ...")
    if not os.path.exists(file_path):
        raise ConfigError(f"ERROR: Config File {file_path} does not exist!")
    fbp = Mgfbp_helical(ReadConfigFile(file_path), device=device, verbose=verbose)
    img = fbp.MainFunction()
    gc.collect()
    if verbose:
        if fbp.file_processed_count > 0:
            print(f"\nA total of {fbp.file_processed_count:d} file(s) are reconstructed!")
            print(f"Time cost: {time.time() - start:.3} sec\n")
        else:
            print(f"\nWarning: Did not find files like {fbp.input_files_pattern:s} in {fbp.input_dir:s}.")
            print("No images are reconstructed!")
    del fbp
    return img
