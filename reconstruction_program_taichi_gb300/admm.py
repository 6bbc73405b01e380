"""ADMM-TV iterative reconstruction: drop-in for run_mgfbp_iterative_recon_ADMM_CGLS.py
(its `run_mgfbp_ir` and its `Mgfbp_ir_piccs` class, an ADMM variant despite the name;
here `run_mgfbp_ir_admm` and `Mgfbp_ir_admm`, with the reference's names as aliases).

The reference alternates, for NumberOfIRNIterations outer steps (:107-125):
  x-step  NumberOfIterations CGLS iterations on (P^T P + rho D^T D) x =
          P^T b + rho (Dt v_y + Dt v_x) - (Dt p_y + Dt p_x)            (:145-162)
  v-step  v = w where |w| > lambda * ratio / rho, else 0, w = D x + p / rho   (:128-136)
  p-step  p += rho (D x - v)                                                 (:139-140)
with rho = 0.1, D the in-plane forward differences and D^T D the 3D interior stencil
of Dt_W_D with unit weights.  Everything stays on the device: the x-step is the
shared CGLS (IrSystem.cgls) with the right-hand side from `mct_admm_rhs`, and the
v- and p-steps are one fused pass (`mct_admm_shrink`).
"""
import gc
import os
import re
import time

import numpy as np
import torch

from . import _lib, ops
from .config import ConfigError, ReadConfigFile, parse_piccs
from .fbp import Mgfbp
from .io import imreadRaw
from .ir import Mgfbp_ir


class Mgfbp_ir_admm(Mgfbp_ir):  # noqa: N801 - reference style
    """Drop-in for the ADMM class of run_mgfbp_iterative_recon_ADMM_CGLS.py:50-221."""

    def __init__(self, config_dict, device=None, verbose=True, compute_loss=False):
        super().__init__(config_dict, device=device, verbose=verbose, compute_loss=compute_loss)
        parse_piccs(self, config_dict)  # Alpha and PriorImageFile are read as the reference does (:55-71)
        prior = imreadRaw(self.prior_image_file, width=self.img_dim, height=self.img_dim, nSlice=self.img_dim_z)
        prior = prior.reshape(self.img_dim_z, self.img_dim, self.img_dim)
        if self.convert_to_HU:
            prior = (prior / 1000 + 1) * self.water_mu
        self.img_prior = np.asarray(prior, dtype=np.float32)
        self.coef_rho = 0.1

    def solve_admm(self, sgm_dev, x0_dev):
        """The ADMM loop on device tensors; returns x (and keeps v, p as attributes)."""
        sy = self.system
        dg, rho = sy.dg, self.coef_rho
        g = dg.g()
        stream = ops._stream()
        x = x0_dev.clone()
        # v = D x (:93-94); p = 0 (:72-76: the duals start as the zero arrays v had)
        vy, vx = torch.zeros_like(x), torch.zeros_like(x)
        py, px = torch.zeros_like(x), torch.zeros_like(x)
        zero = torch.zeros_like(x)
        _lib.call("mct_admm_shrink", g, ops._ptr(x), 1.0, -1.0, ops._ptr(vy), ops._ptr(vx), ops._ptr(zero),
                  ops._ptr(zero), stream)  # threshold -1 keeps every w: v = D x (the p written to `zero` is unused)
        bpb = sy.bp_b(sgm_dev)
        ones = torch.ones_like(x)
        thr = self.coef_lambda * self.pixel_count_ratio / rho
        for _ in range(self.num_irn_iter):
            rhs = torch.empty_like(x)
            _lib.call("mct_admm_rhs", g, ops._ptr(bpb), ops._ptr(vy), ops._ptr(vx), ops._ptr(py), ops._ptr(px),
                      float(rho), ops._ptr(rhs), stream)
            sy.bpb = rhs
            x = sy.cgls(x, [], [(rho, ones)], self.num_iter)
            _lib.call("mct_admm_shrink", g, ops._ptr(x), float(rho), float(thr), ops._ptr(vy), ops._ptr(vx),
                      ops._ptr(py), ops._ptr(px), stream)
            if self.compute_loss:
                self.loss = np.append(self.loss, self._loss(x, sgm_dev))
        self.v, self.p = (vy, vx), (py, px)
        self.num_iter_runned = sy.ptp_calls
        return x

    def _loss(self, x, sgm):
        """LossValCalc of the ADMM script (:216-219)."""
        sy = self.system
        prior = torch.from_numpy(self.img_prior).to(x.device)
        diff = sy.fp(x) - sgm * sy.mask
        lam, a = self.coef_lambda, self.coef_alpha
        return (0.5 * float(ops.dot(diff, diff)) / self.sgm_total_pixel_count
                + lam * (1 - a) * float(ops.tv_penalty(sy.dg, x, self.beta_tv)) / self.img_total_pixel_count
                + lam * a * float(ops.tv_penalty(sy.dg, x - prior, self.beta_tv)) / self.img_total_pixel_count)

    def MainFunction(self, img_recon_seed):  # noqa: N802 - reference name
        """run_mgfbp_iterative_recon_ADMM_CGLS.py:79-147 (the reference also saves the
        image after every outer step; here it is saved once, at the end)."""
        self.file_processed_count = 0
        for file in os.listdir(self.input_dir):
            if re.match(self.input_files_pattern, file):
                if self.ReadSinogram(file):
                    self.file_processed_count += 1
                    self._log("Reconstructing %s ..." % self.input_path)
                    sy = self.system
                    sgm = torch.from_numpy(self.img_sgm).to(sy.device)
                    x0 = torch.from_numpy(self._to_mu(img_recon_seed)).to(sy.device)
                    self.img_x = self.solve_admm(sgm, x0).cpu().numpy()
                    self._log("\nSaving to %s !" % self.output_path)
                    self.SaveReconImg()
        return self.img_recon


def run_mgfbp_ir_admm(file_path, device=None, verbose=True):
    """Drop-in for run_mgfbp_iterative_recon_ADMM_CGLS.run_mgfbp_ir (:14-47): FBP seed,
    then ADMM-TV; returns the reconstruction (HU if WaterMu)."""
    if not os.path.exists(file_path):
        raise ConfigError(f"ERROR: Config File {file_path} does not exist!")
    seed = Mgfbp(ReadConfigFile(file_path), device=device, verbose=verbose).MainFunction()
    start = time.time()
    ir = Mgfbp_ir_admm(ReadConfigFile(file_path), device=device, verbose=verbose)
    img = ir.MainFunction(seed)
    if verbose and ir.file_processed_count > 0:
        t = time.time() - start
        print(f"\nA total of {ir.file_processed_count:d} file(s) are reconstructed!")
        print(f"Time cost: {t:.3} sec ({t / max(ir.num_iter_runned, 1) / ir.file_processed_count:.3} sec per iteration).")
    gc.collect()
    return img


# the reference file's own names
run_mgfbp_ir = run_mgfbp_ir_admm
Mgfbp_ir_piccs = Mgfbp_ir_admm
