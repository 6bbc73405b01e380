"""Iterative reconstruction drop-ins: IRN-CGLS-TV (Mgfbp_ir, run_mgfbp_ir) and
IRN-CGLS-PICCS (Mgfbp_ir_piccs, run_mgfbp_ir_piccs).

Mirrors run_mgfbp_iterative_recon_IRN_CGLS.py:14-370 and
run_mgfbp_iterative_recon_IRN_CGLS_piccs.py:13-161 with everything resident on the
GPU: the reference moves the whole volume between host and device for every
P^T P and runs the CG vector algebra in NumPy; here each CG iteration is one FP
launch, one BP launch (with 16-bit gathers the TV terms and the float64 inner product
<d, q> ride in its epilogue; with float32 gathers the TV stencil and <d, q> are one
more pass), and two fused vector updates (the first also yields |r|^2 for the next
iteration), with alpha and beta kept on the device.

Operators: by default the reference's pair (masked trilinear FP and the
voxel-driven per-view backprojector with distance_factor*pixel_size weights);
config key "BackProjector": "adjoint" selects the exact transpose of the FP.
"""
import gc
import os
import re
import time

import numpy as np
import torch

from . import ops
from .config import ConfigError, ReadConfigFile, parse_fbp, parse_fpj, parse_fpj_v3, parse_ir, parse_piccs
from .fbp import Mgfbp
from .geometry import ir_geometry
from .io import imreadRaw, imwriteRaw, imwriteTiff, read_sinogram_file


class IrSystem:
    """P (masked FP), P^T (reference backprojector or exact adjoint), the TV
    operators and CGLS for one iterative-reconstruction geometry."""

    def __init__(self, obj, device=None, storage=None):
        if not torch.cuda.is_available():
            raise RuntimeError("a CUDA device is required (this package has no CPU fallback)")
        self.obj = obj
        self.dg = ir_geometry(obj, device)
        self.device = self.dg.device
        self.matched = getattr(obj, "back_projector", "reference") == "adjoint"
        storage = storage or getattr(obj, "storage_precision", "float32")
        kinds = {"float32": ops.MCT_F32, "bfloat16": ops.MCT_BF16, "float16": ops.MCT_F16}
        if storage not in kinds:
            raise ValueError("storage must be float32, bfloat16 or float16")
        # 16-bit gathers: FP volume cells (cone beam) and the packed sinogram of the
        # reference backprojector; the exact adjoint scatters float32 either way
        self.dtype = kinds[storage]
        self.fp_dtype = self.dtype if self.dg.geom.flags & ops.MCT_CONE else ops.MCT_F32
        self.data_dtype = kinds[getattr(obj, "sinogram_precision", "float32")]
        self.iter_dtype = {"float32": torch.float32, "bfloat16": torch.bfloat16}[
            getattr(obj, "iterate_storage", "float32")]
        if self.iter_dtype != torch.float32 and (self.matched or not (self.dg.geom.flags & ops.MCT_CONE)
                                                 or self.dg.geom.view_mode != 1):
            raise ConfigError("ERROR: IterateStorage bfloat16 needs cone beam, the reference backprojector and the "
                              "axial view mode")
        self.mask = ops.effective_map(self.dg)
        f32 = dict(dtype=torch.float32, device=self.device)
        self.fp_buf = torch.empty(self.dg.sgm_shape, **f32)
        self.ptp_calls = 0
        self._rr = torch.empty((), dtype=torch.float64, device=self.device)
        self._dq = torch.empty((), dtype=torch.float64, device=self.device)
        self._rr_new = torch.empty((), dtype=torch.float64, device=self.device)

    # ------------------------------------------------------------ operators
    def fp(self, x, out=None):
        return ops.fp(self.dg, x, mask=self.mask, out=out, dtype=self.fp_dtype)

    def _pack(self, sgm, dtype):
        """The sinogram as one-gather bilinear coefficients of storage type dtype, in a
        buffer kept per type."""
        packed = self.__dict__.setdefault("_packed", {})
        if dtype not in packed:
            packed[dtype] = torch.empty(max(ops.packed_bytes(self.dg, dtype), 16), dtype=torch.uint8,
                                        device=self.device)
        return ops.pack_sinogram(self.dg, sgm, dtype=dtype, out=packed[dtype])

    def bp(self, sgm, out=None, dtype=None):
        if self.matched:
            return ops.fp_adjoint(self.dg, sgm, mask=self.mask, out=out)
        dtype = self.dtype if dtype is None else dtype
        return ops.bp_unmatched_packed(self.dg, self._pack(sgm, dtype), dtype=dtype, out=out)

    def ptp(self, x, out=None, full_precision=False):
        """P^T P x (run_mgfbp_iterative_recon_IRN_CGLS.py:288-316).  full_precision
        forces float32 gathers whatever the storage precision."""
        self.ptp_calls += 1
        if full_precision:
            q = ops.fp(self.dg, x, mask=self.mask, out=self.fp_buf)
            return self.bp(q, out=out, dtype=ops.MCT_F32)
        return self.bp(self.fp(x, out=self.fp_buf), out=out)

    def bp_b(self, sgm):
        """P^T (b * mask) (run_mgfbp_iterative_recon_IRN_CGLS.py:319-336).  The measured
        data is stored (packed) at the sinogram precision, float32 unless the config
        asks for 16 bits: rounding b to bf16 adds noise of the order of the photon
        noise, which the iterations would fit; float16 with its power-of-two scale
        rounds to 2^-11 of the largest value's binade."""
        return self.bp(sgm * self.mask, dtype=self.data_dtype)

    def fused_cg(self, n_terms):
        """Whether one CG iteration's operator, TV terms and <d, q> run as the
        backprojector's epilogue (reference backprojector, axial cone beam, at most two
        TV terms); otherwise they are separate passes.  By default the epilogue is used
        with 16-bit gathers, where it measured faster (512^2 x 64, 360 views: 22.96 ms
        per iteration against 23.11 with bf16 gathers); with float32 gathers the fused
        kernel measured 25.89 against 25.20 ms and the separate passes stay.  Setting
        the attribute `fuse` to True or False overrides the choice."""
        g = self.dg.geom
        fuse = self.__dict__.get("fuse")
        if fuse is None:
            fuse = self.dtype != ops.MCT_F32
        return (fuse and not self.matched and bool(g.flags & ops.MCT_CONE) and g.view_mode == 1
                and n_terms <= 2)

    def ptp_cg(self, d, q, op_terms, dq):
        """q = P^T P d + sum_k s_k D^T W_k D d and dq = <d, q>: FP, pack, then the
        backprojector with the TV terms and the inner product in its epilogue."""
        self.ptp_calls += 1
        packed = self._pack(self.fp(d, out=self.fp_buf), self.dtype)
        return ops.bp_unmatched_packed_cg(self.dg, packed, self.dtype, d, list(op_terms), q, dq)

    def dtwd_acc(self, x, wr, s, acc):
        """acc += s * D^T W D x (in place)."""
        return ops.dtwd(self.dg, x, wr, s, out_in=acc, a=1.0, out=acc)

    # ------------------------------------------------------------ CGLS
    def cgls(self, x_seed, rhs_terms, op_terms, n_iter):
        """CG on (P^T P + sum_k s_k D^T W_k D) x = b' from x_seed, where
        b' = P^T b + sum (s, W, y) s * D^T W D y.  Follows TikhonovSol
        (run_mgfbp_iterative_recon_IRN_CGLS.py:188-232 and ..._piccs.py:112-145).
        rhs_terms: list of (s, W, y); op_terms: list of (s, W).
        The initial residual uses float32 gathers whatever the storage precision: with a
        warm start (the previous reweighting's solution, or the PICCS prior) P^T P x_seed
        is of the size of P^T b, and rounding x_seed to bf16 would perturb the right-hand
        side like measurement noise; the per-iteration products P^T P d use the storage
        precision."""
        x0 = x_seed if x_seed.dtype == torch.float32 else x_seed.float()
        d = self.ptp(x0, full_precision=True)
        torch.sub(self.bpb, d, out=d)  # d = P^T b - P^T P x0 (float32 whatever the storage)
        for s, w, y in rhs_terms:
            self.dtwd_acc(y, w, s, d)
        for s, w in op_terms:
            self.dtwd_acc(x0, w, -s, d)
        it = self.iter_dtype
        if it != torch.float32:  # iterates stored rounded to bf16 from here on
            d = d.to(it)
        r = d.clone()
        x = x_seed.to(it, copy=True)
        q = torch.empty_like(x)
        rr, rr_new = self._rr, self._rr_new
        ops.dot(r, r, out=rr)
        fused = self.fused_cg(len(op_terms))
        for _ in range(n_iter):
            if fused:
                # q = P^T P d + the TV terms and <d, q> in the backprojector's epilogue
                self.ptp_cg(d, q, op_terms, self._dq)
            else:
                self.ptp(d, out=q)
                # the last TV term is added in the same pass as <d, q>
                for s, w in op_terms[:-1]:
                    self.dtwd_acc(d, w, s, q)
                if op_terms:
                    ops.dtwd_dot(self.dg, d, op_terms[-1][1], op_terms[-1][0], q, self._dq)
                else:
                    ops.dot(d, q, out=self._dq)
            # x += alpha d, r -= alpha q and rr_new = |r|^2 in one pass; |r|^2 of this
            # iteration is the next iteration's rr (no separate pass over r)
            ops.cgls_update(rr, self._dq, x, r, d, q, rr_new)
            ops.cgls_direction(rr, rr_new, r, d)
            rr, rr_new = rr_new, rr
        return x

    def loss_tv(self, x, sgm, lam, beta, extra=None):
        """0.5 |P x - b*mask|^2 / N_sgm + lam * TV(x) / N_img (IRN_CGLS.py:184-186)."""
        obj = self.obj
        diff = self.fp(x) - sgm * self.mask
        data = 0.5 * float(ops.dot(diff, diff)) / obj.sgm_total_pixel_count
        return data + lam * float(ops.tv_penalty(self.dg, x.float(), beta)) / obj.img_total_pixel_count


class Mgfbp_ir:  # noqa: N801 - reference name
    """Drop-in for Mgfbp_ir (run_mgfbp_iterative_recon_IRN_CGLS.py:53-493)."""

    def __init__(self, config_dict, device=None, verbose=True, compute_loss=False):
        self.verbose = verbose
        parse_fbp(self, config_dict)
        parse_fpj(self, config_dict)
        parse_fpj_v3(self, config_dict)
        parse_ir(self, config_dict)
        self.device = device
        self.compute_loss = compute_loss
        self.loss = np.empty(0)
        self.num_iter_runned = 0
        self.file_processed_count = 0
        self.img_recon = np.zeros((self.img_dim_z, self.img_dim, self.img_dim), dtype=np.float32)
        self.img_x = np.zeros_like(self.img_recon)
        self._sys = None

    @property
    def system(self):
        if self._sys is None:
            self._sys = IrSystem(self, self.device)
        return self._sys

    def _log(self, msg):
        if self.verbose:
            print(msg)

    def output_name(self, file):
        out = file
        for i in range(int(len(self.output_file_replace) / 2)):
            out = re.sub(self.output_file_replace[2 * i], self.output_file_replace[2 * i + 1], out)
        if out == file:
            raise ConfigError(f"ERROR: did not file string to replace in '{out}'")
        if self.output_file_format in ("tif", "tiff"):
            out = re.sub(".raw", ".tif", out)
        return out

    def ReadSinogram(self, file):  # noqa: N802 - reference name
        self.input_path = os.path.join(self.input_dir, file)
        self.output_file = self.output_name(file)
        self.output_path = os.path.join(self.output_dir, self.output_file_prefix + self.output_file)
        self.img_sgm = read_sinogram_file(self, self.input_path)
        return True

    def SaveReconImg(self):  # noqa: N802 - reference name
        """run_mgfbp_iterative_recon_IRN_CGLS.py:485-492."""
        self.img_recon = self.img_x
        if self.convert_to_HU:
            self.img_recon = (self.img_recon / self.water_mu - 1) * 1000
        if self.output_file_format == "raw":
            imwriteRaw(self.img_recon, self.output_path, dtype=np.float32)
        else:
            imwriteTiff(self.img_recon, self.output_path, dtype=np.float32)

    def _to_mu(self, img_hu):
        if self.convert_to_HU:
            return ((img_hu / 1000 + 1) * self.water_mu).astype(np.float32)
        return np.asarray(img_hu, dtype=np.float32)

    def solve_tv(self, sgm_dev, x0_dev):
        """IRN-CGLS-TV on device tensors (run_mgfbp_iterative_recon_IRN_CGLS.py:157-172)."""
        sy = self.system
        lr = self.coef_lambda * self.pixel_count_ratio
        sy.bpb = sy.bp_b(sgm_dev)
        wr = torch.ones_like(x0_dev)
        x = sy.cgls(x0_dev, [], [(lr, wr)], self.num_iter)
        if self.compute_loss:
            self.loss = np.append(self.loss, sy.loss_tv(x, sgm_dev, self.coef_lambda, self.beta_tv))
        for _ in range(self.num_irn_iter):
            ops.tv_weights(sy.dg, x, self.beta_tv, out=wr)
            x = sy.cgls(x, [], [(lr, wr)], self.num_iter)
            if self.compute_loss:
                self.loss = np.append(self.loss, sy.loss_tv(x, sgm_dev, self.coef_lambda, self.beta_tv))
        self.num_iter_runned = sy.ptp_calls
        return x.float()

    def MainFunction(self, img_recon_seed):  # noqa: N802 - reference name
        """run_mgfbp_iterative_recon_IRN_CGLS.py:138-176."""
        self.file_processed_count = 0
        for file in os.listdir(self.input_dir):
            if re.match(self.input_files_pattern, file):
                if self.ReadSinogram(file):
                    self.file_processed_count += 1
                    self._log("Reconstructing %s ..." % self.input_path)
                    sy = self.system
                    sgm = torch.from_numpy(self.img_sgm).to(sy.device)
                    x0 = torch.from_numpy(self._to_mu(img_recon_seed)).to(sy.device)
                    x = self.solve_tv(sgm, x0)
                    self.img_x = x.cpu().numpy()
                    self._log("\nSaving to %s !" % self.output_path)
                    self.SaveReconImg()
        return self.img_recon


class Mgfbp_ir_piccs(Mgfbp_ir):  # noqa: N801 - reference name
    """Drop-in for Mgfbp_ir_piccs (run_mgfbp_iterative_recon_IRN_CGLS_piccs.py:48-161)."""

    def __init__(self, config_dict, device=None, verbose=True, compute_loss=False):
        super().__init__(config_dict, device=device, verbose=verbose, compute_loss=compute_loss)
        parse_piccs(self, config_dict)
        prior = imreadRaw(self.prior_image_file, width=self.img_dim, height=self.img_dim, nSlice=self.img_dim_z)
        prior = prior.reshape(self.img_dim_z, self.img_dim, self.img_dim)
        if self.convert_to_HU:
            prior = (prior / 1000 + 1) * self.water_mu
        self.img_prior = np.asarray(prior, dtype=np.float32)

    def solve_piccs(self, sgm_dev, prior_dev):
        """run_mgfbp_iterative_recon_IRN_CGLS_piccs.py:89-105 with TikhonovSol :112-145."""
        sy = self.system
        lam, a, ratio = self.coef_lambda, self.coef_alpha, self.pixel_count_ratio
        s_tv, s_pr = lam * (1 - a) * ratio, lam * a * ratio
        sy.bpb = sy.bp_b(sgm_dev)
        wr = torch.ones_like(prior_dev)
        wrp = torch.ones_like(prior_dev)
        diff = torch.empty_like(prior_dev)
        x = sy.cgls(prior_dev, [(s_pr, wrp, prior_dev)], [(s_tv, wr), (s_pr, wrp)], self.num_iter)
        for _ in range(self.num_irn_iter):
            ops.tv_weights(sy.dg, x, self.beta_tv, out=wr)
            torch.sub(x, prior_dev, out=diff)
            ops.tv_weights(sy.dg, diff, self.beta_tv, out=wrp)
            x = sy.cgls(x, [(s_pr, wrp, prior_dev)], [(s_tv, wr), (s_pr, wrp)], self.num_iter)
        self.num_iter_runned = sy.ptp_calls
        return x.float()

    def MainFunction(self):  # noqa: N802 - reference name
        """run_mgfbp_iterative_recon_IRN_CGLS_piccs.py:70-110."""
        self.file_processed_count = 0
        for file in os.listdir(self.input_dir):
            if re.match(self.input_files_pattern, file):
                if self.ReadSinogram(file):
                    self.file_processed_count += 1
                    self._log("Reconstructing %s ..." % self.input_path)
                    sy = self.system
                    sgm = torch.from_numpy(self.img_sgm).to(sy.device)
                    prior = torch.from_numpy(self.img_prior).to(sy.device)
                    x = self.solve_piccs(sgm, prior)
                    self.img_x = x.cpu().numpy()
                    self._log("\nSaving to %s !" % self.output_path)
                    self.SaveReconImg()
        return self.img_recon


def run_mgfbp_ir(file_path, device=None, verbose=True):
    """Drop-in for run_mgfbp_iterative_recon_IRN_CGLS.run_mgfbp_ir (:14-49): FBP
    seed, then IRN-CGLS-TV; returns the reconstruction (HU if WaterMu)."""
    if not os.path.exists(file_path):
        raise ConfigError(f"ERROR: Config File {file_path} does not exist!")
    seed = Mgfbp(ReadConfigFile(file_path), device=device, verbose=verbose).MainFunction()
    start = time.time()
    ir = Mgfbp_ir(ReadConfigFile(file_path), device=device, verbose=verbose)
    img = ir.MainFunction(seed)
    if verbose and ir.file_processed_count > 0:
        t = time.time() - start
        print(f"\nA total of {ir.file_processed_count:d} file(s) are reconstructed!")
        print(f"Time cost: {t:.3} sec ({t / max(ir.num_iter_runned, 1) / ir.file_processed_count:.3} sec per iteration).")
    gc.collect()
    return img


def run_mgfbp_ir_piccs(file_path, device=None, verbose=True):
    """Drop-in for run_mgfbp_iterative_recon_IRN_CGLS_piccs.run_mgfbp_ir (:13-45)."""
    if not os.path.exists(file_path):
        raise ConfigError(f"ERROR: Config File {file_path} does not exist!")
    start = time.time()
    ir = Mgfbp_ir_piccs(ReadConfigFile(file_path), device=device, verbose=verbose)
    img = ir.MainFunction()
    if verbose and ir.file_processed_count > 0:
        t = time.time() - start
        print(f"\nA total of {ir.file_processed_count:d} file(s) are reconstructed!")
        print(f"Time cost: {t:.3} sec ({t / max(ir.num_iter_runned, 1) / ir.file_processed_count:.3} sec per iteration).")
    gc.collect()
    return img
