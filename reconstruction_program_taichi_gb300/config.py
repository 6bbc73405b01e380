"""jsonc configuration: loading and parameter parsing with the reference's keys,
aliases, defaults and validation rules.

Follows Mgfbp.__init__ (run_mgfbp.py:87-719), Mgfpj.__init__ (run_mgfpj_v2.py:113-214),
Mgfpj_v3.__init__ (run_mgfpj_v3.py:129-181), Mgfbp_ir.__init__
(run_mgfbp_iterative_recon_IRN_CGLS.py:54-136) and Mgfbp_ir_piccs.__init__
(run_mgfbp_iterative_recon_IRN_CGLS_piccs.py:50-67).  Where the reference prints
"ERROR: ..." and calls sys.exit(), this module raises ConfigError with the same
message.
"""
import json
import os
import re

import numpy as np

PI = 3.1415926536  # run_mgfbp.py:16


class ConfigError(ValueError):
    """Invalid or missing configuration parameter (the reference exits instead)."""


def remove_comments(jsonc_str):
    """Strip // and /* */ comments (run_mgfbp.py:1313-1316)."""
    pattern = re.compile(r"//.*?$|/\*.*?\*/", re.MULTILINE | re.DOTALL)
    return re.sub(pattern, "", jsonc_str)


def load_jsonc(file_path):
    """Parse a jsonc file into a dict (run_mgfbp.py:1323-1329)."""
    with open(file_path, "r") as f:
        return json.loads(remove_comments(f.read()))


def save_jsonc(save_path, data):
    """Write a dict as json to a *.jsonc path (run_mgfbp.py:1318-1321)."""
    if save_path.split(".")[-1] != "jsonc":
        raise ConfigError("save_jsonc: path must end with .jsonc")
    with open(save_path, "w") as f:
        json.dump(data, f)


def ReadConfigFile(file_path):  # noqa: N802 - reference name
    """Alias of load_jsonc (run_mgfbp.py:1344-1349)."""
    return load_jsonc(file_path)


def _is_number(x):
    return isinstance(x, (float, int))


def _err(msg):
    raise ConfigError("ERROR: " + msg)


def _log(obj, msg):
    if getattr(obj, "verbose", True):
        print(msg)


def parse_fbp(self, cfg):
    """Mgfbp.__init__ parameter handling, run_mgfbp.py:87-719 (PMatrix handling is
    delegated to pmatrix.apply_pmatrix_config)."""
    self.config_dict = cfg
    # ---- file names (:89-133)
    for key, attr in (("InputDir", "input_dir"), ("OutputDir", "output_dir"), ("InputFiles", "input_files_pattern"),
                      ("OutputFilePrefix", "output_file_prefix")):
        if key not in cfg:
            _err(f"Can not find {key} in the config file!")
        if not isinstance(cfg[key], str):
            _err(f"{key} is not a string!")
        setattr(self, attr, cfg[key])
    if "OutputFileReplace" not in cfg:
        _err("Can not find OutputFileReplace in the config file!")
    self.output_file_replace = cfg["OutputFileReplace"]
    if not os.path.exists(self.output_dir):
        os.makedirs(self.output_dir)
    self.output_file_format = cfg.get("OutputFileFormat", "raw")
    if self.output_file_format not in ("raw", "tif", "tiff"):
        _err("Output file format can only be 'raw', 'tif' or 'tiff' !")
    self.input_file_form = cfg.get("InputFileForm", "sinogram")
    if self.input_file_form not in ("sinogram", "post_log_images"):
        _err("InputFileForm can only be sinogram or post_log_images!")
    self.output_file_form = cfg.get("OutputFileForm", "sinogram")
    if self.output_file_form not in ("sinogram", "post_log_images"):
        _err("OutputFileForm can only be sinogram or post_log_images!")
    # ---- first sinogram slice = top or bottom detector row (:165-185)
    if self.input_file_form == "post_log_images" or self.output_file_form == "post_log_images":
        self.first_slice_top_row = True
    elif "FirstSinogramSliceIsDetectorTopRow" in cfg:
        if not isinstance(cfg["FirstSinogramSliceIsDetectorTopRow"], bool):
            _err("FirstSinogramSliceIsDetectorTopRow can only be true or false!")
        self.first_slice_top_row = cfg["FirstSinogramSliceIsDetectorTopRow"]
    else:
        self.first_slice_top_row = False
    self.positive_v_is_positive_z = -1 if self.first_slice_top_row else 1
    if "SaveFilteredSinogram" in cfg:
        if not isinstance(cfg["SaveFilteredSinogram"], bool):
            _err("SaveFilteredSinogram can only be true or false!")
        self.save_filtered_sinogram = cfg["SaveFilteredSinogram"]
    else:
        self.save_filtered_sinogram = False
    # ---- detector (:199-313)
    if "CurvedDetector" in cfg:
        if not isinstance(cfg["CurvedDetector"], bool):
            _err("CurvedDetector can only be true or false!")
        self.curved_dect = cfg["CurvedDetector"]
    else:
        self.curved_dect = False
    if "DetectorElementCountHorizontal" in cfg:
        self.det_elem_count_horizontal = cfg["DetectorElementCountHorizontal"]
    elif "SinogramWidth" in cfg:
        self.det_elem_count_horizontal = cfg["SinogramWidth"]
    else:
        _err("Can not find detector element count along horizontal direction!")
    if self.det_elem_count_horizontal <= 0:
        _err("DetectorElementCountHorizontal (SinogramWidth) should be larger than 0!")
    elif self.det_elem_count_horizontal % 1 != 0:
        _err("DetectorElementCountHorizontal (SinogramWidth) should be an integer!")
    self.det_elem_count_horizontal = int(self.det_elem_count_horizontal)
    if "DetectorElementWidth" in cfg:
        self.det_elem_width = cfg["DetectorElementWidth"]
    elif "DetectorElementSize" in cfg:
        self.det_elem_width = cfg["DetectorElementSize"]
    else:
        _err("Can not find detector element width!")
    if self.det_elem_width <= 0:
        _err("DetectorElementWidth (DetectorElementSize) should be larger than 0!")
    self.positive_u_is_positive_y = -1
    if "DetectorOffcenter" in cfg:
        self.det_offset_horizontal = cfg["DetectorOffcenter"]
    elif "DetectorOffsetHorizontal" in cfg:
        self.det_offset_horizontal = cfg["DetectorOffsetHorizontal"]
    else:
        # the reference prints this warning and then fails on the unset attribute
        # (run_mgfbp.py:249-257); the default it announces is used here.
        _log(self, "Warning: Can not find horizontal detector offset; Using default value 0")
        self.det_offset_horizontal = 0.0
    if not isinstance(self.det_offset_horizontal, (float, int, list)):
        _err("DetectorOffsetHorizontal (DetectorOffcenter) should be a number!")
    if "DetectorElementCountVertical" in cfg:
        self.det_elem_count_vertical = cfg["DetectorElementCountVertical"]
    elif "SliceCount" in cfg:
        self.det_elem_count_vertical = cfg["SliceCount"]
    else:
        _err("Can not find detector element count along vertical direction!")
    if self.det_elem_count_vertical <= 0:
        _err("DetectorElementCountVertical (SliceCount) should be larger than 0!")
    elif self.det_elem_count_vertical % 1 != 0:
        _err("DetectorElementCountVertical (SliceCount) should be an integer!")
    self.det_elem_count_vertical = int(self.det_elem_count_vertical)
    if "DetectorElementVerticalReconRange" in cfg:
        rr = cfg["DetectorElementVerticalReconRange"]
        if not isinstance(rr, list) or len(rr) != 2:
            _err("DetectorElementVerticalReconRange should be an array with two numbers!")
        self.det_elem_vertical_recon_range_begin, self.det_elem_vertical_recon_range_end = rr
        if self.det_elem_vertical_recon_range_end > self.det_elem_count_vertical - 1 or \
                self.det_elem_vertical_recon_range_begin < 0:
            _err("Out of detector row range!")
        if rr[0] % 1 != 0 or rr[1] % 1 != 0:
            _err("DetectorElementVerticalReconRange must be integers!")
        self.det_elem_vertical_recon_range_begin = int(rr[0])
        self.det_elem_vertical_recon_range_end = int(rr[1])
        _log(self, f"--Reconstructing from detector row #{rr[0]:d} to #{rr[1]:d}")
        self.det_elem_count_vertical_actual = int(rr[1] - rr[0] + 1)
    else:
        self.det_elem_vertical_recon_range_begin = 0
        self.det_elem_vertical_recon_range_end = self.det_elem_count_vertical - 1
        self.det_elem_count_vertical_actual = self.det_elem_count_vertical
    if "DetectorElementVerticalGaussFilterSize" in cfg:
        self.det_elem_vertical_gauss_filter_size = cfg["DetectorElementVerticalGaussFilterSize"]
        if self.det_elem_vertical_gauss_filter_size <= 0:
            _err("DetectorElementVerticalGaussFilterSize should be larger than 0!")
        self.apply_gauss_vertical = True
    else:
        self.apply_gauss_vertical = False
        self.det_elem_vertical_gauss_filter_size = 0.0001
    # ---- rotation (:319-370)
    if "Views" not in cfg:
        _err("Can not find number of views!")
    self.view_num = cfg["Views"]
    if self.view_num % 1 != 0 or self.view_num < 0:
        _err("Views must be larger than 0 and must be an integer!")
    self.view_num = int(self.view_num)
    self.sgm_height = cfg.get("SinogramHeight", self.view_num)
    if self.sgm_height % 1 != 0 or self.sgm_height < 0:
        _err("SinogramHeight must be larger than 0 and must be an integer!")
    self.sgm_height = int(self.sgm_height)
    if "TotalScanAngle" in cfg:
        tsa = cfg["TotalScanAngle"]
        if isinstance(tsa, list):
            self.array_total_scan_angle = [a / 180.0 * PI for a in tsa]
            self.total_scan_angle = self.array_total_scan_angle[0]
        else:
            self.total_scan_angle = tsa / 180.0 * PI
    else:
        self.total_scan_angle = 2 * PI
    if not isinstance(self.total_scan_angle, (float, int, list)):
        _err("TotalScanAngle should be a number!")
    self.short_scan = 0 if abs(self.total_scan_angle % (2 * PI)) < (0.01 / 180 * PI) else 1
    # ---- beam hardening (:372-385)
    if "BeamHardeningCorrectionCoefficients" in cfg:
        c = cfg["BeamHardeningCorrectionCoefficients"]
        if not isinstance(c, list):
            _err("BeamHardeningCorrectionCoefficients must be an array!")
        self.bool_bh_correction = True
        self.bh_corr_order = len(c)
        self.array_bh_coefficients = np.array(c, dtype=np.float32)
    else:
        self.bool_bh_correction = False
    # ---- distances (:387-413)
    for key, attr in (("SourceIsocenterDistance", "source_isocenter_dis"),
                      ("SourceDetectorDistance", "source_det_dis")):
        if key in cfg:
            val = cfg[key]
            if not isinstance(val, (float, int)):
                _err(f"{key} must be a number!")
            if val <= 0.0:
                _err(f"{key} must be positive!")
            setattr(self, attr, val)
        else:
            setattr(self, attr, self.det_elem_count_horizontal * self.det_elem_width * 1000.0)
            _log(self, f"Warning: Did not find {key}; Set to infinity!")
    # ---- image (:416-470)
    if "ImageDimension" not in cfg:
        _err("can not find ImageDimension!")
    self.img_dim = cfg["ImageDimension"]
    if not isinstance(self.img_dim, int) or self.img_dim < 0:
        _err("ImageDimension must be a positive integer!")
    if "PixelSize" not in cfg:
        _err("can not find PixelSize!")
    self.img_pix_size = cfg["PixelSize"]
    if not isinstance(self.img_pix_size, (float, int)):
        _err("PixelSize must be a number!")
    if self.img_pix_size < 0:
        _err("PixelSize must be positive!")
    if "ImageRotation" in cfg:
        if not isinstance(cfg["ImageRotation"], (float, int)):
            _err("ImageRotation must be a number!")
        self.img_rot = cfg["ImageRotation"] / 180.0 * PI
    else:
        self.img_rot = 0.0
    if "ImageCenter" in cfg:
        ic = cfg["ImageCenter"]
        if not isinstance(ic, list) or len(ic) != 2:
            _err("ImageCenter must be an array with two numbers!")
        self.img_center = ic
        self.img_center_x, self.img_center_y = ic
    else:
        self.img_center_x = 0.0
        self.img_center_y = 0.0
    modes = {"axial": 1, "coronal": 2, "sagittal": 3}
    if "ReconViewMode" in cfg:
        if cfg["ReconViewMode"] not in modes:
            _err("ReconViewMode can only be axial, coronal or sagittal!")
        self.recon_view_mode = modes[cfg["ReconViewMode"]]
    else:
        self.recon_view_mode = 1
    # ---- reconstruction kernel (:472-505)
    if "HammingFilter" in cfg:
        self.kernel_name = "HammingFilter"
        self.kernel_param = cfg["HammingFilter"]
    elif "GaussianApodizedRamp" in cfg:
        self.kernel_name = "GaussianApodizedRamp"
        self.kernel_param = cfg["GaussianApodizedRamp"]
    elif "None" in cfg:
        self.kernel_name = "None"
        self.kernel_param = 0.0
    else:
        self.kernel_name = None  # the reference leaves it unset and fails when filtering
        self.kernel_param = 0.0
    if not isinstance(self.kernel_param, (float, int)):
        _err("Kernel parameter must be a number!")
    self.dbt_or_not = cfg.get("DBTMode", 0)
    # ---- HU (:507-516)
    if "WaterMu" in cfg:
        self.water_mu = cfg["WaterMu"]
        if not isinstance(self.water_mu, (float, int)):
            _err("WaterMu must be a number!")
        self.convert_to_HU = True
    else:
        self.convert_to_HU = False
    # ---- cone beam (:518-687)
    if "ConeBeam" in cfg:
        self.cone_beam = cfg["ConeBeam"]
        if not isinstance(self.cone_beam, bool):
            _err("ConeBeam must be true or false!")
    else:
        self.cone_beam = False
    self.bool_apply_pmatrix = False
    self.img_center_z_auto_set_from_fbp = False
    if self.cone_beam:
        if "SliceThickness" in cfg:
            self.det_elem_height = cfg["SliceThickness"]
        elif "DetectorElementHeight" in cfg:
            self.det_elem_height = cfg["DetectorElementHeight"]
        else:
            _err("Can not find detector element height for cone beam recon! ")
        if not isinstance(self.det_elem_height, (float, int)):
            _err("DetectorElementHeight (SliceThickness) must be a number!")
        if self.det_elem_height <= 0:
            _err("DetectorElementHeight (SliceThickness) must be positive!")
        if "ImageSliceCount" in cfg:
            self.img_dim_z = cfg["ImageSliceCount"]
        elif "ImageDimensionZ" in cfg:
            self.img_dim_z = cfg["ImageDimensionZ"]
        else:
            _err("Can not find image dimension along Z direction for cone beam recon!")
        if not isinstance(self.img_dim_z, int) or self.img_dim_z <= 0:
            _err("ImageDimensionZ (ImageSliceCount) must be a positive integer!")
        if "VoxelHeight" in cfg:
            self.img_voxel_height = cfg["VoxelHeight"]
        elif "ImageSliceThickness" in cfg:
            self.img_voxel_height = cfg["ImageSliceThickness"]
        else:
            _err("Can not find image voxel height for cone beam recon!")
        if not isinstance(self.img_voxel_height, (float, int)):
            _err("VoxelHeight (ImageSliceThickness) must be a number!")
        if self.img_voxel_height <= 0:
            _err("VoxelHeight (ImageSliceThickness) must be positive!")
        if "PMatrixFile" in cfg:
            from .pmatrix import apply_pmatrix_config
            apply_pmatrix_config(self, cfg)
        if not self.bool_apply_pmatrix:
            if "SliceOffCenter" in cfg:
                self.det_offset_vertical = cfg["SliceOffCenter"]
            elif "DetectorOffsetVertical" in cfg:
                self.det_offset_vertical = cfg["DetectorOffsetVertical"]
            else:
                self.det_offset_vertical = 0
                _log(self, "Warning: Can not find vertical detector offset for cone beam recon; Using default value 0")
            if not isinstance(self.det_offset_vertical, (float, int)):
                _err("DetectorOffsetVertical (SliceOffCenter) must be a number!")
        if "ImageCenterZ" in cfg:
            self.img_center_z = cfg["ImageCenterZ"]
            if not isinstance(self.img_center_z, (float, int)):
                _err("ImageCenterZ must be a number!")
        else:
            center_row = (self.det_elem_vertical_recon_range_end + self.det_elem_vertical_recon_range_begin) / 2
            dist = (center_row - (self.det_elem_count_vertical - 1) / 2) * self.det_elem_height
            if self.first_slice_top_row:
                dist = dist * (-1)
            self.img_center_z = (self.det_offset_vertical + dist) * self.source_isocenter_dis / self.source_det_dis
            self.img_center_z_auto_set_from_fbp = True
            cfg["ImageCenterZ"] = self.img_center_z
    else:
        self.det_elem_height = 0.0
        self.det_offset_vertical = 0.0
        self.img_dim_z = self.det_elem_count_vertical
        self.img_voxel_height = 0.0
        self.img_center_z = 0.0
    # ---- derived configuration dump (:690-719)
    if "SaveModifiedConfigFolder" in cfg:
        folder = cfg["SaveModifiedConfigFolder"]
        if not isinstance(folder, str):
            _err("SaveModifiedConfigFolder must be a string!")
        del cfg["SaveModifiedConfigFolder"]
        os.makedirs(folder, exist_ok=True)
        save_jsonc(folder + "/config_mgfbp.jsonc", cfg)
        if self.bool_apply_pmatrix:
            from .pmatrix import save_pmatrix_side_files
            save_pmatrix_side_files(self, folder)


def parse_fpj(self, cfg):
    """Mgfpj.__init__ extras, run_mgfpj_v2.py:113-214."""
    self.output_file_form = cfg.get("OutputFileForm", "sinogram")
    if self.output_file_form not in ("sinogram", "post_log_images"):
        _err("OutputFileForm can only be sinogram or post_log_images!")
    self.oversample_size = cfg.get("OversampleSize", 1)
    if not isinstance(self.oversample_size, (float, int)):
        _err("OversampleSize should be a number!")
    if self.oversample_size % 1 != 0 or self.oversample_size < 0:
        _err("OversampleSize must be a positive integer!")
    self.oversample_size = int(self.oversample_size)
    self.fpj_step_size = cfg.get("ForwardProjectionStepSize", 0.2)
    if "HelicalPitch" in cfg:
        self.helical_scan = True
        self.helical_pitch = cfg["HelicalPitch"]
    else:
        self.helical_scan = False
        self.helical_pitch = 0.0
    if self.helical_scan:
        if ("ImageCenterZ" not in cfg) or self.img_center_z_auto_set_from_fbp:
            self.img_center_z = self.img_voxel_height * (self.img_dim_z - 1) / 2.0 * np.sign(self.helical_pitch)
    if "PhotonNumber" in cfg:
        self.add_possion_noise = True
        self.photon_number = cfg["PhotonNumber"]
        if not isinstance(self.photon_number, (float, int)):
            _err("PhotonNumber must be a number!")
    else:
        self.add_possion_noise = False
        self.photon_number = 0
    if "StartAngle" in cfg:
        # the reference takes StartAngle as-is (no degree conversion), run_mgfpj_v2.py:181-186
        self.img_rot = cfg["StartAngle"]
        if not isinstance(self.img_rot, (float, int)):
            _err("StartAngle must be a number!")
    if self.bool_apply_pmatrix:
        from .pmatrix import matrix_a_from_pmatrix
        self.matrix_A_each_view, self.x_s_each_view = matrix_a_from_pmatrix(self.array_pmatrix, self.view_num)


def _read_value_file(path, name, n):
    d = load_jsonc(path)
    if "Value" not in d:
        _err(f"{name} has no member named 'Value'!")
    v = d["Value"]
    if not isinstance(v, list):
        _err(f"{name}.Value is not an array")
    if len(v) != n:
        _err(f"view number is {n:d} while {name} has {len(v):d} elements!")
    return v


def parse_fpj_v3(self, cfg):
    """Mgfpj_v3.__init__ extras (per-view angle / z-centre files), run_mgfpj_v3.py:129-172."""
    if "ScanAngleFile" in cfg:
        v = _read_value_file(cfg["ScanAngleFile"], "ScanAngleFile", self.view_num)
        # float32 arithmetic, as the reference's array (run_mgfpj_v3.py:142)
        self.array_angle = (np.array(v, dtype=np.float32) / np.float32(180.0) * np.float32(PI)
                            + np.float32(self.img_rot)).astype(np.float64)
        self.bool_uneven_scan_angle = True
    else:
        self.bool_uneven_scan_angle = False
    if "ImageCenterZFile" in cfg:
        v = _read_value_file(cfg["ImageCenterZFile"], "ImageCenterZFile", self.view_num)
        self.array_img_center_z = np.array(v, dtype=np.float32).astype(np.float64)
        self.bool_image_center_z_from_file = True
    else:
        self.array_img_center_z = np.ones(self.view_num, dtype=np.float64) * self.img_center_z
        self.bool_image_center_z_from_file = False


def parse_ir(self, cfg):
    """Mgfbp_ir.__init__ extras, run_mgfbp_iterative_recon_IRN_CGLS.py:57-136."""
    def get(key, default, check, msg, warn):
        if key in cfg:
            val = cfg[key]
            if not check(val):
                _err(msg)
            return val
        _log(self, warn)
        return default

    self.coef_lambda = get("Lambda", 1e-5, lambda x: _is_number(x) and x >= 0.0,
                           "Lambda must be a positive number!", "Warning: Did not find Lambda! Use default value 1e-5. ")
    self.beta_tv = get("BetaTV", 1e-6, lambda x: _is_number(x) and x >= 0.0,
                       "BetaTV must be a positive number!", "Warning: Did not find BetaTV! Use default value 1e-6. ")
    self.num_irn_iter = get("NumberOfIRNIterations", 15, lambda x: isinstance(x, int) and x >= 0,
                            "NumberOfIRNIterations must be a positive integer!",
                            "Warning: Did not find NumberOfIRNIterations! Use default value 15. ")
    self.num_iter = get("NumberOfIterations", 100, lambda x: isinstance(x, int) and x >= 0,
                        "NumberOfIterations must be a positive integer!",
                        "Warning: Did not find NumberOfIterations! Use default value 100. ")
    if "HelicalPitch" in cfg:
        self.helical_scan = True
        self.helical_pitch = cfg["HelicalPitch"]
    else:
        self.helical_scan = False
        self.helical_pitch = 0.0
    self.sgm_total_pixel_count = self.det_elem_count_vertical_actual * self.view_num * self.det_elem_count_horizontal
    self.img_total_pixel_count = self.img_dim_z * self.img_dim * self.img_dim
    self.pixel_count_ratio = float(self.sgm_total_pixel_count / self.img_total_pixel_count)
    # matched-adjoint CGLS instead of the reference's voxel-driven "P^T" (an addition)
    bp = cfg.get("BackProjector", "reference")
    if bp not in ("reference", "adjoint"):
        _err("BackProjector can only be reference or adjoint!")
    self.back_projector = bp
    # storage of the operator gathers (an addition): "float32" (default), "bfloat16" or
    # "float16" (16-bit volume cells in the FP, 16-bit packed sinogram in the
    # backprojector; all arithmetic, iterates and reductions stay float32 / float64)
    sp = cfg.get("StoragePrecision", "float32")
    if sp not in ("float32", "bfloat16", "float16"):
        _err("StoragePrecision can only be float32, bfloat16 or float16!")
    self.storage_precision = sp
    # storage of the measured sinogram in the data term P^T b (an addition): "float32"
    # (default; rounding b to bf16 adds errors of the size of the photon noise, which
    # the iterations fit), "float16" (fp16 with a power-of-two scale, 2^-11 relative)
    # or "bfloat16"
    dp = cfg.get("SinogramPrecision", "float32")
    if dp not in ("float32", "bfloat16", "float16"):
        _err("SinogramPrecision can only be float32, bfloat16 or float16!")
    self.sinogram_precision = dp
    # storage of the CG iterates x, r, d, q between kernels (an addition): "float32"
    # (default) or "bfloat16" (arithmetic in float32, reductions in float64, stored
    # values rounded; cone beam with the reference backprojector in the axial view mode)
    ip = cfg.get("IterateStorage", "float32")
    if ip not in ("float32", "bfloat16"):
        _err("IterateStorage can only be float32 or bfloat16!")
    self.iterate_storage = ip


def parse_piccs(self, cfg):
    """Mgfbp_ir_piccs.__init__ extras, run_mgfbp_iterative_recon_IRN_CGLS_piccs.py:55-67."""
    if "Alpha" in cfg:
        self.coef_alpha = cfg["Alpha"]
        if not _is_number(self.coef_alpha) or self.coef_alpha < 0.0:
            _err("Alpha must be a positive number!")
    else:
        self.coef_alpha = 1e-5
        _log(self, "Warning: Did not find Alpha! Use default value 1e-5. ")
    if "PriorImageFile" not in cfg:
        _err("Can not find PriorImageFile in the config file!")
    self.prior_image_file = cfg["PriorImageFile"]


def parse_fpj_v1(self, cfg):
    """Stand-alone parameter handling of the original projector Mgfpj
    (run_mgfpj.py:98-450): its own aliases (DetectorElementCount,
    DetectorZElementCount, DetectorZOffcenter, SliceCount for the image depth) and
    StartAngle / ImageRotation in degrees."""
    self.config_dict = cfg
    for key, attr in (("InputDir", "input_dir"), ("OutputDir", "output_dir"), ("InputFiles", "input_files_pattern")):
        if key not in cfg:
            _err(f"Can not find {key}!")
        if not isinstance(cfg[key], str):
            _err(f"{key} must be a string!")
        setattr(self, attr, cfg[key])
    self.output_file_prefix = cfg.get("OutputFilePrefix", "")
    if not isinstance(self.output_file_prefix, str):
        _err("OutputFilePrefix must be a string!")
    if "OutputFileReplace" not in cfg:
        _err("Can not find OutputFileReplace in the config file!")
    self.output_file_replace = cfg["OutputFileReplace"]
    os.makedirs(self.output_dir, exist_ok=True)
    self.output_file_form = cfg.get("OutputFileForm", "sinogram")
    if self.output_file_form not in ("sinogram", "post_log_images"):
        _err("OutputFileForm can only be sinogram or post_log_images!")
    if "ImageDimension" not in cfg:
        _err("can not find ImageDimension!")
    self.img_dim = cfg["ImageDimension"]
    if not isinstance(self.img_dim, int) or self.img_dim < 0:
        _err("ImageDimension must be a positive integer!")
    if "PixelSize" not in cfg:
        _err("can not find PixelSize!")
    self.img_pix_size = cfg["PixelSize"]
    if "SliceCount" in cfg:
        self.img_dim_z = cfg["SliceCount"]
    elif "ImageDimensionZ" in cfg:
        self.img_dim_z = cfg["ImageDimensionZ"]
    else:
        _err("Can not find image dimension along Z direction (ImageDimensionZ or SliceCount)!")
    if not isinstance(self.img_dim_z, int) or self.img_dim_z <= 0:
        _err("ImageDimensionZ (ImageSliceCount) must be a positive integer!")
    self.img_center_x, self.img_center_y = cfg.get("ImageCenter", [0.0, 0.0])
    self.img_center_z = cfg.get("ImageCenterZ", 0.0)
    self.cone_beam = cfg.get("ConeBeam", False)
    if not isinstance(self.cone_beam, bool):
        _err("ConeBeam must be true or false!")
    self.curved_dect = cfg.get("CurvedDetector", False)
    if not isinstance(self.curved_dect, bool):
        _err("CurvedDetector can only be true or false!")
    for k in ("DetectorElementCountHorizontal", "SinogramWidth", "DetectorElementCount"):
        if k in cfg:
            self.det_elem_count_horizontal = cfg[k]
            break
    else:
        _err("Can not find DetectorElementCountHorizontal (SinogramWidth or DetectorElementCount)!")
    if self.det_elem_count_horizontal <= 0 or self.det_elem_count_horizontal % 1 != 0:
        _err("DetectorElementCountHorizontal (SinogramWidth) should be a positive integer!")
    self.det_elem_count_horizontal = int(self.det_elem_count_horizontal)
    if "DetectorElementWidth" in cfg:
        self.det_elem_width = cfg["DetectorElementWidth"]
    elif "DetectorElementSize" in cfg:
        self.det_elem_width = cfg["DetectorElementSize"]
    else:
        _err("Can not find DetectorElementWidth (DetectorElementSize)!")
    self.det_offset_horizontal = cfg.get("DetectorOffcenter", cfg.get("DetectorOffsetHorizontal", 0.0))
    for key, attr in (("SourceIsocenterDistance", "source_isocenter_dis"),
                      ("SourceDetectorDistance", "source_det_dis")):
        setattr(self, attr, cfg.get(key, self.det_elem_count_horizontal * self.det_elem_width * 1000.0))
    if "StartAngle" in cfg:
        self.start_angle = cfg["StartAngle"] / 180.0 * PI
    elif "ImageRotation" in cfg:
        self.start_angle = cfg["ImageRotation"] / 180.0 * PI
    else:
        self.start_angle = 0.0
    self.scan_angle = cfg["TotalScanAngle"] / 180.0 * PI if "TotalScanAngle" in cfg else 2 * PI
    if "Views" not in cfg:
        _err("Can not find number of views!")
    self.view_num = int(cfg["Views"])
    self.oversample_size = int(cfg.get("OversampleSize", 1))
    self.fpj_step_size = cfg.get("ForwardProjectionStepSize", 0.2)
    if self.cone_beam:
        self.img_voxel_height = cfg.get("VoxelHeight", cfg.get("ImageSliceThickness"))
        if self.img_voxel_height is None:
            _err("Can not find image voxel height for cone beam recon!")
        nv = cfg.get("DetectorElementCountVertical", cfg.get("DetectorZElementCount"))
        if nv is None:
            _err("Can not find detector element count along vertical direction!")
        self.det_elem_count_vertical = int(nv)
        self.det_elem_height = cfg.get("SliceThickness", cfg.get("DetectorElementHeight"))
        if self.det_elem_height is None:
            _err("Can not find detector element height for cone beam recon! ")
        self.det_offset_vertical = cfg.get("DetectorZOffcenter", cfg.get("DetectorOffsetVertical", 0.0))
    else:
        self.det_elem_count_vertical = self.img_dim_z
        self.img_voxel_height = 0.0
        self.det_elem_height = 0.0
        self.det_offset_vertical = 0.0
    if "WaterMu" in cfg:
        self.water_mu = cfg["WaterMu"]
        self.convert_to_HU = True
    else:
        self.convert_to_HU = False
    self.helical_scan = "HelicalPitch" in cfg
    self.helical_pitch = cfg.get("HelicalPitch", 0)
    if self.helical_scan and "ImageCenterZ" not in cfg:
        self.img_center_z = self.img_voxel_height * (self.img_dim_z - 1) / 2.0 * np.sign(self.helical_pitch)
    self.add_possion_noise = "PhotonNumber" in cfg
    self.photon_number = cfg.get("PhotonNumber", 0)
    # fields shared with the Mgfbp-derived projectors
    self.det_elem_count_vertical_actual = self.det_elem_count_vertical
    self.det_elem_vertical_recon_range_begin = 0
    self.img_rot = self.start_angle
    self.total_scan_angle = self.scan_angle
    self.recon_view_mode = 1
    self.short_scan = 0
    self.bool_apply_pmatrix = False
