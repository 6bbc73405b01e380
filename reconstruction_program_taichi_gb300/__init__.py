"""MandoCT reconstruction hot path on one NVIDIA GB300 (sm_103a).

Drop-in Python API of the reference (MandoCT-Taichi): the jsonc-driven entry points
run_mgfbp / run_mgfpj_v3 / run_mgfbp_ir / run_mgfbp_ir_piccs and the classes Mgfbp,
Mgfpj_v3, Mgfbp_ir, Mgfbp_ir_piccs.  All compute runs in libmandoct_gb300.so
(hand-written CUDA, C ABI in include/mandoct_gb300.h); torch provides device memory
and streams.  There is no CPU fallback.
"""
from ._lib import NativeLibraryError, launch_count
from .config import ConfigError, ReadConfigFile, load_jsonc, remove_comments, save_jsonc
from .fbp import FdkPipeline, Mgfbp, Mgfbp_v2, run_mgfbp, run_mgfbp_v2
from .helical import Mgfbp_helical, run_mgfbp_helical
from .fpj import FpPipeline, Mgfpj_v3, run_mgfpj_v3
from .ir import IrSystem, Mgfbp_ir, Mgfbp_ir_piccs, run_mgfbp_ir, run_mgfbp_ir_piccs
from .admm import Mgfbp_ir_admm, run_mgfbp_ir_admm
from .stream import ScanStream

__all__ = [
    "ConfigError", "NativeLibraryError", "ReadConfigFile", "load_jsonc", "remove_comments", "save_jsonc",
    "FdkPipeline", "Mgfbp", "run_mgfbp", "Mgfbp_v2", "run_mgfbp_v2", "Mgfbp_helical", "run_mgfbp_helical", "FpPipeline", "Mgfpj_v3", "run_mgfpj_v3",
    "IrSystem", "Mgfbp_ir", "Mgfbp_ir_piccs", "run_mgfbp_ir", "run_mgfbp_ir_piccs", "Mgfbp_ir_admm",
    "run_mgfbp_ir_admm", "ScanStream", "launch_count",
]
