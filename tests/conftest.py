import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


_SIDE_DIR = []


def _side_dir():
    if not _SIDE_DIR:
        import atexit
        import shutil
        import tempfile
        d = tempfile.mkdtemp(prefix="mct_side_")
        atexit.register(shutil.rmtree, d, True)
        _SIDE_DIR.append(d)
    return _SIDE_DIR[0]


def load_golden(name):
    """A fixture's arrays and its config; per-view side files the reference read
    (ScanAngleFile, ImageCenterZFile) are written out again and the config points at
    them."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    out = {k: z[k] for k in z.files}
    out["config"] = json.loads(str(z["config"]))
    for key, cfg_key in (("side_scan_angles", "ScanAngleFile"), ("side_center_z", "ImageCenterZFile")):
        if key in out:
            path = os.path.join(_side_dir(), f"{name}_{cfg_key}.jsonc")
            with open(path, "w") as f:
                json.dump({"Value": [float(v) for v in out[key]]}, f)
            out["config"][cfg_key] = path
    return out


def golden_names(prefix, exclude=()):
    return sorted(f[:-4] for f in os.listdir(GOLDEN)
                  if f.endswith(".npz") and f.startswith(prefix) and not f.startswith(tuple(exclude)))


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from reconstruction_program_taichi_gb300 import _lib
    _lib.load()  # a GPU run without the native library is a failure, not a skip
    return torch.device("cuda")
