"""Serving engine host logic without a GPU: admission waits for file inputs, a failed
read fails only its request, results are written to out_path before their futures
resolve, and every request gets its own result.  The CUDA slots are replaced by a
fake whose 'reconstruction' is a function of the input, so only the scheduler runs."""
import threading
import time

import numpy as np
import pytest
import torch

from reconstruction_program_taichi_gb300 import serve


class _Obj:
    """The geometry fields the scheduler reads (slot class key, memory estimate)."""

    def __init__(self, n=8, views=6, nu=10, nv=4):
        self.det_elem_count_horizontal, self.det_elem_count_vertical_actual = nu, nv
        self.det_elem_count_vertical, self.view_num, self.sgm_height = nv, views, views
        self.img_dim, self.img_dim_z = n, 3
        self.det_elem_width = self.det_elem_height = 1.0
        self.img_pix_size = self.img_voxel_height = 1.0
        self.source_isocenter_dis, self.source_det_dis = 300.0, 600.0
        self.total_scan_angle, self.img_rot = 6.2832, 0.0
        self.cone_beam, self.curved_dect = True, False
        self.kernel_name, self.kernel_param = "HammingFilter", 1.0
        self.det_offset_horizontal = self.det_offset_vertical = 0.0
        self.img_center_x = self.img_center_y = self.img_center_z = 0.0
        self.recon_view_mode = 1
        self.input_file_form = "sinogram"
        self.det_elem_vertical_recon_range_begin, self.det_elem_vertical_recon_range_end = 0, nv - 1


class _FakeSlot:
    batch = 2
    nbytes = 1000
    runs = []

    def __init__(self, obj):
        self.obj = obj
        self.last_used = time.perf_counter()

    def run(self, reqs, done=None):
        _FakeSlot.runs.append(len(reqs))
        outs = []
        for i, r in enumerate(reqs):
            time.sleep(0.01)
            outs.append(np.asarray(r.sgm, np.float64).sum(axis=(0, 1)))
            if done is not None and i + 1 < len(reqs):
                done(i, outs[-1])
        return outs


@pytest.fixture
def server(monkeypatch):
    monkeypatch.setattr(torch.cuda, "is_available", lambda: True)
    monkeypatch.setattr(torch.cuda, "set_device", lambda d: None)
    monkeypatch.setattr(serve.ReconServer, "_make_slot", lambda self, req: _FakeSlot(req.obj))
    _FakeSlot.runs = []
    srv = serve.ReconServer(device="cuda:0", hbm_budget_gb=1.0, batch=2)
    yield srv
    srv.close()


def test_file_inputs_are_read_and_results_written(server, tmp_path):
    o = _Obj()
    rng = np.random.default_rng(3)
    scans = [rng.uniform(0, 1, (4, 6, 10)).astype(np.float32) for _ in range(5)]
    futs = []
    for i, s in enumerate(scans):
        if i % 2:
            futs.append(server.submit_fbp(o, s))
        else:
            s.tofile(tmp_path / f"s{i}.raw")
            futs.append(server.submit_fbp(o, str(tmp_path / f"s{i}.raw"), out_path=tmp_path / f"r{i}.raw"))
    for i, (f, s) in enumerate(zip(futs, scans)):
        got = f.result(timeout=30)
        want = s.astype(np.float64).sum(axis=(0, 1))
        assert np.allclose(got, want), i
        if i % 2 == 0:  # the file exists once the future has resolved
            assert np.allclose(np.fromfile(tmp_path / f"r{i}.raw", dtype=np.float32), want)
    assert sum(_FakeSlot.runs) == 5 and max(_FakeSlot.runs) <= 2


def test_a_missing_file_fails_only_its_request(server, tmp_path):
    o = _Obj()
    good = np.ones((4, 6, 10), np.float32)
    bad = server.submit_fbp(o, tmp_path / "missing.raw")
    ok = server.submit_fbp(o, good)
    with pytest.raises(FileNotFoundError):
        bad.result(timeout=30)
    assert np.allclose(ok.result(timeout=30), 24.0)


def test_admission_waits_for_a_slow_read(server, tmp_path, monkeypatch):
    """A request whose file is still being read is not started; later ready requests
    of the same class go ahead, and the slow one runs once its data is in memory."""
    o = _Obj()
    gate = threading.Event()
    real = serve.read_sinogram_file

    def slow_read(obj, path):
        gate.wait(10)
        return real(obj, path)

    monkeypatch.setattr(serve, "read_sinogram_file", slow_read)
    s = np.full((4, 6, 10), 2.0, np.float32)
    s.tofile(tmp_path / "slow.raw")
    slow = server.submit_fbp(o, tmp_path / "slow.raw")
    fast = server.submit_fbp(o, np.ones((4, 6, 10), np.float32))
    assert np.allclose(fast.result(timeout=30), 24.0)
    assert not slow.done()
    gate.set()
    assert np.allclose(slow.result(timeout=30), 48.0)


def _parsed(**kw):
    from reconstruction_program_taichi_gb300 import config

    class O:
        verbose = False

    cfg = {"InputDir": "/tmp/a", "OutputDir": "/tmp/b", "InputFiles": "sgm_.*", "OutputFilePrefix": "",
           "OutputFileReplace": ["sgm", "rec"], "DetectorElementCountHorizontal": 64, "DetectorElementWidth": 0.8,
           "DetectorOffsetHorizontal": 0.0, "DetectorElementCountVertical": 16, "DetectorElementHeight": 0.8,
           "Views": 90, "TotalScanAngle": 360, "SourceIsocenterDistance": 300, "SourceDetectorDistance": 550,
           "ImageDimension": 32, "PixelSize": 0.5, "ImageDimensionZ": 8, "VoxelHeight": 0.5, "ConeBeam": True,
           "HammingFilter": 1, "ForwardProjectionStepSize": 0.3, "Lambda": 1e-3}
    cfg.update(kw)
    cfg = {k: v for k, v in cfg.items() if v is not None}  # None removes a key
    o = O()
    config.parse_fbp(o, cfg)
    config.parse_fpj(o, cfg)
    config.parse_fpj_v3(o, cfg)
    config.parse_ir(o, cfg)
    return o


@pytest.mark.parametrize("kw", [
    {"TotalScanAngle": 220},                                   # short scan (Parker weights)
    {"Lambda": 2e-3},                                          # CGLS regularisation
    {"BeamHardeningCorrectionCoefficients": [0.0, 1.0, 0.1]},  # BH polynomial
    {"ImageRotation": 1.0},
    {"HammingFilter": 0.5},
    {"DetectorOffsetVertical": 0.2},
    {"CurvedDetector": True},
    {"ForwardProjectionStepSize": 0.2},
    {"ImageCenterZ": 0.3},
    {"DetectorElementVerticalGaussFilterSize": 1.5},
    {"GaussianApodizedRamp": 1.2, "HammingFilter": None},
])
def test_slot_key_separates_configs_that_change_the_result(kw):
    """Requests are batched on one slot (whose pipeline is built from the first
    request's config) only when their parsed configs agree in everything that can
    change the result."""
    base, other = _parsed(), _parsed(**kw)
    for kind in ("fbp", "cgls"):
        a = serve._Request(kind, base, None, n_iter=3)
        b = serve._Request(kind, other, None, n_iter=3)
        assert a.key != b.key, kw


def test_slot_key_ignores_file_names():
    a = _parsed()
    b = _parsed(InputDir="/elsewhere", OutputDir="/out2", InputFiles="scan_.*", OutputFilePrefix="p_",
                OutputFileReplace=["scan", "img"])
    assert serve._Request("fbp", a, None).key == serve._Request("fbp", b, None).key
    assert serve._Request("fbp", a, None).key != serve._Request("fbp", a, None, storage="bf16").key
    assert serve._Request("cgls", a, None, n_iter=3).key != serve._Request("cgls", a, None, n_iter=4).key


def test_slot_construction_does_not_block_other_batches(monkeypatch):
    """A new slot is built by its batch's worker outside the scheduler's lock: while
    one class's slot is still being built, requests of a class with a free slot run
    and their futures resolve."""
    monkeypatch.setattr(torch.cuda, "is_available", lambda: True)
    monkeypatch.setattr(torch.cuda, "set_device", lambda d: None)
    gate = threading.Event()
    slow_obj = _Obj(n=9)

    def make(self, req):
        if req.obj is slow_obj:
            assert gate.wait(20)
        return _FakeSlot(req.obj)

    monkeypatch.setattr(serve.ReconServer, "_make_slot", make)
    _FakeSlot.runs = []
    srv = serve.ReconServer(device="cuda:0", hbm_budget_gb=1.0, batch=2)
    try:
        o = _Obj()
        assert np.allclose(srv.submit_fbp(o, np.ones((4, 6, 10), np.float32)).result(timeout=30), 24.0)
        slow = srv.submit_fbp(slow_obj, np.ones((4, 6, 10), np.float32))
        time.sleep(0.1)  # the slow class's worker is now inside the slot construction
        fast = srv.submit_fbp(o, np.full((4, 6, 10), 3.0, np.float32))
        assert np.allclose(fast.result(timeout=10), 72.0)
        assert not slow.done()
        gate.set()
        assert np.allclose(slow.result(timeout=30), 24.0)
        assert srv.stats()["slots"]["fbp"] == 2
    finally:
        gate.set()
        srv.close()


def test_failed_slot_construction_releases_its_reservation(monkeypatch):
    monkeypatch.setattr(torch.cuda, "is_available", lambda: True)
    monkeypatch.setattr(torch.cuda, "set_device", lambda d: None)

    def make(self, req):
        raise RuntimeError("out of device memory")

    monkeypatch.setattr(serve.ReconServer, "_make_slot", make)
    srv = serve.ReconServer(device="cuda:0", hbm_budget_gb=1.0, batch=2)
    try:
        f = srv.submit_fbp(_Obj(), np.ones((4, 6, 10), np.float32))
        with pytest.raises(RuntimeError, match="out of device memory"):
            f.result(timeout=30)
        time.sleep(0.05)
        assert srv.used == 0 and srv.all_slots == {}
    finally:
        srv.close()
