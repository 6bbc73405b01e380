"""run_over_files: the drivers' per-file loop with the next read and the previous
write overlapped with the compute (no GPU: a fake driver records what ran where)."""
import threading
import time

import numpy as np
import pytest

from reconstruction_program_taichi_gb300.file_pipeline import run_over_files


class FakeDriver:
    """Mimics Mgfbp: read sets per-file attributes, save converts the result in place."""

    def __init__(self, fail_read=None, fail_save=None, skip=()):
        self.log = []
        self.lock = threading.Lock()
        self.fail_read, self.fail_save, self.skip = fail_read, fail_save, set(skip)
        self.count = 0
        self.img = None
        self.saved = {}

    def note(self, what):
        with self.lock:
            self.log.append((what, time.perf_counter(), threading.current_thread().name))

    def read(self, file):
        self.note(("read", file))
        time.sleep(0.05)
        if file == self.fail_read:
            raise IOError("cannot read " + file)
        if file in self.skip:
            return False
        self.path = file
        self.data = np.full(3, float(file[1:]))
        return True

    def compute(self):
        self.note(("compute", self.path))
        time.sleep(0.05)
        self.count += 1
        self.img = self.data * 2

    def save(self):
        self.note(("save", self.path))
        if self.path == self.fail_save:
            raise IOError("cannot write " + self.path)
        self.img = self.img + 1000  # rebinds the result at once, as SaveReconImg's HU
        time.sleep(0.05)
        with self.lock:
            self.saved[self.path] = self.img


def _run(d, files):
    return run_over_files(d, files, lambda x, f: x.read(f), lambda x: x.compute(), lambda x: x.save())


def test_results_and_final_state_match_the_sequential_loop():
    files = ["f1", "f2", "f3", "f4"]
    d = FakeDriver()
    assert _run(d, files) == 4
    seq = FakeDriver()
    for f in files:
        if seq.read(f):
            seq.compute()
            seq.save()
    assert d.saved.keys() == seq.saved.keys()
    for f in files:
        assert np.array_equal(d.saved[f], seq.saved[f])
    # the driver ends as the sequential loop leaves it: last file's paths, converted result
    assert d.path == seq.path == "f4" and d.count == seq.count == 4
    assert np.array_equal(d.img, seq.img)


class _RunAtSubmit:
    """Executor whose tasks run inside submit(): the earliest a stage thread could run."""

    def __init__(self, *a, **k):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def submit(self, fn, *args):
        from concurrent.futures import Future
        f = Future()
        try:
            f.set_result(fn(*args))
        except BaseException as e:  # noqa: BLE001 - handed to the caller through the future
            f.set_exception(e)
        return f


def test_final_state_holds_when_a_stage_runs_at_once(monkeypatch):
    """A save that runs before run_over_files takes its next step must still have its
    result (converted in place) moved back to the driver."""
    from reconstruction_program_taichi_gb300 import file_pipeline
    monkeypatch.setattr(file_pipeline, "ThreadPoolExecutor", _RunAtSubmit)
    d = FakeDriver()
    _run(d, ["f1", "f2"])
    assert np.array_equal(d.img, np.full(3, 2.0 * 2 + 1000))
    assert d.saved["f2"] is d.img


def test_reads_and_saves_overlap_the_compute_and_keep_order():
    d = FakeDriver()
    _run(d, ["f1", "f2", "f3"])
    ev = {w: (t, th) for w, t, th in d.log}
    order = [w for w, _, _ in d.log if w[0] == "compute"]
    assert order == [("compute", "f1"), ("compute", "f2"), ("compute", "f3")]
    assert [w for w, _, _ in d.log if w[0] == "save"] == [("save", "f1"), ("save", "f2"), ("save", "f3")]
    # the read of f2 starts before the compute of f1 ends, the save of f1 before the compute of f2 ends
    assert ev[("read", "f2")][0] < ev[("compute", "f1")][0] + 0.05
    assert ev[("save", "f1")][0] < ev[("compute", "f2")][0] + 0.05
    assert ev[("read", "f2")][1].startswith("mct-read") and ev[("save", "f1")][1].startswith("mct-write")
    assert ev[("compute", "f2")][1] == threading.current_thread().name


def test_skipped_files_are_not_computed():
    d = FakeDriver(skip=["f2"])
    assert _run(d, ["f1", "f2", "f3"]) == 2
    assert set(d.saved) == {"f1", "f3"} and d.count == 2


def test_a_failed_read_stops_after_the_previous_file_is_saved():
    d = FakeDriver(fail_read="f3")
    with pytest.raises(IOError, match="cannot read f3"):
        _run(d, ["f1", "f2", "f3", "f4"])
    assert set(d.saved) == {"f1", "f2"}
    assert ("compute", "f4") not in [w for w, _, _ in d.log]


def test_a_failed_save_is_raised():
    d = FakeDriver(fail_save="f2")
    with pytest.raises(IOError, match="cannot write f2"):
        _run(d, ["f1", "f2", "f3", "f4"])
    assert "f1" in d.saved and "f2" not in d.saved
    assert ("save", "f4") not in [w for w, _, _ in d.log]


def test_no_files():
    d = FakeDriver()
    assert _run(d, []) == 0 and d.img is None


# ---------------------------------------------------------------- the drivers' loops on CPU


class _FakeFdk:
    """Stands in for FdkPipeline: a deterministic function of each file's data."""
    device = "cpu"

    def filter(self, sgm, row_stride=None, view_stride=None):
        return sgm * 2.0

    def backproject(self, filtered, out=None):
        import torch
        z = float(filtered.double().sum())
        return torch.arange(8 * 12 * 12, dtype=torch.float32).reshape(8, 12, 12) * 1e-3 + z


class _FakeFp:
    class dg:
        device = "cpu"

    def project(self, vol, seed=0):
        import torch
        return torch.full((12, 12, 24), float(vol.double().sum()) + seed, dtype=torch.float32)


def _folder(tmp_path, golden, prefix, arrays, **extra):
    import json
    from conftest import load_golden
    z = load_golden(golden)
    d_in, d_out = tmp_path / "in", tmp_path / "out"
    d_in.mkdir()
    for tag, a in arrays(z).items():
        a.astype(np.float32).tofile(d_in / f"{prefix}_{tag}.raw")
    return dict(z["config"], InputDir=str(d_in), OutputDir=str(d_out), **extra), d_in, d_out


def test_mgfbp_file_loop_on_cpu(tmp_path):
    """Mgfbp.MainFunction over four files with the pipeline replaced by a CPU stand-in:
    each output is the stand-in's result for that file in HU, and the returned array is
    the last listed file's output (what the sequential loop returns)."""
    import os
    from reconstruction_program_taichi_gb300.fbp import Mgfbp
    scales = {"a": 1.0, "b": 0.5, "c": 2.0, "d": 1.5}
    cfg, d_in, d_out = _folder(tmp_path, "fdk_cone", "sgm", lambda z: {t: z["input_sgm"] * s
                                                                     for t, s in scales.items()}, WaterMu=0.02)
    drv = Mgfbp(cfg, verbose=False)
    drv._pipe = _FakeFdk()
    ret = drv.MainFunction()
    assert drv.file_processed_count == 4
    listed = [f for f in os.listdir(d_in) if f.startswith("sgm_")]
    for f in listed:
        one = Mgfbp(dict(cfg), verbose=False)
        one._pipe = _FakeFdk()
        one.ReadSinogram(f)
        import torch
        vol = one._pipe.backproject(one._pipe.filter(torch.from_numpy(one._raw)))
        want = (vol.numpy() / 0.02 - 1) * 1000
        got = np.fromfile(d_out / f.replace("sgm", "rec"), dtype=np.float32).reshape(want.shape)
        assert np.array_equal(got, want.astype(np.float32)), f
    last = np.fromfile(d_out / listed[-1].replace("sgm", "rec"), dtype=np.float32)
    assert np.array_equal(ret.ravel(), last)
    assert drv.output_path.endswith(listed[-1].replace("sgm", "rec"))


def test_mgfpj_v3_file_loop_on_cpu(tmp_path):
    import os
    from reconstruction_program_taichi_gb300.fpj import Mgfpj_v3
    scales = {"a": 1.0, "b": 0.25, "c": 3.0}
    cfg, d_in, d_out = _folder(tmp_path, "fpj_cone", "img", lambda z: {t: z["input_vol"] * s
                                                                     for t, s in scales.items()})
    drv = Mgfpj_v3(cfg, verbose=False)
    drv._pipe = _FakeFp()
    ret = drv.MainFunction()
    listed = [f for f in os.listdir(d_in) if f.startswith("img_")]
    assert drv.file_processed_count == 3
    for i, f in enumerate(listed):
        vol = np.fromfile(d_in / f, dtype=np.float32)
        want = np.full((12, 12, 24), np.float32(float(vol.astype(np.float64).sum()) + i + 1), dtype=np.float32)
        got = np.fromfile(d_out / f.replace("img", "sgm"), dtype=np.float32)
        assert np.array_equal(got, want[::-1].ravel()), f  # cone beam "sinogram" form: rows flipped
    assert np.array_equal(ret.ravel(), np.fromfile(d_out / listed[-1].replace("img", "sgm"), dtype=np.float32))
