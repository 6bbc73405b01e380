"""Serving loop: results are the same alone and in a concurrent mix; batching and
graphs are used; requests beyond the HBM budget are refused."""
import numpy as np
import pytest

from test_gpu_parity import _cone_obj

pytestmark = pytest.mark.gpu


def _cgls_obj(**kw):
    from reconstruction_program_taichi_gb300 import config
    o = _cone_obj(**kw)
    config.parse_ir(o, {"Lambda": 1e-3})
    return o


def test_same_result_alone_and_in_mix(cuda):
    from reconstruction_program_taichi_gb300.serve import ReconServer
    rng = np.random.default_rng(21)
    objs = [_cone_obj(n=40, nz=16, nu=72, nv=24, views=60), _cone_obj(n=32, nz=8, nu=64, nv=16, views=45)]
    cg = _cgls_obj(n=24, nz=8, nu=48, nv=12, views=30, DetectorElementHeight=1.0)
    reqs = []
    for i in range(10):
        o = objs[i % 2]
        reqs.append(("fbp", o, rng.uniform(0, 1, (o.det_elem_count_vertical, o.view_num,
                                                 o.det_elem_count_horizontal)).astype(np.float32)))
    sgm_cg = rng.uniform(0, 0.5, (12, 30, 48)).astype(np.float32)
    x0 = np.zeros((8, 24, 24), np.float32)

    alone = []
    srv = ReconServer(batch=1, max_slots_per_class=1)
    for kind, o, s in reqs:
        alone.append(srv.submit_fbp(o, s).result(timeout=120))
    cg_alone = srv.submit_cgls(cg, sgm_cg, x0, 3).result(timeout=120)
    srv.close()

    srv = ReconServer(batch=4, max_slots_per_class=2)
    futs = [srv.submit_fbp(o, s) for kind, o, s in reqs[:5]]
    fut_cg = srv.submit_cgls(cg, sgm_cg, x0, 3)
    futs += [srv.submit_fbp(o, s) for kind, o, s in reqs[5:]]
    mixed = [f.result(timeout=120) for f in futs]
    cg_mixed = fut_cg.result(timeout=120)
    st = srv.stats()
    srv.close()
    for a, b in zip(alone, mixed):
        assert np.array_equal(a, b)
    # CGLS uses float64 device reductions with a fixed order: identical too
    assert np.allclose(cg_alone, cg_mixed, rtol=1e-6, atol=1e-7)
    assert st["requests"] == 11 and st["p99_ms"] >= st["p50_ms"] > 0


def test_request_beyond_budget_is_refused(cuda):
    from reconstruction_program_taichi_gb300.serve import ReconServer
    o = _cone_obj(n=40, nz=16, nu=72, nv=24, views=60)
    srv = ReconServer(hbm_budget_gb=0.001, batch=1)
    f = srv.submit_fbp(o, np.zeros((24, 60, 72), np.float32))
    with pytest.raises(MemoryError):
        f.result(timeout=60)
    srv.close()


def test_device_resident_requests_match_host_requests(cuda):
    import torch
    from reconstruction_program_taichi_gb300.serve import ReconServer
    rng = np.random.default_rng(22)
    o = _cone_obj(n=40, nz=16, nu=72, nv=24, views=60)
    s = rng.uniform(0, 1, (24, 60, 72)).astype(np.float32)
    srv = ReconServer(batch=2, max_slots_per_class=1)
    host = srv.submit_fbp(o, s).result(timeout=120)
    dev = srv.submit_fbp(o, torch.from_numpy(s).cuda()).result(timeout=120)
    srv.close()
    assert isinstance(dev, torch.Tensor) and dev.is_cuda
    assert np.array_equal(host, dev.cpu().numpy())


def test_idle_slots_are_evicted_under_budget_pressure(cuda):
    from reconstruction_program_taichi_gb300.serve import ReconServer, _Request
    rng = np.random.default_rng(23)
    objs = [_cone_obj(n=40, nz=16, nu=72, nv=24, views=60), _cone_obj(n=32, nz=8, nu=64, nv=16, views=45)]
    sg = [rng.uniform(0, 1, (o.det_elem_count_vertical, o.view_num, o.det_elem_count_horizontal)).astype(np.float32)
          for o in objs]
    ref = []
    srv = ReconServer(batch=1, max_slots_per_class=1)
    for o, s in zip(objs, sg):
        ref.append(srv.submit_fbp(o, s).result(timeout=120))
    need = max(srv._estimate(_Request("fbp", o, s)) for o, s in zip(objs, sg))
    srv.close()
    # a budget that holds one slot at a time (the two slots together exceed it):
    # alternating classes must evict
    srv = ReconServer(hbm_budget_gb=need * 1.2 / 1e9, batch=1, max_slots_per_class=1)
    outs = [srv.submit_fbp(objs[i % 2], sg[i % 2]).result(timeout=120) for i in range(4)]
    st = srv.stats()
    srv.close()
    assert st["evictions"] >= 3
    for i, out in enumerate(outs):
        assert np.array_equal(out, ref[i % 2])


def test_file_inputs_and_outputs(tmp_path, cuda):
    """Paths as inputs (read on the server's I/O threads, admitted once in memory) and
    out_path (written after the slot is released): same results as array inputs; a
    missing input file fails its own request only."""
    from reconstruction_program_taichi_gb300.serve import ReconServer
    rng = np.random.default_rng(5)
    o = _cone_obj(n=40, nz=16, nu=72, nv=24, views=60)
    cg = _cgls_obj(n=24, nz=8, nu=48, nv=12, views=30, DetectorElementHeight=1.0)
    sg = [rng.uniform(0, 1, (24, 60, 72)).astype(np.float32) for _ in range(3)]
    sgm_cg = rng.uniform(0, 0.5, (12, 30, 48)).astype(np.float32)
    x0 = rng.uniform(0, 0.01, (8, 24, 24)).astype(np.float32)
    paths = []
    for i, s in enumerate(sg):
        paths.append(tmp_path / f"sgm_{i}.raw")
        s.tofile(paths[-1])
    sgm_cg.tofile(tmp_path / "cg_sgm.raw")
    x0.tofile(tmp_path / "cg_x0.raw")

    srv = ReconServer(batch=2)
    want = [srv.submit_fbp(o, s).result(timeout=120) for s in sg]
    want_cg = srv.submit_cgls(cg, sgm_cg, x0, 3).result(timeout=120)
    futs = [srv.submit_fbp(o, p, out_path=tmp_path / f"rec_{i}.raw") for i, p in enumerate(paths)]
    bad = srv.submit_fbp(o, tmp_path / "missing.raw")
    fut_cg = srv.submit_cgls(cg, str(tmp_path / "cg_sgm.raw"), tmp_path / "cg_x0.raw", 3,
                             out_path=tmp_path / "cg_out.raw")
    got = [f.result(timeout=120) for f in futs]
    got_cg = fut_cg.result(timeout=120)
    with pytest.raises(FileNotFoundError):
        bad.result(timeout=60)
    srv.close()
    for i in range(3):
        assert np.array_equal(got[i], want[i])
        assert np.array_equal(np.fromfile(tmp_path / f"rec_{i}.raw", dtype=np.float32).reshape(want[i].shape),
                              want[i])
    assert np.allclose(got_cg, want_cg, rtol=1e-6, atol=1e-7)
    assert np.array_equal(np.fromfile(tmp_path / "cg_out.raw", dtype=np.float32).reshape(got_cg.shape), got_cg)


def test_batched_cgls_requests_match_alone(cuda):
    """Several CGLS requests of one class run as one batch (a captured graph per member
    on a slot that shares the projector workspace between members): each result equals
    the request run alone."""
    from reconstruction_program_taichi_gb300.serve import ReconServer
    rng = np.random.default_rng(31)
    cg = _cgls_obj(n=24, nz=8, nu=48, nv=12, views=30, DetectorElementHeight=1.0)
    sg = [rng.uniform(0, 0.5, (12, 30, 48)).astype(np.float32) for _ in range(3)]
    x0 = [rng.uniform(0, 0.01, (8, 24, 24)).astype(np.float32) for _ in range(3)]
    srv = ReconServer(batch=1, max_slots_per_class=1)
    alone = [srv.submit_cgls(cg, s, x, 4).result(timeout=120) for s, x in zip(sg, x0)]
    srv.close()
    srv = ReconServer(batch=4, max_slots_per_class=1)
    srv.submit_cgls(cg, sg[0], x0[0], 4).result(timeout=120)  # builds the slot (a graph per member)
    futs = [srv.submit_cgls(cg, s, x, 4) for s, x in zip(sg, x0)]
    got = [f.result(timeout=120) for f in futs]
    st = srv.stats()
    srv.close()
    assert st["slots"]["cgls"] == 1
    for a, b in zip(alone, got):
        assert np.allclose(a, b, rtol=1e-6, atol=1e-7)


def test_partial_batch_runs_only_its_members(cuda):
    """A batch of k requests on a slot of `batch` members replays the graphs of its
    first k members only: the other members' outputs are not recomputed."""
    import torch
    from reconstruction_program_taichi_gb300.serve import _FbpSlot, _Request
    o = _cone_obj(n=40, nz=16, nu=72, nv=24, views=60)
    slot = _FbpSlot(o, 3, "f32", torch.device("cuda"), use_graph=True)
    assert len(slot.graphs) == 3
    rng = np.random.default_rng(33)
    s = rng.uniform(0, 1, (24, 60, 72)).astype(np.float32)
    for t in slot.out[1:]:
        t.fill_(7.0)
    out = slot.run([_Request("fbp", o, s)])
    torch.cuda.synchronize()
    assert all(bool((t == 7.0).all()) for t in slot.out[1:])
    full = slot.run([_Request("fbp", o, s)] * 3)
    assert all(np.array_equal(out[0], f) for f in full)


def test_configs_that_differ_only_in_the_scan_range_are_not_batched(cuda):
    """A short scan (Parker weights, other angles and redundancy factor) and a full scan
    of otherwise equal configs go to different slots: in a mix each result equals its
    own config's result alone."""
    from reconstruction_program_taichi_gb300.serve import ReconServer
    rng = np.random.default_rng(34)
    full, short = _cone_obj(n=40, nz=16, nu=72, nv=24, views=60), _cone_obj(n=40, nz=16, nu=72, nv=24, views=60,
                                                                          TotalScanAngle=220)
    s = rng.uniform(0, 1, (24, 60, 72)).astype(np.float32)
    srv = ReconServer(batch=1, max_slots_per_class=1)
    want = [srv.submit_fbp(o, s).result(timeout=120) for o in (full, short)]
    srv.close()
    assert not np.array_equal(want[0], want[1])
    srv = ReconServer(batch=4, max_slots_per_class=1)
    futs = [srv.submit_fbp(o, s) for o in (full, short, full, short)]
    got = [f.result(timeout=120) for f in futs]
    st = srv.stats()
    srv.close()
    assert st["classes"] == 2
    for i, g in enumerate(got):
        assert np.array_equal(g, want[i % 2])


def test_mixed_precision_requests(cuda):
    """storage='bf16' serves the mixed path (two-part tensor-core filter, bf16
    backprojection coefficients; bf16 projector cells in CGLS): the same result as the
    pipeline run directly, close to the plain result, in its own slot class."""
    import torch
    from reconstruction_program_taichi_gb300.fbp import FdkPipeline
    from reconstruction_program_taichi_gb300.serve import ReconServer
    rng = np.random.default_rng(35)
    o = _cone_obj(n=40, nz=16, nu=72, nv=24, views=60)
    s = rng.uniform(0, 1, (24, 60, 72)).astype(np.float32)
    cg = _cgls_obj(n=24, nz=8, nu=48, nv=12, views=30, DetectorElementHeight=1.0)
    sc = rng.uniform(0, 0.5, (12, 30, 48)).astype(np.float32)
    x0 = np.zeros((8, 24, 24), np.float32)
    srv = ReconServer(batch=2, max_slots_per_class=1)
    plain, mixed = srv.submit_fbp(o, s).result(timeout=120), srv.submit_fbp(o, s, storage="bf16").result(timeout=120)
    cg_plain = srv.submit_cgls(cg, sc, x0, 3).result(timeout=120)
    cg_mixed = srv.submit_cgls(cg, sc, x0, 3, storage="bf16").result(timeout=120)
    st = srv.stats()
    srv.close()
    assert st["classes"] == 4
    direct = FdkPipeline(o, storage="bf16", filter_impl="tc").run(torch.from_numpy(s).cuda()).cpu().numpy()
    assert np.array_equal(mixed, direct)
    assert np.array_equal(plain == 0, mixed == 0)
    assert np.linalg.norm(mixed - plain) / np.linalg.norm(plain) < 5e-3
    assert np.linalg.norm(cg_mixed - cg_plain) / np.linalg.norm(cg_plain) < 2e-2
