"""ScanStream: pipelined scans give exactly the results of the sequential flow, each
scan its own (the two buffer sets and three streams never mix scans up)."""
import numpy as np
import pytest

from test_gpu_parity import _cone_obj

pytestmark = pytest.mark.gpu


def test_scan_stream_matches_sequential(cuda):
    import torch
    from reconstruction_program_taichi_gb300 import fbp, geometry, ops
    from reconstruction_program_taichi_gb300.stream import ScanStream
    o = _cone_obj(n=40, nz=16, nu=72, nv=24, views=60)
    pipe = fbp.FdkPipeline(o)
    fpg = geometry.fpj_geometry(_cone_obj(n=40, nz=16, nu=72, nv=24, views=36))
    rng = np.random.default_rng(31)
    shape = (o.det_elem_count_vertical, o.view_num, o.det_elem_count_horizontal)
    scans = [rng.uniform(0, 1, shape).astype(np.float32) for _ in range(5)]

    want = []
    for s in scans:
        vol = pipe.run(torch.from_numpy(s).cuda()).clone()
        want.append((vol.cpu().numpy(), ops.fp(fpg, vol).cpu().numpy()))

    st = ScanStream(pipe, fpg)
    host_in = [torch.from_numpy(s).pin_memory() for s in scans]
    host_vol = [torch.empty(pipe.dg.vol_shape, dtype=torch.float32, pin_memory=True) for _ in scans]
    host_fp = [torch.empty(fpg.sgm_shape, dtype=torch.float32, pin_memory=True) for _ in scans]
    for i in range(len(scans)):
        st.submit(host_in[i], host_vol[i], host_fp[i])
    st.synchronize()
    for i, (v, p) in enumerate(want):
        assert np.array_equal(host_vol[i].numpy(), v), i
        assert np.array_equal(host_fp[i].numpy(), p), i


def test_scan_stream_rejects_pageable_buffers(cuda):
    import torch
    from reconstruction_program_taichi_gb300 import fbp
    from reconstruction_program_taichi_gb300.stream import ScanStream
    o = _cone_obj(n=24, nz=8, nu=48, nv=12, views=30)
    pipe = fbp.FdkPipeline(o)
    st = ScanStream(pipe)
    sgm = torch.zeros((o.det_elem_count_vertical, o.view_num, o.det_elem_count_horizontal))
    with pytest.raises(ValueError, match="pinned"):
        st.submit(sgm, torch.empty(pipe.dg.vol_shape, pin_memory=True))
    with pytest.raises(ValueError, match="host_proj"):
        st.submit(sgm.pin_memory(), torch.empty(pipe.dg.vol_shape, pin_memory=True),
                  torch.empty((1,), pin_memory=True))
    with pytest.raises(ValueError, match="shape"):
        st.submit(sgm.pin_memory(), torch.empty((1, 2, 3), pin_memory=True))
