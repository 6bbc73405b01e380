"""mct_dot_f64_noalloc: the float64 inner product for callers that cannot allocate
device memory (an application that owns every GPU buffer and hands the library only
its inputs and outputs).  Called through the C ABI and checked against the
allocating entry point mct_dot_f64 on two calls in a row, so that a result left in
the shared scratch by the first call cannot leak into the second.

This file is named so that pytest collects it last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_dot_matches_allocating_entry_point(cuda):
    import torch
    from reconstruction_program_taichi_gb300 import _lib
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    scratch = torch.empty(int(lib.mct_reduce_scratch_size()) // 8, dtype=torch.float64, device="cuda")
    gen = torch.Generator(device="cuda").manual_seed(12)
    for n in (3_000_001, 4097):  # two calls in a row; the second is much shorter than the first
        a = torch.randn(n, device="cuda", generator=gen)
        b = torch.randn(n, device="cuda", generator=gen)
        want = torch.empty((), dtype=torch.float64, device="cuda")
        got = torch.full((), float("nan"), dtype=torch.float64, device="cuda")
        assert lib.mct_dot_f64(_p(a), _p(b), n, _p(scratch), _p(want), stream) == 0
        assert lib.mct_dot_f64_noalloc(_p(a), _p(b), n, _p(got), stream) == 0, lib.mct_last_error_string()
        torch.cuda.synchronize()
        exact = float(np.dot(a.double().cpu().numpy(), b.double().cpu().numpy()))
        assert abs(float(got) - float(want)) <= 1e-9 * max(1.0, abs(float(want)))
        assert abs(float(got) - exact) <= 1e-9 * max(1.0, abs(exact))


def test_noalloc_dot_rejects_sizes_beyond_its_scratch(cuda):
    import torch
    from reconstruction_program_taichi_gb300 import _lib
    lib = _lib.load()
    out = torch.empty((), dtype=torch.float64, device="cuda")
    x = torch.zeros(16, device="cuda")
    rc = lib.mct_dot_f64_noalloc(_p(x), _p(x), 134_217_729, _p(out), None)
    assert rc == -1
    assert b"exceeds the maximum of 134217728" in lib.mct_last_error_string()
    assert lib.mct_dot_f64_noalloc(_p(x), _p(x), 0, _p(out), None) == 0
    torch.cuda.synchronize()
    assert float(out) == 0.0
