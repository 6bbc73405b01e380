"""Photon noise of the forward projector (AddPossionNoise, run_mgfpj_v3.py:381-391):
per detector element, t = N0 exp(-p) + g sqrt(N0 exp(-p)) with g standard normal,
t <= 0 replaced by 1e-6, and the output log(N0 / t).  The generator is seeded here (the
reference's ti.randn is not), so the checks are statistical: over many elements the
output's mean and variance follow from the formula (mean p + 1/(2 mu), variance 1/mu
with mu = N0 exp(-p), to first order), about 68.3 % lie within one standard deviation,
the clamp fires with the normal distribution's tail probability, neighbours are
uncorrelated, and a seed reproduces its noise exactly."""
import math

import numpy as np
import pytest

from test_gpu_parity import _cone_obj

pytestmark = pytest.mark.gpu


def _geom(nv, views, nu):
    from reconstruction_program_taichi_gb300 import geometry
    o = _cone_obj(n=16, nz=8, nu=nu, nv=nv, views=views)
    return geometry.fpj_geometry(o)


def _phi(x):
    return 0.5 * math.erfc(-x / math.sqrt(2.0))


@pytest.mark.parametrize("p", [0.5, 2.0, 4.0])
def test_noise_mean_variance_and_spread(p, cuda):
    import torch
    from reconstruction_program_taichi_gb300 import ops
    dg = _geom(64, 128, 128)  # 1,048,576 elements
    n0 = 1e5
    x = torch.full(dg.sgm_shape, p, dtype=torch.float32, device="cuda")
    y = ops.bin_noise(dg, x, 1, photons=n0, seed=11).double().cpu().numpy().ravel()
    mu = n0 * math.exp(-p)
    n = y.size
    var = 1.0 / mu
    mean_want = p + 0.5 / mu
    assert abs(y.mean() - mean_want) < 5 * math.sqrt(var / n), (y.mean(), mean_want)
    assert abs(y.var() / var - 1.0) < 0.015, y.var() / var
    inside = np.mean(np.abs(y - p) < math.sqrt(var))
    assert abs(inside - 0.6827) < 0.003, inside
    # neighbouring elements (same row, next column; same column, next view) are independent
    a = y.reshape(dg.sgm_shape) - y.mean()
    for b, c in ((a[:, :, 1:], a[:, :, :-1]), (a[:, 1:, :], a[:, :-1, :])):
        corr = float((b * c).mean() / a.var())
        assert abs(corr) < 0.005, corr


def test_noise_clamp_at_low_counts(cuda):
    """N0 = 20, p = 3: mu ~ 1, t < 0 whenever g < -sqrt(mu); such elements read
    log(N0 / 1e-6)."""
    import torch
    from reconstruction_program_taichi_gb300 import ops
    dg = _geom(32, 128, 128)
    n0, p = 20.0, 3.0
    x = torch.full(dg.sgm_shape, p, dtype=torch.float32, device="cuda")
    y = ops.bin_noise(dg, x, 1, photons=n0, seed=5).cpu().numpy()
    mu = n0 * math.exp(-p)
    clamp_val = np.float32(math.log(n0 / 1e-6))
    frac = float(np.mean(np.isclose(y, clamp_val, rtol=1e-6)))
    want = _phi(-math.sqrt(mu))
    assert abs(frac - want) < 0.005, (frac, want)


def test_noise_is_reproducible_per_seed_and_follows_binning(cuda):
    """The same seed gives the same noise, another seed other noise; with oversampling
    the noise is applied to the binned (averaged) sub-columns, and without photons the
    result is the plain binning."""
    import torch
    from reconstruction_program_taichi_gb300 import ops
    dg = _geom(16, 64, 96)
    g = torch.Generator(device="cuda").manual_seed(3)
    big = torch.rand((16, 64, 96 * 2), device="cuda", generator=g) * 3
    a = ops.bin_noise(dg, big, 2, photons=1e4, seed=9)
    b = ops.bin_noise(dg, big, 2, photons=1e4, seed=9)
    c = ops.bin_noise(dg, big, 2, photons=1e4, seed=10)
    assert torch.equal(a, b) and not torch.equal(a, c)
    binned = ops.bin_noise(dg, big, 2)
    assert torch.allclose(binned, big.view(16, 64, 96, 2).mean(-1), rtol=1e-6, atol=1e-6)
    mu = 1e4 * torch.exp(-binned.double())
    z = ((a.double() - binned.double()) * mu.sqrt()).cpu().numpy()  # ~ standard normal
    assert abs(z.mean()) < 0.02 and abs(z.var() - 1.0) < 0.05


def test_run_mgfpj_v3_with_photon_number(tmp_path, cuda):
    """The drop-in with PhotonNumber: the noisy projection minus the noiseless one,
    scaled by sqrt(N0 exp(-p)) per ray, is standard normal; other noise seeds give other
    noise."""
    import copy
    import json
    from conftest import load_golden
    from reconstruction_program_taichi_gb300 import run_mgfpj_v3
    z = load_golden("fpj_cone")
    outs = []
    for photons, seed in ((None, 0), (1e5, 0), (1e5, 1)):
        cfg = copy.deepcopy(z["config"])
        d = tmp_path / f"run_{seed}_{photons}"
        (d / "in").mkdir(parents=True)
        cfg.update(InputDir=str(d / "in"), OutputDir=str(d / "out"))
        if photons:
            cfg["PhotonNumber"] = photons
        z["input_vol"].astype(np.float32).tofile(d / "in" / "img_a.raw")
        (d / "c.jsonc").write_text(json.dumps(cfg))
        outs.append(run_mgfpj_v3(str(d / "c.jsonc"), verbose=False, noise_seed=seed).astype(np.float64))
    clean, noisy, other = outs
    assert np.linalg.norm(clean - z["sgm"]) / np.linalg.norm(z["sgm"]) < 1e-4
    zsc = (noisy - clean) * np.sqrt(1e5 * np.exp(-clean))
    assert abs(zsc.mean()) < 5 / math.sqrt(zsc.size) and abs(zsc.var() - 1.0) < 0.1
    assert not np.array_equal(noisy, other)
