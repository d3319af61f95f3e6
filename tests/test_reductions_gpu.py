"""The f32 engine's reductions (merit sums, merit seed, clip norm) against
FP64 computations from the same f32 values.

Their per-thread partials run on the FP32 pipe as error-free pairs (exact
products by FMA, TwoSum), so a sum matches the exactly rounded FP64 sum of
the same f32 products to ~1e-13 (relative), far inside the f32 engine's own
error; the seed c w is the f32 rounding of the FP64 product (within one f32
ulp).
"""

import ctypes as C
import math

import numpy as np
import pytest

from oracle import adam as o_adam

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from optics_studio_gb300 import _ffi, inverse as inv  # noqa: E402

# frame lengths: a few elements, one partial per thread, and a multi-block grid
LENS = [7, 1000, 3 * 2**20 + 5]


@pytest.mark.parametrize("n", LENS)
def test_weighted_sums_and_seed_f32(n):
    rng = np.random.default_rng(n)
    frames = 3
    obs = rng.uniform(0.0, 3.0, (frames, n)).astype(np.float32)
    w = rng.uniform(0.0, 1.0, n).astype(np.float32)  # spot weights are non-negative
    w[rng.random(n) < 0.3] = 0.0  # zero weights are skipped
    p_in = [1.7, 2.9, 0.4][:frames]
    d_obs = torch.from_numpy(obs).cuda()
    d_w = torch.from_numpy(w).cuda()
    d_seed = torch.full((frames, n), float("nan"), dtype=torch.float32, device="cuda")
    v = C.c_double()
    pin = (C.c_double * frames)(*p_in)
    _ffi.check(_ffi.lib().osgpu_merit_weighted_efficiency_device(
        d_obs.data_ptr(), _ffi.F32, frames, n, d_w.data_ptr(), pin, d_seed.data_ptr(), None,
        C.byref(v)))
    torch.cuda.synchronize()
    sums = [math.fsum((w.astype(np.float64) * obs[f].astype(np.float64)).tolist())
            for f in range(frames)]
    want = -sum(s / p for s, p in zip(sums, p_in))
    assert v.value == pytest.approx(want, rel=1e-12, abs=1e-12)
    seed = d_seed.cpu().numpy().astype(np.float64)
    ref = np.stack([(-1.0 / p) * w.astype(np.float64) for p in p_in])
    np.testing.assert_allclose(seed, ref, rtol=2 ** -23, atol=0)


@pytest.mark.parametrize("n", LENS)
def test_adam_clip_norm_of_f32_gradient(n):
    rng = np.random.default_rng(100 + n)
    x = rng.uniform(0.0, 2 * math.pi, n)
    g32 = (rng.normal(size=n) * 3.0).astype(np.float32)
    cfg = inv.AdamConfig(lr_frac=0.05 / (2 * math.pi), clip_norm=1.0)
    xd = torch.from_numpy(x).cuda()
    opt = inv.Adam(xd, 0.0, 2 * math.pi, cfg)
    opt.step(torch.from_numpy(g32).cuda())
    torch.cuda.synchronize()
    xo, _, _ = o_adam.adam_step(x, g32.astype(np.float64), np.zeros(n), np.zeros(n), 1, 0.0,
                                2 * math.pi, cfg.lr_frac, cfg.beta1, cfg.beta2, cfg.eps, 1.0)
    np.testing.assert_allclose(xd.cpu().numpy(), xo, rtol=1e-12, atol=1e-12)
