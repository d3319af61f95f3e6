"""The detector-metric merits (osgpu_merit_{spot_rms,strehl,mtf}_device)
against the oracle's restatement of crates/optics-inverse/src/merit.rs:248-400.

Values and obs gradients are FP64 reductions of the same observation, so they
match the oracle to 1e-12 (relative; the spot seed relative to its largest
entry, the MTF merit absolutely since it is a ratio of at most 1); a seed
written into an f32 observation carries its f32 rounding (2e-7).  The
reference's own merit tests (merit.rs:474-576) are repeated on the device, and
the spot merit drives a full adjoint gradient compared with the oracle's.
"""

import math

import numpy as np
import pytest

from oracle import adjoint as o_adj, analysis as o_an, asm as o_asm, carrier as o_car
from oracle import element as o_el, field as o_field, merit as o_merit, observe as o_obs

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from optics_studio_gb300 import _ffi, inverse as inv, element as el  # noqa: E402
from optics_studio_gb300.propagation.asm import AsmConfig  # noqa: E402

NX, NY, D = 64, 48, 4e-6
BANDS = [5e-7, 6e-7]


def observations(dtype, seed=9, B=2, S=3):
    rng = np.random.default_rng(seed)
    data = rng.uniform(0.0, 2.0, (1, B, S, NY, NX))
    if dtype == torch.float32:
        data = data.astype(np.float32).astype(np.float64)
    args = (["intensity"], BANDS[:B], [(0, 0)] * S, (NX, NY), (D, D))
    return (o_obs.Observation(*args, data),
            inv.Observation(*args, torch.from_numpy(data).to("cuda", dtype)))


SELECTORS = [(None, None), (1, None), (None, 2), (0, 1)]


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_merits_match_oracle_with_selectors(dtype):
    obs_o, obs_g = observations(dtype)
    ref = np.random.default_rng(3).uniform(0.0, 1.0, (NY, NX))
    seed_tol = 1e-12 if dtype == torch.float64 else 2e-7
    for band, scene in SELECTORS:
        om, gm = o_merit.SpotRmsMerit(band, scene), inv.SpotRmsMerit(band, scene)
        assert gm.evaluate(obs_g) == pytest.approx(om.evaluate(obs_o), rel=1e-12)
        want = om.obs_gradient(obs_o)
        got = gm.obs_gradient(obs_g).cpu().numpy().astype(np.float64)
        assert got.shape == want.shape
        assert np.max(np.abs(got - want)) <= seed_tol * np.max(np.abs(want))
        # the merit-and-seed call used by grid_gradient writes the same seed
        seed = torch.zeros_like(obs_g.data)
        v, ok = inv.merit_value_and_seed(gm, obs_g, seed)
        assert ok and v == pytest.approx(om.evaluate(obs_o), rel=1e-12)
        got = seed.cpu().numpy().astype(np.float64)
        assert np.max(np.abs(got - want)) <= seed_tol * np.max(np.abs(want))

        os_, gs_ = o_merit.StrehlMerit(ref, band, scene), inv.StrehlMerit(ref, band, scene)
        assert gs_.evaluate(obs_g) == pytest.approx(os_.evaluate(obs_o), rel=1e-12)
        assert gs_.obs_gradient(obs_g) is None

        for m in (0, 1, 5, NX // 2 - 1, NX // 2):
            f = m / (NX * D)
            if 2.0 * f * D >= 1.0:
                continue
            want_m = o_merit.MtfMerit(f, band, scene).evaluate(obs_o)
            got_m = inv.MtfMerit(f, band, scene).evaluate(obs_g)
            assert abs(got_m - want_m) <= 1e-13, (band, scene, m, got_m, want_m)


def gaussian_frame(n):
    """merit.rs:427-438."""
    w = n * 10e-6 / 6.0
    c = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * 10e-6
    return np.exp(-2.0 * (c[None, :] ** 2 + c[:, None] ** 2) / (w * w))


def test_reference_merit_anchors_on_device():
    """merit.rs:474-520, 556-576: spot merit = spot_rms_radius (1e-9), Strehl
    of a frame against itself = -1 (1e-12), MTF merit at the fifth bin = -mtf
    (2e-3)."""
    n = 32
    frame = gaussian_frame(n)
    obs = inv.Observation(["intensity"], [500e-9], [(0.0, 0.0)], (n, n), (10e-6, 10e-6),
                          torch.from_numpy(frame.reshape(1, 1, 1, n, n)).cuda())
    want = o_an.spot_rms_radius(frame, (10e-6, 10e-6))
    assert abs(inv.SpotRmsMerit().evaluate(obs) - want) / want < 1e-9
    assert abs(inv.StrehlMerit(frame).evaluate(obs) + 1.0) < 1e-12
    freqs, vals = o_an.mtf(frame, (10e-6, 10e-6))
    assert abs(inv.MtfMerit(freqs[4]).evaluate(obs) + vals[4]) < 2e-3


def test_merit_errors_and_dark_frames():
    _, obs_g = observations(torch.float64, B=2, S=1)
    with pytest.raises(_ffi.OsgpuError) as e:
        inv.SpotRmsMerit(band=5).evaluate(obs_g)
    assert e.value.code == 102  # BadArgument
    for f in (1.5 / (NX * D), 0.6 / D, -1.0):  # between bins, above Nyquist, negative
        with pytest.raises(_ffi.OsgpuError) as e:
            inv.MtfMerit(f).evaluate(obs_g)
        assert e.value.code == 43
    with pytest.raises(_ffi.OsgpuError) as e:
        inv.StrehlMerit(np.ones(NX * NY + 1)).evaluate(obs_g)
    assert e.value.code == 43
    dark = inv.Observation(["intensity"], [5e-7], [(0, 0)], (NX, NY), (D, D),
                           torch.zeros((1, 1, 1, NY, NX), dtype=torch.float64, device="cuda"))
    assert inv.SpotRmsMerit().evaluate(dark) == 0.0
    assert inv.SpotRmsMerit().obs_gradient(dark) is None
    assert inv.StrehlMerit(np.ones((NY, NX))).evaluate(dark) == 0.0
    assert inv.MtfMerit(0.0).evaluate(dark) == 0.0


# ---- the spot merit through the adjoint ----------------------------------------
N, Z1, Z2, R_AP = 64, 2e-3, 3e-3, 100e-6
RB = [520e-9, 580e-9]


def o_source(x0, y0, lam):
    return o_field.gaussian(60e-6, 1.0, (x0, y0), 0.0, lam, N, N, D, D)


def o_design(v, lam):
    d = o_car.Design()
    d.push(o_el.PhaseMask.sampled(v, (N, N), (D, D)), Z1)
    d.push(o_el.EllipticalAperture.circle(R_AP), Z2)
    return d


def g_renderer(precision):
    cdt = torch.complex128 if precision == "f64" else torch.complex64

    def source(x0, y0, lam):
        return torch.from_numpy(o_source(x0, y0, lam).samples).to("cuda", cdt)

    def carrier(values, lam):
        d = inv.Design()
        d.push(inv.DevicePhaseMask(values, (N, N), (D, D)), Z1)
        d.push(el.EllipticalAperture.circle(R_AP), Z2)
        return d

    return inv.Renderer(carrier, source, (D, D), bands=list(RB), asm_cfg=AsmConfig(),
                        precision=precision)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_spot_rms_grid_gradient_matches_oracle(precision):
    phi = np.random.default_rng(21).uniform(0.0, 2 * math.pi, (N, N))
    car = o_car.Carrier.analytic(N * N, 0.0, 2 * math.pi, o_design)
    rend_o = o_obs.Renderer(car, o_source, bands=list(RB), scenes=[(0.0, 0.0)],
                            asm_cfg=o_asm.AsmConfig())
    om = o_merit.SpotRmsMerit()
    want = o_adj.grid_gradient(rend_o, phi.reshape(-1), om)
    want_val = om.evaluate(rend_o.render(phi.reshape(-1)))
    got, val, _ = inv.grid_gradient(g_renderer(precision), torch.from_numpy(phi).cuda(),
                                    inv.SpotRmsMerit())
    torch.cuda.synchronize()
    tol = 1e-12 if precision == "f64" else 1e-4
    assert sorted(got) == [0, 1]
    for ei in (0, 1):
        g, w = got[ei].cpu().numpy(), want[ei].reshape(N, N)
        assert np.linalg.norm(g - w) / np.linalg.norm(w) <= tol, ei
    assert abs(val - want_val) <= (1e-12 if precision == "f64" else 1e-5) * abs(want_val)
    # a merit without obs gradient is rejected, as adjoint.rs:274-281 does
    with pytest.raises(_ffi.OsgpuError) as e:
        inv.grid_gradient(g_renderer(precision), torch.from_numpy(phi).cuda(),
                          inv.MtfMerit(0.0))
    assert e.value.code == 44
