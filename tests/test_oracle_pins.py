"""Pins the f64 oracle against the reference's own known-answer tests and its
hypercam golden vector.  CPU only (no GPU marker)."""

import math
import pathlib

import numpy as np
import pytest

from oracle import asm, fresnel, fraunhofer, rs, element, field, gs, adjoint, carrier, observe, merit, adam
from oracle.fft import fft2, ifft2, fftfreq, padded_len

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
LAM = 500e-9


def noise(n):
    """xorshift64 noise of ``fft.rs:134-150`` (same recurrence)."""
    state = 0x2545F491
    mask = (1 << 64) - 1
    out = []
    for _ in range(n):
        state ^= (state << 13) & mask
        state ^= state >> 7
        state ^= (state << 17) & mask
        re = state / float(mask) - 0.5
        state ^= (state << 13) & mask
        state ^= state >> 7
        state ^= (state << 17) & mask
        im = state / float(mask) - 0.5
        out.append(complex(re, im))
    return np.array(out)


# ---- fft.rs:159-259 convention pins ---------------------------------------

@pytest.mark.parametrize("nx,ny", [(8, 8), (6, 7), (1, 5), (5, 1)])
def test_fft_roundtrip(nx, ny):
    u = noise(nx * ny).reshape(ny, nx)
    assert np.max(np.abs(ifft2(fft2(u)) - u)) < 1e-12


def test_fft_parseval_delta_sign_convolution():
    u = noise(54).reshape(6, 9)
    assert abs(np.sum(np.abs(fft2(u)) ** 2) - 54 * np.sum(np.abs(u) ** 2)) < 1e-9 * 54
    d = np.zeros((4, 8), complex)
    d[0, 0] = 1
    assert np.all(np.abs(fft2(d) - 1) < 1e-12)
    nx, ny, k0 = 16, 4, 3
    buf = np.exp(1j * 2 * math.pi * k0 * np.arange(nx) / nx)[None, :].repeat(ny, 0)
    f = fft2(buf)
    assert abs(f[0, k0] - nx * ny) < 1e-9
    u = noise(20).reshape(4, 5)
    h = noise(20).reshape(4, 5)[::-1].copy()
    prod = ifft2(fft2(u) * fft2(h))
    direct = np.zeros_like(u)
    for iy in range(4):
        for ix in range(5):
            direct[iy, ix] = sum(u[jy, jx] * h[(iy - jy) % 4, (ix - jx) % 5]
                                 for jy in range(4) for jx in range(5))
    assert np.max(np.abs(prod - direct)) < 1e-9


def test_fftfreq_matches_numpy_semantics():
    assert list(fftfreq(4, 1.0)) == [0.0, 0.25, -0.5, -0.25]
    assert list(fftfreq(5, 1.0)) == [0.0, 0.2, 0.4, -0.4, -0.2]
    assert padded_len(100, 2.0) == 200 and padded_len(100, 1.5) == 150
    assert padded_len(100, 1.0) == 100 and padded_len(100, 0.5) == 100


# ---- asm.rs:548-790 + tests/asm.rs -----------------------------------------

def band_uniform(a, n, d):
    return field.uniform(a, 0.0, n, n, d, d, LAM)


def test_asm_z0_identity_and_plane_wave_phase():
    b = band_uniform(1.5, 16, 20e-6)
    assert np.array_equal(asm.propagate(b, 0.0).samples, b.samples)
    cfg = asm.AsmConfig(padding=1.0)
    out = asm.propagate(band_uniform(1.0, 16, 20e-6), 1e-3, cfg)
    k = 2 * math.pi / LAM
    assert abs(out.samples[9, 3] - np.exp(1j * k * 1e-3)) < 1e-9
    rt = asm.propagate(out, -1e-3, cfg)
    assert np.max(np.abs(rt.samples - 1.0)) < 1e-9


def test_asm_medium_piston_and_guard():
    cfg = asm.AsmConfig(padding=1.0, medium=1.5)
    out = asm.propagate(band_uniform(1.0, 16, 20e-6), 1e-3, cfg)
    k = 2 * math.pi / LAM
    assert abs(out.samples[9, 3] - np.exp(1j * 1.5 * k * 1e-3)) < 1e-9
    for n in [0.0, -1.5, float("nan"), float("inf")]:
        with pytest.raises(asm.PropagationError) as e:
            asm.propagate(band_uniform(1.0, 8, 20e-6), 1e-3, asm.AsmConfig(medium=n))
        assert e.value.variant == "InvalidMedium"
    b = band_uniform(1.0, 32, 1e-6)
    base = asm.AsmConfig(padding=2.0, band_limited=False, strict=False)
    r1 = asm.sampling_report(b, 0.5, base)
    r2 = asm.sampling_report(b, 0.5, asm.AsmConfig(2.0, False, False, 8.0, 1.5))
    assert abs(r2.band_limit_fx - 1.5 * r1.band_limit_fx) < 1e-9
    assert 0.55 < r2.max_phase_step_x / r1.max_phase_step_x < 1.0


def test_asm_sampling_guard_and_mitigation():
    """tests/asm.rs:286-345."""
    b = band_uniform(1.0, 64, 1e-6)
    z = 7.68e-4
    risk = asm.AsmConfig(1.0, False, True, 1.0, 1.0)
    with pytest.raises(asm.PropagationError) as e:
        asm.propagate(b, z, risk)
    assert e.value.variant == "AliasingRisk" and e.value.report.max_phase_step_x > math.pi
    assert e.value.report.used_padding == 1.0
    loose = asm.AsmConfig(1.0, False, False, 1.0, 1.0)
    assert asm.propagate(b, z, loose).samples.shape == (64, 64)
    fix = asm.AsmConfig(1.0, False, True, 8.0, 1.0)
    assert asm.resolve_report(b, z, fix).used_padding == 8.0
    assert not asm.sampling_report(b, z, asm.AsmConfig(4.0, False, True, 8.0, 1.0)).nyquist_ok


def gaussian_env(n, d, sigma):
    x = field.axis_coords(n, d)
    return np.exp(-((x[None, :] ** 2 + x[:, None] ** 2) / (2 * sigma * sigma))) + 0j


def test_asm_energy_and_round_trip():
    """tests/asm.rs:91-98, 356-373."""
    b = field.BandField(gaussian_env(256, 10e-6, 0.15e-3), 10e-6, 10e-6, LAM)
    out = asm.propagate(b, 0.1)
    assert abs(out.power() - b.power()) / b.power() <= 1e-9
    back = asm.propagate(out, -0.1)
    rel = np.linalg.norm(back.samples - b.samples) / np.linalg.norm(b.samples)
    assert rel < 1e-6


def test_asm_tilted_plane_wave():
    """tests/asm.rs:143-168."""
    n, dx, m = 128, 10e-6, 3.0
    alpha = m * LAM / (n * dx)
    b = field.plane_wave(math.asin(alpha), 0.0, 1.0, n, n, dx, dx, LAM)
    out = asm.propagate(b, 0.01, asm.AsmConfig(1.0, True, False, 1.0, 1.0))
    step = np.exp(1j * 2 * math.pi / LAM * alpha * dx)
    for iy in [0, 64, 127]:
        assert abs(out.samples[iy, 60] / out.samples[iy, 59] - step) < 1e-6


# ---- fresnel / fraunhofer / RS unit pins -----------------------------------

def test_fresnel_conv_of_delta_is_sampled_kernel_and_tf_close_to_conv():
    n, d = 64, 10e-6
    u = np.zeros((n, n), complex)
    u[n // 2, n // 2] = 1.0
    b = field.BandField(u, d, d, LAM)
    lam_z = n * 2 * d * d  # critical sampling n_pad dx^2 = lam z
    z = lam_z / LAM
    conv = fresnel.propagate_convolution(b, z, fresnel.FresnelConfig(strict=False))
    tf = fresnel.propagate(b, z, fresnel.FresnelConfig(strict=False))
    assert np.linalg.norm(conv.samples - tf.samples) / np.linalg.norm(tf.samples) < 0.2
    # The convolution of a centred delta is the sampled kernel around the centre.
    h = fresnel.impulse_response(2 * n, 2 * n, d, d, LAM, z)
    assert abs(conv.samples[n // 2, n // 2] - h[0, 0]) < 1e-12 * abs(h[0, 0])


def test_fraunhofer_delta_prefactor_and_parseval():
    """fraunhofer.rs:466-531: delta at the origin sample -> flat |quad| dx dy."""
    n, d, z = 33, 10e-6, 1.0
    u = np.zeros((n, n), complex)
    u[16, 16] = 1.0
    b = field.BandField(u, d, d, LAM)
    out = fraunhofer.propagate(b, z, fraunhofer.FraunhoferConfig(strict=False))
    assert np.allclose(np.abs(out.samples), d * d / (LAM * z), rtol=1e-12)
    u2 = noise(32 * 32).reshape(32, 32)
    b2 = field.BandField(u2, d, d, LAM)
    o2 = fraunhofer.propagate(b2, z, fraunhofer.FraunhoferConfig(strict=False))
    assert abs(o2.power() - b2.power()) / b2.power() < 1e-9


def test_rs_delta_is_kernel_and_matches_asm_on_smooth_band():
    """rayleigh_sommerfeld.rs:532-601."""
    n, d, z = 32, 1e-5, 1e-3
    u = np.zeros((n, n), complex)
    u[0, 0] = 1.0
    b = field.BandField(u, d, d, LAM)
    out = rs.propagate(b, z, rs.RayleighSommerfeldConfig(padding=1.0, strict=False))
    h = rs.impulse_response(n, n, d, d, LAM, z)
    assert np.max(np.abs(out.samples - h)) < 1e-12
    n, d, z = 200, 2e-6, 5e-3
    g = field.BandField(gaussian_env(n, d, 30e-6), d, d, LAM)
    assert rs.sampling_report(g, z, rs.RayleighSommerfeldConfig()).kernel_nyquist_ok
    r = rs.propagate(g, z, rs.RayleighSommerfeldConfig())
    a = asm.propagate(g, z, asm.AsmConfig(padding=2.0))
    assert np.linalg.norm(a.samples - r.samples) / np.linalg.norm(a.samples) < 5e-2


# ---- element.rs pins ---------------------------------------------------------

def test_elements_boundary_inclusive_and_outside_field():
    b = band_uniform(1.0, 11, 1.0)
    circ = element.EllipticalAperture.circle(3.0)
    t = circ.transmission(b)
    assert t[5, 8] == 1 and t[5, 9] == 0 and t[2, 5] == 1
    rect = element.RectangularAperture((2.0, 1.0))
    tr = rect.transmission(b)
    assert tr[5, 7] == 1 and tr[5, 8] == 0 and tr[6, 5] == 1 and tr[7, 5] == 0
    with pytest.raises(element.OpticsError) as e:
        element.EllipticalAperture.circle(6.0).transmission(b)
    assert e.value.variant == "OutsideField"
    lens = element.ThinLens.fixed(0.1)
    tl = lens.transmission(field.uniform(1, 0, 8, 8, 1e-5, 1e-5, LAM))
    assert np.allclose(np.abs(tl), 1.0)


def test_sampled_phase_bilinear_and_zero_outside():
    vals = np.arange(12, dtype=float).reshape(3, 4)
    lat = (vals, 4, 3, 1.0, 1.0)
    assert element.sampled_at(lat, 0.0, 0.0) == pytest.approx(5.5)
    assert element.sampled_at(lat, -1.5, -1.0) == pytest.approx(0.0)
    assert element.sampled_at(lat, 1.5, 1.0) == pytest.approx(11.0)
    assert element.sampled_at(lat, 1.6, 0.0) == 0.0


# ---- gs.rs / adjoint.rs pins ---------------------------------------------------

def test_wrap_pi_and_encode_bounds():
    assert gs.wrap_pi(np.array([math.pi]))[0] == pytest.approx(-math.pi)
    assert gs.wrap_pi(np.array([0.5]))[0] == pytest.approx(0.5)
    assert gs.encode_bounds(np.array([7.0]), 0.0, 2 * math.pi)[0] == pytest.approx(7.0 - 2 * math.pi)
    assert gs.encode_bounds(np.array([7.0]), 0.0, 1.0)[0] == 1.0


def chirp_band(n, d, lam, a=3e7):
    x = field.axis_coords(n, d)
    r2 = x[None, :] ** 2 + x[:, None] ** 2
    return field.BandField(np.exp(-r2 / (2 * (n * d / 6) ** 2)) * np.exp(1j * a * r2), d, d, lam)


def test_asm_adjoint_inner_product_identity():
    """adjoint.rs:406-440: <w, A d> = <A(-z) w, d>."""
    cfg = asm.AsmConfig(padding=2.0, strict=False)
    d = chirp_band(32, 4e-6, LAM)
    w = field.BandField(noise(32 * 32).reshape(32, 32), 4e-6, 4e-6, LAM)
    ad = asm.propagate(d, 1e-3, cfg).samples
    aw = adjoint.asm_adjoint(w, 1e-3, cfg).samples
    lhs = np.vdot(w.samples, ad)
    rhs = np.vdot(aw, d.samples)
    assert abs(lhs - rhs) < 1e-12 * max(abs(lhs), 1e-30) + 1e-14


def test_adjoint_matches_central_fd_on_6x6():
    """adjoint.rs:499-544: grid gradient vs central FD, rel < 1e-4."""
    n, d, lam = 6, 10e-6, 633e-9
    geom_ap = element.ClearAperture.field()
    car = carrier.Carrier.grid_phase((n, n), (d, d), geom_ap, (0.0, 0.0), -10.0, 10.0)

    def build(v, lam_):
        des = car.build(v, lam_)
        return des

    car2 = carrier.Carrier.analytic(n * n, -10.0, 10.0, lambda v, lam_: _design(v, lam_, n, d))
    rng = np.random.default_rng(3)
    target = rng.uniform(0, 1, (n, n))
    src = lambda x0, y0, lam_: chirp_band(n, d, lam_, 1e8)
    rend = observe.Renderer(car2, src, bands=[lam], asm_cfg=asm.AsmConfig(1.0, False, False, 1.0))
    m = merit.MseToTarget(target)
    vals = rng.uniform(-1, 1, n * n)
    g = adjoint.grid_gradient(rend, vals, m)[0].reshape(-1)
    h = 1e-5
    fd = np.empty(n * n)
    for i in range(n * n):
        vp = vals.copy(); vp[i] += h
        vm = vals.copy(); vm[i] -= h
        fd[i] = (m.evaluate(rend.render(vp)) - m.evaluate(rend.render(vm))) / (2 * h)
    assert np.max(np.abs(g - fd)) / np.max(np.abs(fd)) < 1e-4


def _design(v, lam, n, d):
    des = carrier.Design()
    mask = element.PhaseMask.sampled(v, (n, n), (d, d))
    des.push(mask, 2e-4)
    des.push(element.ThinLens.fixed(0.05), 1e-4)
    return des


def test_hypercam_golden_forward_render():
    """crates/optics-inverse/tests/hypercam_forward.rs:89-207, rel 1e-6 of peak."""
    meta = {}
    for line in (GOLDEN / "hypercam/meta.txt").read_text().splitlines():
        line = line.strip()
        if line and not line.startswith("#"):
            k, v = line.split("=", 1)
            meta[k] = float(v)
    n = int(meta["n"])
    pitch, lam, index = meta["pitch"], meta["lambda"], meta["index"]
    z_gap, f, ap_r, w0, h = meta["z_gap"], meta["f_relay"], meta["aperture_r"], meta["w0"], meta["h_scene"]
    thick = np.load(GOLDEN / "hypercam/thickness.npy")
    ref = np.load(GOLDEN / "hypercam/forward.npy")

    def build(v, lam_):
        scale = 2.0 * math.pi * (index - 1.0) / lam_
        mask = element.PhaseMask.sampled(scale * v, (n, n), (pitch, pitch))
        lens = lambda: element.ThinLens.fixed(f, None, element.ClearAperture.circle(ap_r))
        des = carrier.Design()
        des.gap(z_gap)
        des.push(mask, f)
        des.push(lens(), 2 * f)
        des.push(lens(), f)
        return des

    car = carrier.Carrier.analytic(n * n, 0.0, meta["t_max"], build)
    src = lambda x0, y0, lam_: field.gaussian(w0, 1.0, (x0, y0), 0.0, lam_, n, n, pitch, pitch)
    rend = observe.Renderer(car, src, bands=[lam],
                            scenes=[(0.0, 0.0), (h, 0.0), (-h, 0.0), (0.0, h), (0.0, -h)],
                            asm_cfg=asm.AsmConfig(1.0, False, False, 1.0, 1.0),
                            deriv_x=True, deriv_y=True, scene_step=h)
    obs = rend.render(thick.reshape(-1))
    assert obs.data.shape == ref.shape
    rel = np.max(np.abs(obs.data - ref)) / np.max(np.abs(ref))
    assert rel < 1e-6, rel


# ---- merit.rs / fd.rs restatements -------------------------------------------

def test_encircled_energy_gradient_is_derivative_of_merit():
    """merit.rs:214-244: obs_gradient is dM/dI of evaluate (central differences)."""
    rng = np.random.default_rng(4)
    data = rng.uniform(0.1, 1.0, (1, 2, 1, 8, 8))
    obs = observe.Observation(["intensity"], [5e-7, 6e-7], [(0, 0)], (8, 8), (1e-6, 1e-6), data)
    m = merit.EncircledEnergyMerit(2.5e-6)
    g = m.obs_gradient(obs)
    for idx in [(0, 0, 0, 3, 4), (0, 1, 0, 0, 0), (0, 1, 0, 7, 2)]:
        h = 1e-6
        dp = data.copy(); dp[idx] += h
        dm = data.copy(); dm[idx] -= h
        fd = (m.evaluate(observe.Observation(obs.channels, obs.bands, obs.scenes, obs.dims,
                                             obs.pitch, dp))
              - m.evaluate(observe.Observation(obs.channels, obs.bands, obs.scenes, obs.dims,
                                               obs.pitch, dm))) / (2 * h)
        assert g[idx] == pytest.approx(fd, rel=1e-6, abs=1e-12)


def test_adam_first_step_by_hand():
    """fd.rs:217-235 at t = 1: m^ = g, v^ = g^2, so x -= lr_frac span g / (|g| + eps)."""
    x = np.array([1.0, 2.0, 3.0])
    g = np.array([0.3, -0.4, 0.0])  # |g| = 0.5 < clip 1.0
    xo, m, v = adam.adam_step(x, g, np.zeros(3), np.zeros(3), 1, 0.0, 4.0, lr_frac=0.1)
    step = 0.1 * 4.0 * g / (np.abs(g) + 1e-8)
    np.testing.assert_allclose(xo, x - step, rtol=1e-12)
    # |10 g| = 5 > clip 1: g is rescaled to 2 g before the moments
    xc, _, _ = adam.adam_step(x, g * 10, np.zeros(3), np.zeros(3), 1, 0.0, 4.0, lr_frac=0.1)
    np.testing.assert_allclose(xc, x - 0.1 * 4.0 * (2 * g) / (np.abs(2 * g) + 1e-8), rtol=1e-12)


# ---- analysis.rs restatement ---------------------------------------------------

def _gaussian_psf(w, n, d):
    c = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * d
    return np.exp(-(c[None, :] ** 2 + c[:, None] ** 2) / (w * w))


def test_analysis_encircled_energy_of_airy():
    """analysis.rs:444-474: EE(r1) = 0.84 +- 0.02 at the first dark ring."""
    from oracle import analysis, fraunhofer
    lam, a, z = 500e-9, 0.5e-3, 0.5
    band = field.uniform(1.0, 0.0, 128, 128, 50e-6, 50e-6, lam)
    masked = element.EllipticalAperture.circle(a).apply(band)
    far = fraunhofer.propagate(masked, z, fraunhofer.FraunhoferConfig(aperture_extent=a))
    psf = np.abs(far.samples) ** 2
    ee = analysis.encircled_energy(psf, (far.dx, far.dy))
    r1 = 1.22 * lam * z / (2.0 * a)
    assert abs(ee.value_at(r1) - 0.84) < 0.02, ee.value_at(r1)
    assert ee.radius_for_fraction(1.0) == pytest.approx(float(ee.radii[-1]))


def test_analysis_gaussian_anchors_and_strehl():
    """analysis.rs:475-505: spot RMS = w (1 %), MTF = exp(-pi^2 w^2 f^2) (0.02 below
    0.8 f_nyq), Strehl of a PSF with itself 1, wide vs narrow in (0.2, 0.6),
    Marechal bounds."""
    from oracle import analysis
    w, d = 100e-6, 10e-6
    psf = _gaussian_psf(w, 512, d)
    assert abs(analysis.spot_rms_radius(psf, (d, d)) / w - 1.0) < 0.01
    freqs, vals = analysis.mtf(psf, (d, d))
    assert abs(vals[0] - 1.0) < 1e-12
    err = max(abs(v - math.exp(-math.pi ** 2 * w * w * f * f))
              for f, v in zip(freqs[1:], vals[1:]) if f <= 800e3)
    assert err < 0.02
    narrow, wide = _gaussian_psf(80e-6, 256, 10e-6), _gaussian_psf(160e-6, 256, 10e-6)
    assert abs(analysis.strehl(narrow, (d, d), narrow, (d, d)) - 1.0) < 1e-12
    s = analysis.strehl(wide, (d, d), narrow, (d, d))
    assert 0.2 < s < 0.6
    assert 0.67 < analysis.marechal_strehl(0.1) < 0.68
    assert analysis.marechal_strehl(0.0) == 1.0


# ---- merit.rs built-ins over the analysis metrics -----------------------------

def _merit_obs(frame, pitch=10e-6, bands=(500e-9,)):
    n = frame.shape[-1]
    data = np.asarray(frame, dtype=np.float64).reshape(1, len(bands), 1, n, n)
    return observe.Observation(["intensity"], list(bands), [(0.0, 0.0)], (n, n),
                               (pitch, pitch), data, (1e-6, 1e-9))


def _merit_gaussian(n):
    """merit.rs:427-438: exp(-2 rho^2 / w^2), w = n 10 um / 6."""
    w = n * 10e-6 / 6.0
    c = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * 10e-6
    return np.exp(-2.0 * (c[None, :] ** 2 + c[:, None] ** 2) / (w * w))


def test_spot_strehl_mtf_merits_match_analysis():
    """merit.rs:474-520 and 556-576: SpotRmsMerit = spot_rms_radius (1e-9),
    StrehlMerit of a frame against itself = -1 (1e-12), MtfMerit at the fifth
    MTF bin = -mtf (2e-3)."""
    from oracle import analysis
    frame = _merit_gaussian(32)
    obs = _merit_obs(frame)
    want = analysis.spot_rms_radius(frame, (10e-6, 10e-6))
    got = merit.SpotRmsMerit().evaluate(obs)
    assert abs(got - want) / want < 1e-9
    assert abs(merit.StrehlMerit(frame).evaluate(obs) + 1.0) < 1e-12
    freqs, vals = analysis.mtf(frame, (10e-6, 10e-6))
    assert abs(merit.MtfMerit(freqs[4]).evaluate(obs) + vals[4]) < 2e-3
    assert merit.StrehlMerit(frame).obs_gradient(obs) is None
    assert merit.MtfMerit(freqs[4]).obs_gradient(obs) is None


def test_spot_rms_merit_gradient_fd():
    """merit.rs:522-554: the analytic obs gradient against central differences
    (eps 1e-9) at samples 0, 68, 255 of a 16 x 16 Gaussian frame."""
    frame = _merit_gaussian(16)
    obs = _merit_obs(frame)
    m = merit.SpotRmsMerit()
    g = m.obs_gradient(obs).reshape(-1)
    eps = 1e-9
    for k in (0, 68, 255):
        up, dn = frame.copy().reshape(-1), frame.copy().reshape(-1)
        up[k] += eps
        dn[k] -= eps
        fd = (m.evaluate(_merit_obs(up.reshape(16, 16)))
              - m.evaluate(_merit_obs(dn.reshape(16, 16)))) / (2 * eps)
        assert abs(fd - g[k]) < 1e-4 * (abs(fd) + 1.0), (k, fd, g[k])


def test_merit_selector_and_errors():
    """merit.rs:578-600: a selector over two bands sums them; an out-of-range band
    and an off-bin or super-Nyquist MTF frequency are errors; a dark frame
    gives 0 and no spot gradient."""
    ones = np.ones((2, 4, 4))
    obs = _merit_obs(ones, bands=(450e-9, 550e-9))
    assert merit.SpotRmsMerit().evaluate(obs) == pytest.approx(
        merit.SpotRmsMerit(band=0).evaluate(obs), rel=1e-15)
    with pytest.raises(ValueError):
        merit.SpotRmsMerit(band=5).evaluate(obs)
    with pytest.raises(ValueError):
        merit.MtfMerit(0.6 / 10e-6).evaluate(obs)  # above Nyquist
    with pytest.raises(ValueError):
        merit.MtfMerit(1.5 / (4 * 10e-6)).evaluate(obs)  # between bins
    dark = _merit_obs(np.zeros((4, 4)))
    assert merit.SpotRmsMerit().evaluate(dark) == 0.0
    assert merit.SpotRmsMerit().obs_gradient(dark) is None
    assert merit.StrehlMerit(np.ones(16)).evaluate(dark) == 0.0
    assert merit.MtfMerit(0.0).evaluate(dark) == 0.0
