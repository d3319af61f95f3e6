"""The reference's unit and golden tests restated against the oracle (CPU;
pins the oracle to the reference's known answers): the Fresnel, Fraunhofer
and Rayleigh-Sommerfeld engine tests, the ASM Airy test, element tests
(lens, ramp, blaze, wedge, rotated stop, sag), the Gaussian source and
field tests, the element-transmission probe, the Gerchberg-Saxton convention
pins and golden tests, the carrier tests, the renderer tests and the
detector-metric safety test.  The field and ASM-analysis tests also check
the product's host side (BandField validation, the C library's padded
sizes, band limits and phase steps).

Each test cites the test it restates (src/propagation/fresnel.rs,
fraunhofer.rs, rayleigh_sommerfeld.rs, src/element.rs, src/sources.rs,
src/field.rs, src/analysis.rs, tests/asm.rs, or
crates/optics-inverse/src/adjoint.rs, carrier.rs, gs.rs, observe.rs) and
keeps its geometry and tolerance.
"""

import math

import numpy as np
import pytest

from oracle import field as ofield, fraunhofer as ofh, fresnel as ofr, rs as ors
from oracle import element as oel

LAMBDA = 500e-9


def uniform(a, n, d):
    return ofield.uniform(a, 0.0, n, n, d, d, LAMBDA)


def gaussian(n, d, sigma, c=(0.0, 0.0)):
    x = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * d - c[0]
    y = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * d - c[1]
    u = np.exp(-(x[None, :] ** 2 + y[:, None] ** 2) / (2.0 * sigma * sigma))
    return ofield.BandField(u.astype(np.complex128), d, d, LAMBDA)


def power(b):
    return float(np.sum(np.abs(b.samples) ** 2)) * b.dx * b.dy


# ---- src/propagation/fresnel.rs ---------------------------------------------------

def test_fresnel_closed_form_step_is_the_sweep_maximum():
    """fresnel.rs closed_form_step_is_the_exact_sweep_maximum."""
    nx_pad, ny_pad, d, z = 12, 8, 2e-6, 0.037
    fx = np.fft.fftfreq(nx_pad, d)
    fy = np.fft.fftfreq(ny_pad, d)
    ph = -math.pi * LAMBDA * z * (fx[None, :] ** 2 + fy[:, None] ** 2)
    sweep = float(np.max(np.abs(ph - np.roll(ph, -1, axis=1))))
    assert abs(sweep - ofr.worst_axis_step(nx_pad, d, LAMBDA, z)) < 1e-9


def test_fresnel_z_zero_and_invalid_inputs():
    """fresnel.rs z_zero_is_identity, convolution_z_zero_is_identity,
    invalid_inputs_rejected."""
    b = uniform(1.5, 16, 20e-6)
    np.testing.assert_array_equal(ofr.propagate(b, 0.0).samples, b.samples)
    b2 = uniform(2.0, 16, 20e-6)
    np.testing.assert_array_equal(ofr.propagate_convolution(b2, 0.0).samples, b2.samples)
    small = uniform(1.0, 8, 20e-6)
    with pytest.raises(ofr.FresnelError) as e:
        ofr.propagate(small, math.inf)
    assert e.value.variant == "InvalidDistance"
    with pytest.raises(ofr.FresnelError) as e:
        ofr.propagate_convolution(small, math.nan)
    assert e.value.variant == "InvalidDistance"


def test_fresnel_plane_wave_bins_pick_up_exact_quadratic_phase():
    """fresnel.rs plane_wave_bins_pick_up_exact_quadratic_phase."""
    n, d, z, m = 32, 20e-6, 1e-3, 2.0
    alpha = m * LAMBDA / (n * d)
    b = ofield.plane_wave(math.asin(alpha), 0.0, 1.0, n, n, d, d, LAMBDA)
    out = ofr.propagate(b, z, ofr.FresnelConfig(1.0, False, 1.0))
    k = 2.0 * math.pi / LAMBDA
    fx = m / (n * d)
    want = np.exp(1j * (k * z - math.pi * LAMBDA * z * fx * fx))
    for iy in (0, 16, 31):
        assert abs(out.samples[iy, 10] / b.samples[iy, 10] - want) < 1e-9


def test_fresnel_round_trip_on_periodic_grid_is_exact():
    """fresnel.rs round_trip_on_periodic_grid_is_exact."""
    b = uniform(1.0, 16, 20e-6)
    cfg = ofr.FresnelConfig(1.0, False, 1.0)
    rt = ofr.propagate(ofr.propagate(b, 2e-3, cfg), -2e-3, cfg)
    assert float(np.max(np.abs(rt.samples - b.samples))) < 1e-9


def test_fresnel_strict_mode_flags_undersampled_chirp_and_mitigates():
    """fresnel.rs strict_mode_flags_undersampled_chirp_and_mitigates."""
    b = uniform(1.0, 32, 1e-6)
    z = 3e-4
    risk = ofr.FresnelConfig(1.0, True, 1.0)
    rep = ofr.sampling_report(b, z, risk)
    assert not rep.nyquist_ok and rep.max_phase_step_x > math.pi
    with pytest.raises(ofr.FresnelError) as e:
        ofr.propagate(b, z, risk)
    assert e.value.variant == "AliasingRisk"
    ofr.propagate(b, z, ofr.FresnelConfig(1.0, False, 1.0))
    fix = ofr.FresnelConfig(1.0, True, 8.0)
    assert not ofr.sampling_report(b, z, fix).nyquist_ok
    assert ofr.propagate(b, z, fix).samples.shape == b.samples.shape
    at8 = ofr.sampling_report(b, z, ofr.FresnelConfig(8.0, True, 8.0))
    assert at8.nyquist_ok and at8.max_phase_step_x < math.pi


def test_fresnel_paraxial_flag_tracks_grid_angular_extent():
    """fresnel.rs paraxial_flag_tracks_grid_angular_extent."""
    rep = ofr.sampling_report(uniform(1.0, 32, 1e-3), 0.1, ofr.FresnelConfig())
    assert rep.paraxial_ok and rep.max_phase_error_vs_asm < 0.01
    rep = ofr.sampling_report(uniform(1.0, 32, 1e-6), 0.05, ofr.FresnelConfig())
    assert not rep.paraxial_ok and rep.max_phase_error_vs_asm > 0.01


def test_fresnel_convolution_guard_is_reciprocal_to_transfer_guard():
    """fresnel.rs convolution_guard_is_reciprocal_to_transfer_guard."""
    b = uniform(1.0, 64, 1e-6)
    z = 5e-4
    cfg = ofr.FresnelConfig(1.0, True, 1.0)
    rep = ofr.sampling_report(b, z, cfg)
    assert rep.kernel_nyquist_ok and rep.max_kernel_step_x < math.pi
    assert not rep.nyquist_ok and rep.max_phase_step_x > math.pi
    ofr.propagate_convolution(b, z, cfg)
    with pytest.raises(ofr.FresnelError) as e:
        ofr.propagate(b, z, cfg)
    assert e.value.variant == "AliasingRisk"
    ofr.propagate(b, z, ofr.FresnelConfig(1.0, True, 8.0))


def test_fresnel_convolution_matches_tf_at_critical_sampling():
    """fresnel.rs convolution_matches_tf_at_critical_sampling: n d^2 = lambda z,
    the two forms agree within 1e-6."""
    n, z = 256, 2e-3
    d = math.sqrt(LAMBDA * z / n)
    b = gaussian(n, d, 50.0 * d)
    cfg = ofr.FresnelConfig(1.0, True, 1.0)
    rep = ofr.sampling_report(b, z, cfg)
    assert rep.nyquist_ok and rep.kernel_nyquist_ok
    tf = ofr.propagate(b, z, cfg).samples
    conv = ofr.propagate_convolution(b, z, cfg).samples
    assert np.linalg.norm(tf - conv) / np.linalg.norm(tf) < 1e-6


# ---- src/propagation/fraunhofer.rs ------------------------------------------------

def test_fraunhofer_uniform_input_concentrates_at_dc():
    """fraunhofer.rs uniform_input_concentrates_at_dc: |U(0)| = a (n d)^2 /
    (lambda z), every other bin below 1e-9."""
    n, d, z, a = 15, 2e-5, 4.0, 0.75
    out = ofh.propagate(ofield.uniform(a, 0.0, n, n, d, d, LAMBDA), z)
    mag = np.abs(out.samples).reshape(-1)
    c = (n // 2) * n + n // 2
    assert abs(mag[c] - a * (n * d) ** 2 / (LAMBDA * z)) < 1e-9
    assert float(np.max(np.delete(mag, c))) < 1e-9


def test_fraunhofer_power_regime_gate_and_mirror():
    """fraunhofer.rs far_field_power_equals_input_power,
    regime_gate_blocks_near_field_geometry, negative_z_mirrors_the_pattern,
    invalid_inputs_rejected."""
    n, d = 64, 1e-5
    b = gaussian(n, d, 5.0 * d)
    assert ofh.regime_report(b, 2.0, ofh.FraunhoferConfig()).regime_ok
    out = ofh.propagate(b, 2.0)
    assert abs(power(out) - power(b)) / power(b) < 1e-9
    with pytest.raises(ofh.FraunhoferError) as e:
        ofh.propagate(b, 0.01)
    assert e.value.variant == "RegimeViolation"
    assert not e.value.report.regime_ok and e.value.report.n_f_x > 1.0
    loose = ofh.FraunhoferConfig(strict=False)
    assert ofh.propagate(b, 0.01, loose).samples.shape == (n, n)
    assert not ofh.regime_report(b, 0.01, loose).regime_ok
    tight = ofh.FraunhoferConfig(max_n_f=0.05)
    assert not ofh.regime_report(b, 2.0, tight).regime_ok
    assert ofh.regime_report(b, 5.0, tight).regime_ok
    back = ofh.propagate(b, -2.0)
    assert float(np.max(np.abs(np.abs(out.samples) - np.abs(back.samples[::-1, ::-1])))) < 1e-12
    small = ofield.uniform(1.0, 0.0, 8, 8, 20e-6, 20e-6, LAMBDA)
    for z in (0.0, math.nan):
        with pytest.raises(ofh.FraunhoferError) as e:
            ofh.propagate(small, z, loose)
        assert e.value.variant == "InvalidDistance"


def test_fraunhofer_source_position_and_off_axis_power():
    """fraunhofer.rs source_pos_none_equals_explicit_origin,
    off_axis_propagation_conserves_power."""
    b = gaussian(64, 1e-5, 5e-5)
    a = ofh.propagate(b, 2.0, ofh.FraunhoferConfig(source_pos=None))
    o = ofh.propagate(b, 2.0, ofh.FraunhoferConfig(source_pos=(0.0, 0.0)))
    np.testing.assert_array_equal(a.samples, o.samples)
    s = (1e-4, -5e-5)
    cfg = ofh.FraunhoferConfig(source_pos=s)
    shifted = gaussian(64, 1e-5, 5e-5, s)
    assert ofh.regime_report(shifted, 2.0, cfg).regime_ok
    out_s = ofh.propagate(shifted, 2.0, cfg)
    assert abs(power(out_s) - power(shifted)) / power(shifted) < 1e-9
    assert abs(power(out_s) - power(a)) / power(a) < 1e-9


def test_fraunhofer_aperture_extent_declares_true_source_size():
    """fraunhofer.rs aperture_extent_declares_true_source_size."""
    b = gaussian(64, 1e-5, 2.0e-5)
    z = 0.05
    win = ofh.regime_report(b, z, ofh.FraunhoferConfig())
    assert not win.regime_ok and not win.extent_is_aperture
    with pytest.raises(ofh.FraunhoferError) as e:
        ofh.propagate(b, z)
    assert e.value.variant == "RegimeViolation"
    cfg = ofh.FraunhoferConfig(aperture_extent=1e-4)
    rep = ofh.regime_report(b, z, cfg)
    assert rep.regime_ok and rep.extent_is_aperture
    assert abs(rep.extent_used - 1e-4) < 1e-15
    assert abs(rep.n_f_x - 0.4) < 1e-9
    assert ofh.propagate(b, z, cfg).samples.shape == (64, 64)
    with pytest.raises(ofh.FraunhoferError) as e:
        ofh.propagate(b, z, ofh.FraunhoferConfig(aperture_extent=0.0))
    assert e.value.variant == "RegimeViolation"


# ---- src/propagation/rayleigh_sommerfeld.rs ---------------------------------------

def _dft_coord(i, n, d):
    return (i if i <= n // 2 else i - n) * d


def test_rs_kernel_reduces_to_fresnel_paraxially_and_conjugates_for_minus_z():
    """rayleigh_sommerfeld.rs kernel_reduces_to_fresnel_paraxially (1e-6),
    negative_z_kernel_is_conjugate (exact)."""
    n, d, z = 64, 10e-6, 5.0
    k = 2.0 * math.pi / LAMBDA
    worst = 0.0
    for iy in (0, 16, 31, 32, 48, 63):
        for ix in (0, 16, 31, 32, 48, 63):
            x, y = _dft_coord(ix, n, d), _dft_coord(iy, n, d)
            rs = complex(ors.kernel_value(x, y, LAMBDA, z))
            fr = (complex(math.cos(k * z), math.sin(k * z)) / (1j * LAMBDA * z)
                  * np.exp(1j * math.pi * (x * x + y * y) / (LAMBDA * z)))
            worst = max(worst, abs(rs / fr - 1.0))
    assert worst < 1e-6
    fwd = ors.impulse_response(32, 32, 10e-6, 10e-6, LAMBDA, 2e-3)
    bwd = ors.impulse_response(32, 32, 10e-6, 10e-6, LAMBDA, -2e-3)
    np.testing.assert_array_equal(bwd, np.conj(fwd))


def test_rs_engine_agrees_with_asm_on_smooth_band():
    """rayleigh_sommerfeld.rs engine_agrees_with_asm_on_smooth_band (5e-2)."""
    from oracle import asm as oasm
    b = gaussian(200, 2e-6, 30e-6)
    cfg = ors.RayleighSommerfeldConfig(2.0, True)
    assert ors.sampling_report(b, 5e-3, cfg).kernel_nyquist_ok
    rs = ors.propagate(b, 5e-3, cfg).samples
    asm = oasm.propagate(b, 5e-3, oasm.AsmConfig(padding=2.0)).samples
    assert np.linalg.norm(rs - asm) / np.linalg.norm(asm) < 5e-2


def test_rs_kernel_step_closed_form_brackets_sweep():
    """rayleigh_sommerfeld.rs kernel_step_closed_form_brackets_sweep."""
    n, d, z = 64, 2e-6, 3e-4
    k = 2.0 * math.pi / LAMBDA
    c = np.array([_dft_coord(i, n, d) for i in range(n)])
    r = np.sqrt(c[None, :] ** 2 + c[:, None] ** 2 + z * z)
    ph = k * r - np.arctan(k * r)
    sweep = float(np.max(np.abs(ph - np.roll(ph, -1, axis=1))))
    closed = ors.worst_kernel_axis_step(n, d, LAMBDA, z)
    assert sweep <= closed + 1e-12
    assert closed < 2.0 * sweep + 1e-12


def test_rs_strict_guard_invalid_inputs_and_back_propagation():
    """rayleigh_sommerfeld.rs strict_guard_raises_immediately_and_padding_worsens_it,
    z_zero_and_invalid_inputs_rejected, back_propagation_inverts_on_smooth_band."""
    b = uniform(1.0, 64, 10e-6)
    cfg = ors.RayleighSommerfeldConfig(1.0, True)
    rep = ors.sampling_report(b, 1e-3, cfg)
    assert not rep.kernel_nyquist_ok and rep.max_kernel_step_x > math.pi
    with pytest.raises(ors.RayleighSommerfeldError) as e:
        ors.propagate(b, 1e-3, cfg)
    assert e.value.variant == "AliasingRisk"
    rep4 = ors.sampling_report(b, 1e-3, ors.RayleighSommerfeldConfig(4.0, True))
    assert rep4.max_kernel_step_x > rep.max_kernel_step_x
    ors.propagate(b, 1e-3, ors.RayleighSommerfeldConfig(1.0, False))
    ok = ors.sampling_report(b, 0.5, ors.RayleighSommerfeldConfig(2.0, True))
    assert ok.kernel_nyquist_ok and ok.paraxial_ok
    small = uniform(1.0, 8, 20e-6)
    for z in (0.0, math.inf, math.nan):
        with pytest.raises(ors.RayleighSommerfeldError) as e:
            ors.propagate(small, z)
        assert e.value.variant == "InvalidDistance"
    g = gaussian(128, 10e-6, 80e-6)
    cfg2 = ors.RayleighSommerfeldConfig(2.0, True)
    rep = ors.sampling_report(g, 0.2, cfg2)
    assert rep.kernel_nyquist_ok and rep.paraxial_ok
    rt = ors.propagate(ors.propagate(g, 0.2, cfg2), -0.2, cfg2).samples
    assert np.linalg.norm(rt - g.samples) / np.linalg.norm(g.samples) < 1e-2


# ---- crates/optics-inverse/src/gs.rs ----------------------------------------------

def _gs_asm(n, d, z_total, lam=LAMBDA):
    """gs.rs tests' asm_plain (no band limit, not strict): half transforms of
    z_total / 2 and the back-propagation."""
    from oracle import asm as oasm
    cfg = oasm.AsmConfig(band_limited=False, strict=False)
    half = z_total / 2.0
    fwd = lambda s: oasm.propagate(ofield.BandField(s, d, d, lam), half, cfg).samples
    back = lambda s: oasm.propagate(ofield.BandField(s, d, d, lam), -half, cfg).samples
    return fwd, back


def _mse_merit(target):
    tint = target * target  # gs.rs tests' mse_merit: MseToTarget on the squared target
    return lambda inten: float(np.sum((inten - tint) ** 2) / inten.size)


def test_gs_golden_lens_phase_recovered_from_target_intensity():
    """gs.rs golden_lens_phase_recovered_from_target_intensity (zero start, so
    fully deterministic): a 150 um lens aperture, f = 12 mm; GS over 2 f
    brings the merit below 0.1 of the first and recovers the lens phase
    (cos-score > 0.9 inside 0.9 of the radius)."""
    from oracle import gs as ogs
    n, d, f, radius = 128, 5e-6, 12e-3, 150e-6
    k = 2.0 * math.pi / LAMBDA
    c = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * d
    r2 = c[None, :] ** 2 + c[:, None] ** 2
    true_phase = ogs.wrap_pi(-k * r2 / (2.0 * f))
    inside = r2 <= radius * radius
    mask = np.where(inside, np.exp(1j * true_phase), 0.0)
    from oracle import asm as oasm
    u_true = oasm.propagate(ofield.BandField(mask, d, d, LAMBDA), f,
                            oasm.AsmConfig(band_limited=False, strict=False)).samples
    target = np.abs(u_true)
    u_in = ofield.plane_wave(0.0, 0.0, 1.0, n, n, d, d, LAMBDA).samples
    fwd, back = _gs_asm(n, d, 2.0 * f)
    sol = ogs.run(u_in, inside, target, -math.pi, math.pi, np.zeros((n, n)), fwd, back,
                  _mse_merit(target), max_iterations=60, patience=10, merit_tolerance=1e-5)
    first = sol.history[0].merit
    assert sol.merit < 0.1 * max(first, 1e-30)
    sel = r2 <= (0.9 * radius) ** 2
    diff = ogs.wrap_pi(np.asarray(sol.phase).reshape(n, n)[sel] - true_phase[sel])
    assert float(np.mean(np.cos(diff - diff.mean()))) > 0.9


def test_gs_golden_tophat_shaper_is_flat_and_best_merit_monotone():
    """gs.rs golden_tophat_shaper_is_flat_and_mse_monotone: a 150 um Gaussian
    shaped into a 250 um disk over 8 mm: best-so-far merit monotone, final
    merit below half the first, interior (0.7 r) coefficient of variation
    below 0.35.  The reference starts from rand's StdRng (seed 7), which only
    Rust reproduces; a seeded uniform start in [-pi, pi) stands in."""
    from oracle import gs as ogs
    n, d, z_total, target_r = 128, 8e-6, 8e-3, 250e-6
    u_in = ofield.gaussian(150e-6, 1.0, (0.0, 0.0), 0.0, LAMBDA, n, n, d, d).samples
    c = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * d
    r2 = c[None, :] ** 2 + c[:, None] ** 2
    disk = r2 <= target_r * target_r
    amp = math.sqrt(float(np.sum(np.abs(u_in) ** 2)) / float(np.sum(disk)))
    target = np.where(disk, amp, 0.0)
    init = np.random.default_rng(7).uniform(-math.pi, math.pi, (n, n))
    fwd, back = _gs_asm(n, d, z_total)
    sol = ogs.run(u_in, np.ones((n, n), bool), target, -math.pi, math.pi, init, fwd, back,
                  _mse_merit(target), max_iterations=120, patience=10, merit_tolerance=1e-4)
    best = [r.best_merit for r in sol.history]
    assert all(b1 <= b0 + 1e-15 for b0, b1 in zip(best, best[1:]))
    assert sol.merit < 0.5 * sol.history[0].merit
    v = np.asarray(sol.target_intensity).reshape(n, n)[r2 <= (0.7 * target_r) ** 2]
    assert float(np.std(v) / np.mean(v)) < 0.35
    assert all(math.isfinite(r.target_error_rms) and math.isfinite(r.phase_update_rms)
               for r in sol.history)


# ---- crates/optics-inverse/src/observe.rs -----------------------------------------

def _obs_mods():
    from oracle import asm as oasm, carrier as ocar, element as oel, observe as oobs
    return oasm, ocar, oel, oobs


def _gauss_src(w0, n=64, d=10e-6):
    return lambda x0, y0, lam: ofield.gaussian(w0, 1.0, (x0, y0), 0.0, lam, n, n, d, d)


def _plane_src(n=64, d=10e-6):
    return lambda x0, y0, lam: ofield.plane_wave(0.0, 0.0, 1.0, n, n, d, d, lam)


def _relay_carrier(dist, n_idx):
    """observe.rs relay_carrier: defocus -d, a uniform phase 2 pi (n - 1) h /
    lambda, refocus +d."""
    oasm, ocar, oel, _ = _obs_mods()

    def build(v, lam):
        phase = 2.0 * math.pi * (n_idx - 1.0) * v[0] / lam
        d = ocar.Design()
        d.gap(-dist, 1.0)
        d.push(oel.PhaseMask.sampled(np.full(64 * 64, phase), (64, 64), (10e-6, 10e-6)), 0.0, 1.0)
        d.gap(dist, 1.0)
        return d
    return ocar.Carrier.analytic(1, 0.0, 20e-6, build)


def test_observe_piston_chain_zero_xy_channels_and_round_trip():
    """observe.rs defocus_mask_defocus_chain_is_pure_piston (1e-6 of peak),
    plane_wave_x_y_channels_are_exactly_zero, round_trip_propagation_preserves_gaussian
    (power and overlap within 1e-6)."""
    oasm, ocar, oel, oobs = _obs_mods()
    plain = oasm.AsmConfig(band_limited=False, strict=False)
    r = oobs.Renderer(_relay_carrier(5e-3, 1.5), _gauss_src(80e-6), asm_cfg=plain)
    obs = r.render(np.array([2e-6]))
    i_in = np.abs(_gauss_src(80e-6)(0.0, 0.0, LAMBDA).samples) ** 2
    assert float(np.max(np.abs(obs.data[0, 0, 0] - i_in))) < 1e-6 * float(np.max(i_in))
    r = oobs.Renderer(_relay_carrier(5e-3, 1.5), _plane_src(), deriv_x=True, deriv_y=True)
    obs = r.render(np.array([2e-6]))
    assert np.all(obs.data[1:, 0, 0] == 0.0)
    d = ocar.Design()
    d.gap(2e-3, 1.0)
    d.gap(-2e-3, 1.0)
    u = _gauss_src(100e-6)(0.0, 0.0, LAMBDA)
    out = d.beamline().trace(u, lambda b, z, m: oasm.propagate(
        b, z, oasm.AsmConfig(band_limited=False, strict=False, medium=m)))
    s_in = float(np.sum(np.abs(u.samples) ** 2))
    s_out = float(np.sum(np.abs(out.samples) ** 2))
    assert abs(s_out / s_in - 1.0) < 1e-6
    ip = abs(np.sum(u.samples * np.conj(out.samples)))
    assert abs(ip / math.sqrt(s_in * s_out) - 1.0) < 1e-6


def test_observe_dx_channel_matches_translation_invariance():
    """observe.rs dx_channel_matches_translation_invariance: after a 3 mm gap
    dI/dx0 = -dI/dx (five-point stencil), within 0.02 of peak / w0 over the
    pixels above 2 % of the peak."""
    oasm, ocar, oel, oobs = _obs_mods()

    def build(v, lam):
        d = ocar.Design()
        d.gap(3e-3, 1.0)
        return d
    r = oobs.Renderer(ocar.Carrier.analytic(0, 0.0, 1.0, build), _gauss_src(80e-6),
                      asm_cfg=oasm.AsmConfig(band_limited=False, strict=False), deriv_x=True,
                      scene_step=1e-6)
    obs = r.render(np.zeros(0))
    i, dx = obs.data[0, 0, 0], obs.data[1, 0, 0]
    peak = float(np.max(i))
    scale = peak / 80e-6
    gx = (i[:, :-4] - 8.0 * i[:, 1:-3] + 8.0 * i[:, 3:-1] - i[:, 4:]) / (12.0 * obs.pitch[0])
    core = i[1:-1, 2:-2] >= 0.02 * peak
    err = np.abs(dx[1:-1, 2:-2] + gx[1:-1]) / scale
    assert int(np.sum(core)) > 100
    assert float(np.max(err[core])) < 0.02


def test_observe_lambda_channel_detects_chromatic_focus():
    """observe.rs lambda_channel_detects_chromatic_focus: a diffractive lens
    (f = f0 lambda0 / lambda, 300 um stop) at f0: max |dI/dlambda| at the
    middle band exceeds 1e5 times that band's peak intensity."""
    oasm, ocar, oel, oobs = _obs_mods()
    lam0, f0 = 500e-9, 50e-3

    def build(v, lam):
        f = v[0] * lam0 / lam
        d = ocar.Design()
        d.push(oel.ThinLens(lambda _l: f, None, oel.ClearAperture.circle(300e-6)), v[0], 1.0)
        return d
    r = oobs.Renderer(ocar.Carrier.analytic(1, 0.01, 1.0, build), _plane_src(128),
                      bands=[450e-9, 500e-9, 550e-9], deriv_lambda=True, lambda_step=5e-9,
                      asm_cfg=oasm.AsmConfig(band_limited=False, strict=False))
    obs = r.render(np.array([f0]))
    assert float(np.max(np.abs(obs.data[1, 1, 0]))) > 1.0e5 * float(np.max(obs.data[0, 1, 0]))


def test_observe_layout_and_rejections():
    """observe.rs observation_layout_is_contiguous_frames,
    renderer_rejects_empty_axes_and_bad_steps (observe.rs:214-230)."""
    oasm, ocar, oel, oobs = _obs_mods()
    car = _relay_carrier(5e-3, 1.5)
    r = oobs.Renderer(car, _plane_src(), bands=[450e-9, 550e-9],
                      scenes=[(0.0, 0.0), (20e-6, 0.0)], deriv_x=True, deriv_lambda=True)
    obs = r.render(np.array([1e-6]))
    assert obs.data.shape == (3, 2, 2, 64, 64)
    assert obs.channels[1:] == [oobs.DX, oobs.DLAMBDA]
    assert obs.channel_index(oobs.DY) is None
    for kw in ({"bands": []}, {"scenes": []}, {"deriv_x": True, "scene_step": 0.0},
               {"deriv_y": True, "scene_step": math.nan},
               {"deriv_lambda": True, "lambda_step": -1e-9}):
        with pytest.raises(ocar.InverseError):
            oobs.Renderer(car, _plane_src(), **kw).render(np.array([1e-6]))


def _plain(u, n, d, z):
    from oracle import asm as oasm
    return oasm.propagate(ofield.BandField(u, d, d, LAMBDA), z,
                          oasm.AsmConfig(band_limited=False, strict=False)).samples


def test_gs_convention_pins():
    """gs.rs asm_roundtrip_is_identity (1e-9), two_half_transforms_compose_to_full_transform
    (1e-6 of the mean modulus), converging_lens_phase_focuses_at_positive_z (peak
    above 5x the bare propagation, centroid within 10 um of the axis),
    blaze_phase_steers_spot_to_positive_x (centroid at lambda z / period within 15 %)."""
    n, d, z = 64, 10e-6, 2e-3
    g = ofield.gaussian(60e-6, 1.0, (0.0, 0.0), 0.0, LAMBDA, n, n, d, d).samples
    back = _plain(_plain(g, n, d, z), n, d, -z)
    assert float(np.max(np.abs(back - g))) < 1e-9
    full = _plain(g, n, d, 2.0 * z)
    half = _plain(_plain(g, n, d, z), n, d, z)
    assert float(np.max(np.abs(full - half))) < 1e-6 * float(np.mean(np.abs(full)))

    n, d, f = 128, 5e-6, 12e-3
    k = 2.0 * math.pi / LAMBDA
    c = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * d
    r2 = c[None, :] ** 2 + c[:, None] ** 2
    pw = ofield.plane_wave(0.0, 0.0, 1.0, n, n, d, d, LAMBDA).samples
    focused = _plain(pw * np.exp(-1j * k * r2 / (2.0 * f)), n, d, f)
    bare = _plain(pw, n, d, f)
    w = np.abs(focused) ** 2
    assert float(np.max(w)) > 5.0 * float(np.max(np.abs(bare) ** 2))
    assert abs(float(np.sum(w * c[None, :])) / float(np.sum(w))) < 10e-6

    z, period = 4e-3, 60e-6
    gb = ofield.gaussian(120e-6, 1.0, (0.0, 0.0), 0.0, LAMBDA, n, n, d, d).samples
    out = _plain(gb * np.exp(1j * 2.0 * math.pi * c[None, :] / period), n, d, z)
    w = np.abs(out) ** 2
    shift = float(np.sum(w * c[None, :])) / float(np.sum(w))
    want = LAMBDA * z / period
    assert abs(shift - want) < 0.15 * want


# ---- tests/asm.rs -----------------------------------------------------------------

def test_asm_airy_pattern_far_field():
    """tests/asm.rs airy_pattern_far_field: a 1 mm circular aperture on a 1536^2
    grid (20 um) propagated 40 m by ASM; the ring-binned profile (bins of 2 dx)
    follows [2 J1(v)/v]^2 within 2 % of the on-axis value out to 12.6 mm and the
    first zero lies within 2 % of 1.22 lambda z / 2a."""
    from scipy import special
    from oracle import asm as oasm, element as oel
    n, dx, a, z = 1536, 20e-6, 1.0e-3, 40.0
    band = ofield.uniform(1.0, 0.0, n, n, dx, dx, LAMBDA)
    far = oasm.propagate(oel.EllipticalAperture.circle(a).apply(band), z)
    dr, r_max = 2.0 * dx, 12.6e-3
    nbins = int(r_max / dr)
    c = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * dx
    r = np.sqrt(c[None, :] ** 2 + c[:, None] ** 2)
    b = (r / dr).astype(np.int64).reshape(-1)
    keep = b < nbins
    i = (np.abs(far.samples) ** 2).reshape(-1)
    prof = (np.bincount(b[keep], weights=i[keep], minlength=nbins)
            / np.maximum(np.bincount(b[keep], minlength=nbins), 1))
    i0 = float(np.mean(prof[:3]))
    rc = (np.arange(nbins) + 0.5) * dr
    v = 2.0 * math.pi / LAMBDA * a * rc / z
    airy = (2.0 * special.j1(v) / v) ** 2
    sel = rc <= r_max - dr
    assert float(np.max(np.abs(prof[sel] / i0 - airy[sel]))) <= 0.02
    r1 = 1.22 * LAMBDA * z / (2.0 * a)
    lo, hi = int(8.0e-3 / dr), int(12.4e-3 / dr)
    bm = lo + int(np.argmin(prof[lo:hi]))
    y0, ym, y1 = prof[bm - 1], prof[bm], prof[bm + 1]
    d2 = y0 - 2.0 * ym + y1
    frac = 0.5 * (y0 - y1) / d2 if d2 != 0.0 else 0.0
    r_zero = (bm + min(max(frac, -0.5), 0.5)) * dr
    assert abs(r_zero - r1) / r1 <= 0.02


# ---- crates/optics-inverse/src/adjoint.rs -----------------------------------------

def _chirp(n, d):
    """adjoint.rs tests' chirp_field: a Gaussian envelope (60 um) with a tilt and
    a quadratic phase."""
    c = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * d
    x, y = c[None, :], c[:, None]
    r2 = x * x + y * y
    ph = 3.7 * x / 1e-3 + 2.1 * y / 1e-3 + 9.0e6 * r2
    return ofield.BandField(np.exp(-r2 / (2.0 * 60e-6 ** 2)) * np.exp(1j * ph), d, d, LAMBDA)


def test_adjoint_element_transmission_probe_and_identity():
    """adjoint.rs element_transmission_probe_and_adjoint_identity: the probe of a
    sampled phase mask behind a 120 um stop is e^{i phase} inside, 0 outside
    (1e-12), equals apply(1), and <w, t d> = <conj(t) w, d> (1e-12)."""
    from oracle import element as oel
    n, d = 32, 10e-6
    phase = np.sin(np.arange(n * n, dtype=np.float64) * 0.37)
    mask = oel.PhaseMask.sampled(phase, (n, n), (d, d), None, oel.ClearAperture.circle(120e-6))
    like = _chirp(n, d)
    t = oel.transmission(mask, like)
    c = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * d
    inside = c[None, :] ** 2 + c[:, None] ** 2 <= 120e-6 ** 2
    want = np.where(inside, np.exp(1j * phase.reshape(n, n)), 0.0)
    assert float(np.max(np.abs(t - want))) < 1e-12
    ones = ofield.BandField(np.ones((n, n), complex), d, d, LAMBDA)
    np.testing.assert_array_equal(mask.apply(ones).samples, t)
    dvec, w = _chirp(n, d).samples, _chirp(n, d).samples
    lhs = np.vdot(w, t * dvec)
    rhs = np.vdot(np.conj(t) * w, dvec)
    assert abs(lhs - rhs) / abs(lhs) < 1e-12


# ---- src/element.rs ---------------------------------------------------------------

def _wrap(p):
    return (p + math.pi) % (2.0 * math.pi) - math.pi


def _xy(n, d):
    c = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * d
    return c[None, :], c[:, None]


def test_element_thin_lens_phase_and_diverging_conjugate():
    """element.rs phase_profile_is_the_negative_quadratic (|t| = 1 to 1e-12, phase
    -k r^2 / 2f to 1e-9), diverging_lens_conjugates_the_converging_phase (1e-12)."""
    from oracle import element as oel
    n, d, f = 128, 1e-5, 0.1
    band = ofield.uniform(2.0, 0.0, n, n, d, d, LAMBDA)
    out = oel.ThinLens.fixed(f).apply(band).samples
    k = 2.0 * math.pi / LAMBDA
    x, y = _xy(n, d)
    for ix, iy in ((0, 0), (63, 64), (127, 127), (10, 120)):
        s = out[iy, ix]
        assert abs(abs(s) - 2.0) < 1e-12
        want = -k * (x[0, ix] ** 2 + y[iy, 0] ** 2) / (2.0 * f)
        assert abs(_wrap(np.angle(s) - want)) < 1e-9
    b = ofield.uniform(1.0, 0.0, 64, 64, 1e-5, 1e-5, LAMBDA)
    conv = oel.ThinLens.fixed(0.1).apply(b).samples
    div = oel.ThinLens.fixed(-0.1).apply(b).samples
    assert float(np.max(np.abs(np.conj(conv) - div))) < 1e-12


def test_element_linear_ramp_and_blazes():
    """element.rs linear_ramp_reproduces_a_tilted_plane_wave (1e-9),
    blaze_integer_2pi_depth_is_a_pure_tilted_plane_wave (phase 1e-9, modulus
    1e-12), orientation_rotates_the_grating_vector (a kinoform at pi/2 follows
    2 pi frac(y / period), 1e-9)."""
    from oracle import element as oel
    theta = 0.02
    k = 2.0 * math.pi / LAMBDA
    alpha = math.sin(theta)
    b = ofield.uniform(1.0, 0.0, 101, 101, 1e-3, 1e-3, LAMBDA)
    out = oel.PhaseMask(lambda x, y: k * alpha * x).apply(b).samples
    want = ofield.plane_wave(theta, 0.0, 1.0, 101, 101, 1e-3, 1e-3, LAMBDA).samples
    assert float(np.max(np.abs(out - want))) < 1e-9
    period = 100e-6
    b = ofield.uniform(1.0, 0.0, 64, 64, 5e-6, 5e-6, LAMBDA)
    x, y = _xy(64, 5e-6)
    for m in (1.0, 2.0):
        s = oel.BlazedGrating(period, 2.0 * math.pi * m, 0.0).apply(b).samples
        kg = 2.0 * math.pi * m / period
        assert float(np.max(np.abs(_wrap(np.angle(s) - kg * x)))) < 1e-9
        assert float(np.max(np.abs(np.abs(s) - 1.0))) < 1e-12
    s = oel.BlazedGrating(period, 2.0 * math.pi, math.pi / 2.0).apply(b).samples
    for ix, iy in ((0, 0), (63, 17), (40, 5), (12, 63)):
        u = y[iy, 0] / period
        assert abs(_wrap(np.angle(s[iy, ix]) - 2.0 * math.pi * (u - math.floor(u)))) < 1e-9


def test_element_wedge_convention_and_rotated_ellipse():
    """element.rs wedge_ramp_piston_and_deflection_convention (centre phase
    pi/3 + k (n - 1) t0, 10 samples to the right k (n - 1) tan(alpha) 0.01
    lower, 1e-9), rotated_ellipse_aperture (45 deg: (85, 85) passes, (100, 50)
    blocked; a rotated circle equals the plain one exactly)."""
    from oracle import element as oel
    band = ofield.uniform(1.0, math.pi / 3.0, 101, 101, 1e-3, 1e-3, LAMBDA)
    alpha, t0 = 1e-3, 1e-3
    w = oel.Wedge(alpha, 1.5, t0, 0.0, oel.ClearAperture.circle(20e-3))
    out = w.apply(band).samples
    k = 2.0 * math.pi / LAMBDA
    centre = np.angle(out[50, 50])
    assert abs(_wrap(centre - (math.pi / 3.0 + k * 0.5 * t0))) < 1e-9
    assert abs(_wrap(np.angle(out[50, 60]) - (centre - k * 0.5 * math.tan(alpha) * 0.01))) < 1e-9
    ap = oel.EllipticalAperture((50e-3, 20e-3), math.pi / 4.0)
    o = ap.apply(band).samples
    assert o[85, 85] == band.samples[50, 50] and o[50, 100] == 0.0
    circ = oel.EllipticalAperture((31.7e-3, 31.7e-3), math.pi / 2.0).apply(band).samples
    plain = oel.EllipticalAperture.circle(31.7e-3).apply(band).samples
    np.testing.assert_array_equal(circ, plain)


def test_element_sag_matches_standard_surface():
    """element.rs sag_matches_zemax_standard_surface: sphere (1e-12 relative),
    paraboloid r^2 / 2R (1e-15), even asphere with 2e9 r^4 - 3e13 r^6 (1e-15)."""
    from oracle import element as oel
    r = 3.0e-3
    geo = 5e-3 - math.sqrt(5e-3 ** 2 - r * r)
    assert abs(oel.conic_sag(r, 5e-3, 0.0) - geo) / geo < 1e-12
    for r in (1e-3, 7e-3, 30e-3):
        assert abs(oel.conic_sag(r, 0.1, -1.0) - r * r / 0.2) < 1e-15
    r, c = 4e-3, 10.0
    want = c * r * r / (1.0 + math.sqrt(1.0 - c * c * r * r)) + 2.0e9 * r ** 4 - 3.0e13 * r ** 6
    assert abs(oel.conic_sag(r, 0.1, 0.0, (2.0e9, -3.0e13)) - want) < 1e-15


# ---- src/sources.rs ---------------------------------------------------------------

def test_gaussian_source_pins():
    """sources.rs waist_plane_is_real_gaussian_with_analytic_power (real,
    exp(-r^2 / w0^2) to 1e-12, power pi w0^2 / 2 to 1e-3),
    on_axis_amplitude_and_gouy_match_q_form (1e-12, phase 1e-9),
    negative_z_is_complex_conjugate (1e-12),
    off_center_waist_translates_by_integer_samples (1e-15),
    analytic_beam_matches_own_engines (ASM and Fresnel TF within 1e-3)."""
    g = ofield.gaussian
    w0 = 1e-3
    d = w0 / 20.0
    b = g(w0, 1.0, (0.0, 0.0), 0.0, LAMBDA, 201, 201, d, d)
    x, y = (np.arange(201) - 100.0) * d, (np.arange(201) - 100.0) * d
    for ix, iy in ((0, 0), (100, 100), (200, 200), (37, 160)):
        s = b.samples[iy, ix]
        assert abs(s.imag) < 1e-15
        assert abs(s.real - math.exp(-(x[ix] ** 2 + y[iy] ** 2) / (w0 * w0))) < 1e-12
    p = float(np.sum(np.abs(b.samples) ** 2)) * d * d
    assert abs(p - math.pi * w0 * w0 / 2.0) / (math.pi * w0 * w0 / 2.0) < 1e-3

    w0, z, n = 0.5e-3, 0.25, 129
    d = w0 / 20.0
    c = g(w0, 2.0, (0.0, 0.0), z, LAMBDA, n, n, d, d).samples[n // 2, n // 2]
    z_r = math.pi * w0 * w0 / LAMBDA
    w_z = w0 * math.sqrt(1.0 + (z / z_r) ** 2)
    assert abs(abs(c) - 2.0 * w0 / w_z) / (2.0 * w0 / w_z) < 1e-12
    ph = 2.0 * math.pi * z / LAMBDA - math.atan(z / z_r)
    assert abs((np.angle(c) - ph + math.pi) % (2.0 * math.pi) - math.pi) < 1e-9

    pos = g(0.5e-3, 1.0, (0.0, 0.0), 0.2, LAMBDA, 64, 64, 1e-5, 1e-5).samples
    neg = g(0.5e-3, 1.0, (0.0, 0.0), -0.2, LAMBDA, 64, 64, 1e-5, 1e-5).samples
    assert float(np.max(np.abs(np.conj(pos) - neg))) < 1e-12

    w0, n = 1e-3, 161
    d = w0 / 20.0
    on = g(w0, 1.0, (0.0, 0.0), 0.0, LAMBDA, n, n, d, d).samples
    sh = g(w0, 1.0, (3.0 * d, -2.0 * d), 0.0, LAMBDA, n, n, d, d).samples
    # shifted(ix, iy) = on_axis(ix - 3, iy + 2) over the interior
    assert float(np.max(np.abs(sh[5:n - 5, 5:n - 5] - on[7:n - 3, 2:n - 8]))) < 1e-15

    from oracle import asm as oasm
    w0, z, n, d = 0.15e-3, 0.1, 255, 1e-5
    analytic = g(w0, 1.0, (0.0, 0.0), z, LAMBDA, n, n, d, d).samples
    waist = g(w0, 1.0, (0.0, 0.0), 0.0, LAMBDA, n, n, d, d)
    fr = ofr.propagate(waist, z, ofr.FresnelConfig(2.0, False, 8.0)).samples
    asm = oasm.propagate(waist, z).samples
    assert np.linalg.norm(fr - analytic) / np.linalg.norm(analytic) < 1e-3
    assert np.linalg.norm(asm - analytic) / np.linalg.norm(analytic) < 1e-3


# ---- src/field.rs -----------------------------------------------------------------

def test_field_pins():
    """field.rs plane_wave_phase_ramp_matches_direction_cosines (1e-9, a flat wave
    exactly A), coordinates_are_centered_on_origin (exact), uniform_field_power
    (1e-6; amplitude, phase, intensity 1e-12), band_field_validates_wavelength;
    the product's BandField rejects the same wavelengths."""
    from optics_studio_gb300.field import BandField
    lam = 500e-9
    b = ofield.plane_wave(0.05, 0.0, 1.0, 16, 16, 10e-6, 10e-6, lam).samples
    step = np.exp(1j * 2.0 * math.pi / lam * math.sin(0.05) * 10e-6)
    for iy in (0, 7, 15):
        assert abs(b[iy, 8] / b[iy, 7] - step) < 1e-9
    flat = ofield.plane_wave(0.0, 0.0, 3.0, 16, 16, 10e-6, 10e-6, lam).samples
    assert np.all(flat == 3.0 + 0.0j)
    x = (np.arange(5) - 2.0) * 1e-3
    y = (np.arange(3) - 1.0) * 1e-3
    assert (x[2], y[1]) == (0.0, 0.0) and (x[0], y[0]) == (-2e-3, -1e-3)
    assert (x[4], y[2]) == (2e-3, 1e-3)
    u = ofield.uniform(2.0, math.pi / 3.0, 8, 4, 1e-3, 5e-4, lam)
    want = 4.0 * 8 * 4 * 1e-3 * 5e-4
    assert abs(power(u) - want) < 1e-6 * want
    assert float(np.max(np.abs(np.abs(u.samples) - 2.0))) < 1e-12
    assert float(np.max(np.abs(np.angle(u.samples) - math.pi / 3.0))) < 1e-12
    for lam_bad in (0.0, math.nan, -1.0):
        with pytest.raises(Exception):
            ofield.uniform(1.0, 0.0, 2, 2, 1e-3, 1e-3, lam_bad)
        with pytest.raises(ValueError):
            BandField(np.zeros((2, 2), complex), 1e-3, 1e-3, lam_bad)


# ---- src/propagation/asm.rs (host analysis: oracle and product) -------------------

def _product_asm_report(n, d, z, cfg):
    import optics_studio_gb300 as og
    from optics_studio_gb300 import _ffi
    rep = _ffi.AsmReportC()
    assert og.lib().osgpu_asm_sampling_report(_ffi.Grid(n, n, d, d, LAMBDA), z, cfg.c(), rep) == 0
    return rep


def test_asm_padding_band_limit_and_medium_pins():
    """asm.rs padding_rounds_up_and_clamps, band_limit_uses_padded_width_and_shrinks_with_z,
    medium_scales_band_limit_and_guard, medium_round_trip_inverts (1e-9),
    invalid_inputs_rejected; the product's host analysis gives the same padded
    sizes, band limits and steps as the oracle."""
    from oracle import asm as oasm
    from oracle.fft import padded_len
    from optics_studio_gb300.propagation import asm as gasm
    for pad, want in ((2.0, 200), (1.5, 150), (1.0, 100), (0.5, 100)):
        assert padded_len(100, pad) == want
        rep = _product_asm_report(100, 10e-6, 1e-3, gasm.AsmConfig(pad, True, False, 8.0, 1.0))
        assert rep.nx_pad == want
    lp = 200.0 * 10e-6
    f0 = oasm.axis_band_limit(LAMBDA, 0.0, lp, True, 1.0)
    assert abs(f0 - 1.0 / LAMBDA) < 1e-6
    assert oasm.axis_band_limit(LAMBDA, 0.05, lp, True, 1.0) < f0
    assert abs(oasm.axis_band_limit(LAMBDA, 1.0, lp, False, 1.0) - 1.0 / LAMBDA) < 1e-9
    rep = _product_asm_report(100, 10e-6, 0.05, gasm.AsmConfig(2.0, True, False, 8.0, 1.0))
    assert rep.band_limit_fx == oasm.axis_band_limit(LAMBDA, 0.05, lp, True, 1.0)

    b = uniform(1.0, 32, 1e-6)
    base = oasm.AsmConfig(2.0, False, False, 8.0, 1.0)
    dense = oasm.AsmConfig(2.0, False, False, 8.0, 1.5)
    r1, r2 = oasm.sampling_report(b, 0.5, base), oasm.sampling_report(b, 0.5, dense)
    assert abs(r2.band_limit_fx - 1.5 * r1.band_limit_fx) < 1e-9
    assert 0.55 < r2.max_phase_step_x / r1.max_phase_step_x < 1.0 and r2.medium == 1.5
    p1 = _product_asm_report(32, 1e-6, 0.5, gasm.AsmConfig(2.0, False, False, 8.0, 1.0))
    p2 = _product_asm_report(32, 1e-6, 0.5, gasm.AsmConfig(2.0, False, False, 8.0, 1.5))
    assert (p1.band_limit_fx, p1.max_phase_step_x) == (r1.band_limit_fx, r1.max_phase_step_x)
    assert (p2.band_limit_fx, p2.max_phase_step_x, p2.medium) == (
        r2.band_limit_fx, r2.max_phase_step_x, 1.5)

    b = uniform(1.0, 16, 20e-6)
    cfg = oasm.AsmConfig(padding=1.0, medium=2.0)
    rt = oasm.propagate(oasm.propagate(b, 1e-3, cfg), -1e-3, cfg)
    assert float(np.max(np.abs(rt.samples - b.samples))) < 1e-9
    with pytest.raises(oasm.PropagationError) as e:
        oasm.propagate(uniform(1.0, 8, 20e-6), math.nan)
    assert e.value.variant == "InvalidDistance"


def test_fraunhofer_regime_extent_is_measured_from_the_axis():
    """fraunhofer.rs regime_extent_is_measured_from_the_axis: with max N_F 0.15
    the centred Gaussian passes (N_F 0.099); declared 0.2 mm off axis it fails
    (0.265), reports the position and the strict propagation refuses; the
    product's host regime report agrees."""
    import optics_studio_gb300 as og
    from optics_studio_gb300 import _ffi
    from optics_studio_gb300.propagation import fraunhofer as gfh
    b = gaussian(64, 1e-5, 5e-5)
    assert ofh.regime_report(b, 2.0, ofh.FraunhoferConfig(max_n_f=0.15)).regime_ok
    off = ofh.FraunhoferConfig(max_n_f=0.15, source_pos=(2e-4, 0.0))
    rep = ofh.regime_report(b, 2.0, off)
    assert not rep.regime_ok and tuple(rep.source_pos) == (2e-4, 0.0)
    with pytest.raises(ofh.FraunhoferError) as e:
        ofh.propagate(b, 2.0, off)
    assert e.value.variant == "RegimeViolation"
    for cfg, ok in ((gfh.FraunhoferConfig(max_n_f=0.15), True),
                    (gfh.FraunhoferConfig(max_n_f=0.15, source_pos=(2e-4, 0.0)), False)):
        r = _ffi.FraunhoferReportC()
        og.lib().osgpu_fraunhofer_regime_report(_ffi.Grid(64, 64, 1e-5, 1e-5, LAMBDA), 2.0,
                                                cfg.c(), r)
        assert bool(r.regime_ok) == ok


# ---- crates/optics-inverse/src/carrier.rs -----------------------------------------

def test_carrier_pins():
    """carrier.rs grid_phase_roundtrip_matches_manual_mask (the built design
    traced without propagation equals the sampled mask exactly),
    grid_carriers_validate_before_building, analytic_rejects_bad_values_at_apply."""
    from oracle import carrier as ocar, element as oel
    values = np.arange(16, dtype=np.float64) * 0.2
    car = ocar.Carrier.grid_phase((4, 4), (20e-6, 20e-6), oel.ClearAperture.field(), (0.0, 0.0),
                                  0.0, math.pi)
    assert car.dim == 16 and car.slot_bounds() == (0.0, math.pi)
    b = ofield.uniform(1.0, 0.0, 32, 32, 20e-6, 20e-6, LAMBDA)
    out = car.build(values, LAMBDA).beamline().trace(b, lambda x, z, m: x)
    manual = oel.PhaseMask.sampled(values, (4, 4), (20e-6, 20e-6)).apply(b)
    np.testing.assert_array_equal(out.samples, manual.samples)
    g = ocar.Carrier.grid_phase((2, 2), (1e-5, 1e-5), oel.ClearAperture.field(), (0.0, 0.0),
                                0.0, 1.0)
    for vals, variant in (([0.5, 0.5, 0.5, 1.5], "OutOfBounds"), ([0.5] * 3, "WrongDimension")):
        with pytest.raises(ocar.InverseError) as e:
            g.build(np.array(vals), LAMBDA)
        assert e.value.variant == variant
    with pytest.raises(ocar.InverseError):
        ocar.Carrier.grid_phase((0, 4), (1e-5, 1e-5), oel.ClearAperture.field(), (0.0, 0.0),
                                0.0, 1.0)

    def build(v, lam):
        d = ocar.Design()
        d.gap(v[0], 1.0)
        return d
    an = ocar.Carrier.analytic(1, 0.01, 1.0, build)
    for vals, variant in (([5.0], "OutOfBounds"), ([math.nan], "NotFinite"),
                          ([], "WrongDimension")):
        with pytest.raises(ocar.InverseError) as e:
            an.build(np.array(vals), LAMBDA)
        assert e.value.variant == variant


def test_fresnel_transfer_matches_asm_at_low_frequencies():
    """fresnel.rs transfer_function_matches_asm_at_low_frequencies: at
    (lambda f)^2 = s = 1e-4 the Fresnel transfer differs from the ASM one by
    at most 2 k z s^2 / 8, and the DC bin is e^{ikz} (1e-12)."""
    z, s = 0.1, 1e-4
    k = 2.0 * math.pi / LAMBDA
    f = math.sqrt(s) / LAMBDA
    h = ofr.transfer_function(2, 1, 1.0 / (2.0 * f), 1.0, LAMBDA, z)  # bins 0 and -f
    h_asm = np.exp(1j * k * z * math.sqrt(1.0 - s))
    assert abs(h[0, 1] - h_asm) < 2.0 * k * z * s * s / 8.0 + 1e-12
    assert abs(h[0, 0] - np.exp(1j * k * z)) < 1e-12


def test_adjoint_gs_phase_error_is_negative_mse_gradient():
    """adjoint.rs gs_phase_error_is_adjoint_mse_negative_gradient: after 40 GS
    iterations (32^2, 20 um, z/2 = 1.5 mm), the adjoint gradient of the
    amplitude MSE, g = -2 Im(conj(mu) mask), anti-correlates with A^2 dphi
    (corr > 0.9) and its least-squares scale lies within 25 % of 2 / N."""
    from oracle import adjoint as oadj, asm as oasm
    n, d, half_z = 32, 20e-6, 1.5e-3
    npx = n * n
    cfg = oasm.AsmConfig(band_limited=False, strict=False)
    c = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * d
    r2 = c[None, :] ** 2 + c[:, None] ** 2
    inp = ofield.BandField(np.exp(-r2 / (2.0 * 90e-6 ** 2)).astype(complex), d, d, LAMBDA)
    illum = np.abs(oasm.propagate(inp, half_z, cfg).samples)
    gi = np.exp(-r2 / (120e-6 ** 2))
    target = np.sqrt(gi) / math.sqrt(float(np.max(gi))) * 0.8
    band = lambda s: ofield.BandField(s, d, d, LAMBDA)
    phi = np.zeros((n, n))
    dphi = np.zeros((n, n))
    for _ in range(40):
        u_t = oasm.propagate(band(illum * np.exp(1j * phi)), half_z, cfg).samples
        v = oadj.asm_adjoint(band(target * np.exp(1j * np.angle(u_t))), half_z, cfg).samples
        dphi = (np.angle(v) - phi + math.pi) % (2.0 * math.pi) - math.pi
        phi = phi + dphi
    phi_prev = (phi - dphi + math.pi) % (2.0 * math.pi) - math.pi
    mask = illum * np.exp(1j * phi_prev)
    u_t = oasm.propagate(band(mask), half_z, cfg).samples
    a = np.abs(u_t)
    w = np.where(a > 1e-30, (a - target) / npx * u_t / np.where(a > 1e-30, a, 1.0), 0.0)
    mu = oadj.asm_adjoint(band(w), half_z, cfg).samples
    g = (-2.0 * np.imag(np.conj(mu) * mask)).reshape(-1)
    pred = (illum * illum * dphi).reshape(-1)
    cov = -np.sum((g - g.mean()) * (pred - pred.mean()))
    corr = cov / (np.linalg.norm(g - g.mean()) * np.linalg.norm(pred - pred.mean()))
    assert corr > 0.9, corr
    ls = -float(np.sum(g * pred)) / float(np.sum(pred * pred))
    assert abs(ls / (2.0 / npx) - 1.0) < 0.25, ls


def _disk_target(u_in, n, d, r, amp=None):
    c = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * d
    disk = c[None, :] ** 2 + c[:, None] ** 2 <= r * r
    if amp is None:
        amp = math.sqrt(float(np.sum(np.abs(u_in) ** 2)) / float(np.sum(disk)))
    return np.where(disk, amp, 0.0)


def test_gs_dvr_and_fpr_variants():
    """gs.rs dvr_variant_converges_on_tophat (DVR = phase relaxation beta 0.7:
    best-so-far monotone, final merit below half the first) and
    fpr_variant_stops_on_merit_seam (FPR = Fourier-plane relaxation beta 0.8
    stops by the patience rule within 120 iterations).  Seeded uniform starts
    stand in for rand's StdRng."""
    from oracle import gs as ogs
    n, d = 96, 8e-6
    u = ofield.gaussian(140e-6, 1.0, (0.0, 0.0), 0.0, LAMBDA, n, n, d, d).samples
    t = _disk_target(u, n, d, 220e-6)
    fwd, back = _gs_asm(n, d, 8e-3)
    init = np.random.default_rng(11).uniform(-math.pi, math.pi, (n, n))
    sol = ogs.run(u, np.ones((n, n), bool), t, -math.pi, math.pi, init, fwd, back, _mse_merit(t),
                  max_iterations=150, patience=10, merit_tolerance=1e-4, beta_p=0.7)
    best = [r.best_merit for r in sol.history]
    assert all(b1 <= b0 + 1e-15 for b0, b1 in zip(best, best[1:]))
    assert sol.merit < 0.5 * sol.history[0].merit

    n, d = 64, 10e-6
    u = ofield.gaussian(120e-6, 1.0, (0.0, 0.0), 0.0, LAMBDA, n, n, d, d).samples
    t = _disk_target(u, n, d, 180e-6, amp=1.0)
    fwd, back = _gs_asm(n, d, 6e-3)
    init = np.random.default_rng(3).uniform(-math.pi, math.pi, (n, n))
    sol = ogs.run(u, np.ones((n, n), bool), t, -math.pi, math.pi, init, fwd, back, _mse_merit(t),
                  max_iterations=120, patience=5, merit_tolerance=1e-3, beta_f=0.8)
    assert sol.converged and sol.iterations <= 120


# ---- src/analysis.rs --------------------------------------------------------------

def test_analysis_mtf_dc_and_zero_field_safety():
    """analysis.rs mtf_dc_and_zero_field_safety: a flat PSF's MTF vanishes off
    DC (1e-9); a dark PSF has spot RMS 0, Strehl 0 and an encircled energy of
    0 everywhere."""
    from oracle import analysis as oan
    flat, zero = np.ones((8, 8)), np.zeros((8, 8))
    _, vals = oan.mtf(flat, (1e-3, 1e-3))
    assert max(vals[1:]) < 1e-9
    assert oan.spot_rms_radius(zero, (1e-3, 1e-3)) == 0.0
    assert oan.strehl(zero, (1e-3, 1e-3), flat, (1e-3, 1e-3)) == 0.0
    assert oan.encircled_energy(zero, (1e-3, 1e-3)).value_at(1.0) == 0.0


def _wrap(p):
    return (p + math.pi) % (2 * math.pi) - math.pi


def test_thick_lens_paraxial_matches_thin_lens_with_piston():
    """element.rs thick_lens_paraxial_matches_thin_lens_with_piston: biconvex
    R1 = +0.1, R2 = -0.1, n = 1.5 gives f = 0.1 m; the vertex phase is the
    piston k (n - 1) t0; at rho = 2 mm the relative phase equals the exact
    two-sphere sag to 1e-9 and differs from the paraxial quadratic by the r^4
    residual (~ -0.025 rad).  The product's host-evaluated thickness screen
    takes the same values."""
    from optics_studio_gb300 import element as gel
    lam, t0 = 500e-9, 2e-3
    lens = oel.ThickLens(oel.SurfaceProfile.spherical(0.1), oel.SurfaceProfile.spherical(-0.1),
                         1.5, t0, None, oel.ClearAperture.circle(2e-2))
    f = lens.focal_at(lam)
    assert abs(f - 0.1) < 1e-12
    k = 2 * math.pi / lam
    band = ofield.uniform(1.0, math.pi / 3.0, 101, 101, 1e-3, 1e-3, lam)
    out = lens.apply(band).samples
    center = np.angle(out[50, 50])
    assert abs(_wrap(center - (math.pi / 3.0 + k * 0.5 * t0))) < 1e-9
    rho = 2e-3
    rel = _wrap(np.angle(out[50, 52]) - center)
    exact = -k * 0.5 * 2.0 * (0.1 - math.sqrt(0.1 ** 2 - rho * rho))
    assert abs(_wrap(rel - exact)) < 1e-9
    paraxial = -k * rho * rho / (2.0 * f)
    assert abs(_wrap(rel - paraxial) - (-0.025)) < 0.005
    assert abs(lens.thickness_profile(0.0) - t0) < 1e-18
    assert lens.thickness_profile(1e-2) < t0
    g = gel.ThickLens(gel.SurfaceProfile.spherical(0.1), gel.SurfaceProfile.spherical(-0.1),
                      1.5, t0, None, gel.ClearAperture.circle(2e-2))
    assert g.focal_at(lam) == f
    from optics_studio_gb300.field import BandField
    d, v = g.descriptor(BandField(band.samples, 1e-3, 1e-3, lam))
    xs = ofield.axis_coords(101, 1e-3)
    r = np.hypot(xs[None, :], xs[:, None])
    inside = r <= 2e-2
    assert np.array_equal(v[inside], lens.thickness_profile(r)[inside])
    assert d.depth == k * (1.5 - 1.0)


def test_thick_lens_validation_matches_reference_errors():
    """element.rs thick_lens_validation: negative thickness -> InvalidThickness;
    a back surface whose conic domain the stop exceeds -> InvalidSurface;
    analytic profiles have no power; zero thickness adds no piston.  The
    product's binding raises the same variants (host-side construction and
    apply checks: OutsideField, InvalidMedium, InvalidSag)."""
    import optics_studio_gb300 as og
    from optics_studio_gb300 import element as gel
    from optics_studio_gb300.field import BandField
    lam = 500e-9
    sph = oel.SurfaceProfile.spherical
    with pytest.raises(oel.OpticsError) as e:
        oel.ThickLens(sph(0.1), sph(-0.1), 1.5, -1e-3, None, oel.ClearAperture.circle(2e-2))
    assert e.value.variant == "InvalidThickness"
    with pytest.raises(oel.OpticsError) as e:
        oel.ThickLens(sph(0.1), sph(1e-3), 1.5, 1e-3, None, oel.ClearAperture.circle(2e-3))
    assert e.value.variant == "InvalidSurface"
    an = oel.ThickLens(oel.SurfaceProfile(analytic=lambda r: r * r), sph(0.1), 1.5, 0.0, None,
                       oel.ClearAperture.circle(1e-3))
    assert an.power_at(lam) is None and an.focal_at(lam) is None
    flat = oel.ThickLens(sph(0.1), sph(-0.1), 1.5, 0.0, None, oel.ClearAperture.circle(1e-3))
    band = ofield.uniform(1.0, math.pi / 3.0, 101, 101, 1e-3, 1e-3, lam)
    assert abs(_wrap(np.angle(flat.apply(band).samples[50, 50]) - math.pi / 3.0)) < 1e-12

    gs = gel.SurfaceProfile.spherical
    for args, variant in [
        ((gs(0.1), gs(-0.1), 1.5, -1e-3, None, gel.ClearAperture.circle(2e-2)), "InvalidThickness"),
        ((gs(0.1), gs(1e-3), 1.5, 1e-3, None, gel.ClearAperture.circle(2e-3)), "InvalidSurface"),
        ((gs(0.0), gs(-0.1), 1.5, 1e-3, None, gel.ClearAperture.circle(2e-3)), "InvalidSurface"),
        ((gs(0.1), gs(-0.1), 1.5, 1e-3, None, gel.ClearAperture.circle(-1.0)), "InvalidAperture"),
        ((gs(0.1), gs(-0.1), 1.5, 1e-3, math.nan), "InvalidOrientation"),
    ]:
        with pytest.raises(og.OsgpuError) as e:
            gel.ThickLens(*args)
        assert e.value.variant == variant
    gb = BandField(band.samples, 1e-3, 1e-3, lam)
    big = gel.ThickLens(gs(1.0), gs(-1.0), 1.5, 1e-3, None, gel.ClearAperture.circle(60e-3))
    with pytest.raises(og.OsgpuError) as e:
        big.descriptor(gb)
    assert e.value.variant == "OutsideField"
    bad_n = gel.ThickLens(gs(0.1), gs(-0.1), lambda l: -1.0, 1e-3, None,
                          gel.ClearAperture.circle(2e-2))
    with pytest.raises(og.OsgpuError) as e:
        bad_n.descriptor(gb)
    assert e.value.variant == "InvalidMedium"
    nan_sag = gel.ThickLens(gel.SurfaceProfile(analytic=lambda r: np.where(r > 5e-3, np.nan, 0.0)),
                            gs(-0.1), 1.5, 1e-3, None, gel.ClearAperture.circle(2e-2))
    with pytest.raises(og.OsgpuError) as e:
        nan_sag.descriptor(gb)
    assert e.value.variant == "InvalidSag"
