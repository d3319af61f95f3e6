"""GPU parity: every engine of the hot path through the C ABI against the f64
oracle on the same seeded inputs.

Tolerances (relative L2 over the output field):
  * f64 engine: <= 1e-12 (the plain path);
  * f32 engine: <= 1e-5 (FP32 complex FFTs, FP64-derived phase tables).
Element transmissions are compared elementwise (decisions bit-exact).
"""

import math

import numpy as np
import pytest

import optics_studio_gb300 as og
from optics_studio_gb300 import element as gel
from optics_studio_gb300.beamline import AsmEngine, Beamline
from optics_studio_gb300.field import BandField
from optics_studio_gb300.propagation import asm as gasm, fresnel as gfr, fraunhofer as gfh
from optics_studio_gb300.propagation import rayleigh_sommerfeld as grs
from oracle import asm as oasm, fresnel as ofr, fraunhofer as ofh, rs as ors
from oracle import field as ofield, element as oel, beamline as obl

from _util import rel_l2, to_gpu_band, rng_field

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5


def c1_band():
    """Plain f64 ASM workload: 512^2, dx 2 um, lambda 633 nm, Gaussian waist
    100 um x circular aperture r 400 um."""
    b = ofield.gaussian(100e-6, 1.0, (0.0, 0.0), 0.0, 633e-9, 512, 512, 2e-6, 2e-6)
    return oel.EllipticalAperture.circle(400e-6).apply(b)


@pytest.mark.parametrize("prec,tol", [("f64", TOL64), ("f32", TOL32)])
def test_asm_c1_plain_workload(prec, tol):
    ob = c1_band()
    ref = oasm.propagate(ob, 10e-3)
    out = gasm.propagate(to_gpu_band(ob), 10e-3, gasm.AsmConfig(), prec)
    assert (out.report.nx_pad, out.report.ny_pad) == (2048, 2048)
    assert rel_l2(out.samples, ref.samples) <= tol


ASM_CASES = [
    # ny, nx, dx, dy, lam, z, cfg
    (64, 48, 10e-6, 8e-6, 500e-9, 1e-3, oasm.AsmConfig()),
    (37, 45, 4e-6, 5e-6, 532e-9, -2e-3, oasm.AsmConfig(1.5, True, True, 8.0, 1.3)),
    (32, 32, 1e-6, 1e-6, 500e-9, 0.5, oasm.AsmConfig(2.0, False, False, 8.0, 1.5)),
    (64, 64, 1e-6, 1e-6, 500e-9, 7.68e-4, oasm.AsmConfig(1.0, False, True, 8.0, 1.0)),
    (128, 96, 3e-6, 3e-6, 450e-9, 0.1, oasm.AsmConfig()),
    (1, 16, 5e-6, 5e-6, 600e-9, 1e-3, oasm.AsmConfig(padding=1.0, strict=False)),
    (30, 1, 5e-6, 5e-6, 600e-9, 1e-3, oasm.AsmConfig(padding=3.0, strict=False)),
]


@pytest.mark.parametrize("case", ASM_CASES)
@pytest.mark.parametrize("prec,tol", [("f64", TOL64), ("f32", TOL32)])
def test_asm_matches_oracle(case, prec, tol):
    ny, nx, dx, dy, lam, z, cfg = case
    ob = ofield.BandField(rng_field(ny, nx, seed=ny * 7 + nx), dx, dy, lam)
    ref = oasm.propagate(ob, z, cfg)
    gcfg = gasm.AsmConfig(cfg.padding, cfg.band_limited, cfg.strict, cfg.max_padding, cfg.medium)
    out = gasm.propagate(to_gpu_band(ob), z, gcfg, prec)
    assert rel_l2(out.samples, ref.samples) <= tol


def test_asm_errors_map_to_reference_variants():
    b = BandField(np.ones((64, 64), complex), 1e-6, 1e-6, 500e-9)
    with pytest.raises(og.OsgpuError) as e:
        gasm.propagate(b, 7.68e-4, gasm.AsmConfig(1.0, False, True, 1.0, 1.0))
    assert e.value.variant == "AliasingRisk"
    assert e.value.report.used_padding == 1.0 and e.value.report.max_phase_step_x > math.pi
    bad = np.ones((16, 16), complex)
    bad[4, 5] = np.nan
    with pytest.raises(og.OsgpuError) as e:
        gasm.propagate(BandField(bad, 20e-6, 20e-6, 500e-9), 1e-3)
    assert e.value.variant == "NonFiniteSample"
    # the library stays usable after a device-detected error
    ok = gasm.propagate(BandField(np.ones((16, 16), complex), 20e-6, 20e-6, 500e-9), 1e-3,
                        gasm.AsmConfig(padding=1.0))
    k = 2 * math.pi / 500e-9
    assert abs(ok.samples[9, 3] - np.exp(1j * k * 1e-3)) < 1e-9


def test_asm_round_trip_and_energy_gpu():
    """tests/asm.rs:91-98, 356-373 on the GPU path."""
    x = ofield.axis_coords(256, 10e-6)
    u = np.exp(-((x[None, :] ** 2 + x[:, None] ** 2) / (2 * 0.15e-3 ** 2))) + 0j
    b = BandField(u, 10e-6, 10e-6, 500e-9)
    out = gasm.propagate(b, 0.1)
    assert abs(out.power() - b.power()) / b.power() <= 1e-9
    back = gasm.propagate(out, -0.1)
    assert rel_l2(back.samples, u) < 1e-6


FRESNEL_CASES = [
    (128, 128, 10e-6, 10e-6, 532e-9, 5e-3),
    (96, 80, 8e-6, 6e-6, 633e-9, -3e-3),
]


@pytest.mark.parametrize("case", FRESNEL_CASES)
@pytest.mark.parametrize("prec,tol", [("f64", TOL64), ("f32", TOL32)])
def test_fresnel_tf_and_conv_match_oracle(case, prec, tol):
    ny, nx, dx, dy, lam, z = case
    ob = ofield.BandField(rng_field(ny, nx, seed=3), dx, dy, lam)
    cfg = ofr.FresnelConfig(strict=False)
    ref_tf = ofr.propagate(ob, z, cfg)
    ref_cv = ofr.propagate_convolution(ob, z, cfg)
    g = to_gpu_band(ob)
    gcfg = gfr.FresnelConfig(strict=False)
    assert rel_l2(gfr.propagate(g, z, gcfg, prec).samples, ref_tf.samples) <= tol
    assert rel_l2(gfr.propagate_convolution(g, z, gcfg, prec).samples, ref_cv.samples) <= tol


FRAUN_CASES = [
    (64, 64, 10e-6, 10e-6, 633e-9, 0.5, ofh.FraunhoferConfig(strict=False)),
    (31, 33, 12e-6, 10e-6, 532e-9, -0.3, ofh.FraunhoferConfig(strict=False)),
    (40, 36, 10e-6, 10e-6, 500e-9, 0.8,
     ofh.FraunhoferConfig(strict=False, source_pos=(3e-5, -2e-5))),
]


@pytest.mark.parametrize("case", FRAUN_CASES)
@pytest.mark.parametrize("prec,tol", [("f64", TOL64), ("f32", TOL32)])
def test_fraunhofer_matches_oracle(case, prec, tol):
    ny, nx, dx, dy, lam, z, cfg = case
    ob = ofield.BandField(rng_field(ny, nx, seed=5), dx, dy, lam)
    ref = ofh.propagate(ob, z, cfg)
    gcfg = gfh.FraunhoferConfig(cfg.strict, cfg.max_n_f, cfg.source_pos, cfg.aperture_extent)
    out = gfh.propagate(to_gpu_band(ob), z, gcfg, prec)
    assert (out.dx, out.dy) == (ref.dx, ref.dy)
    assert rel_l2(out.samples, ref.samples) <= tol


@pytest.mark.parametrize("prec,tol", [("f64", TOL64), ("f32", TOL32)])
def test_rayleigh_sommerfeld_matches_oracle(prec, tol):
    n, d, z = 100, 2e-6, 5e-3
    x = ofield.axis_coords(n, d)
    u = np.exp(-((x[None, :] ** 2 + x[:, None] ** 2) / (2 * 30e-6 ** 2))) + 0j
    ob = ofield.BandField(u * np.exp(1j * rng_field(n, n, 9).real), d, d, 500e-9)
    ref = ors.propagate(ob, z, ors.RayleighSommerfeldConfig(strict=False))
    out = grs.propagate(to_gpu_band(ob), z, grs.RayleighSommerfeldConfig(strict=False), prec)
    assert rel_l2(out.samples, ref.samples) <= tol


def element_pairs(n):
    """(product element, oracle element) pairs covering every kind and stop."""
    lat = np.random.default_rng(1).uniform(0, 2 * np.pi, (n, n))
    d = 5e-6
    return [
        (gel.EllipticalAperture.circle(40e-6, (3e-6, -2e-6)),
         oel.EllipticalAperture.circle(40e-6, (3e-6, -2e-6))),
        (gel.EllipticalAperture((60e-6, 30e-6), 0.4, (0.0, 5e-6)),
         oel.EllipticalAperture((60e-6, 30e-6), 0.4, (0.0, 5e-6))),
        (gel.RectangularAperture((50e-6, 25e-6), None, (-5e-6, 0.0)),
         oel.RectangularAperture((50e-6, 25e-6), None, (-5e-6, 0.0))),
        (gel.RectangularAperture((50e-6, 25e-6), 1.1),
         oel.RectangularAperture((50e-6, 25e-6), 1.1)),
        (gel.ThinLens.fixed(0.02, None, gel.ClearAperture.circle(70e-6)),
         oel.ThinLens.fixed(0.02, None, oel.ClearAperture.circle(70e-6))),
        (gel.ThinLens(lambda lam: 0.03 * lam / 500e-9, 0.3, gel.ClearAperture.ellipse(80e-6, 50e-6),
                      (4e-6, 4e-6)),
         oel.ThinLens(lambda lam: 0.03 * lam / 500e-9, 0.3, oel.ClearAperture.ellipse(80e-6, 50e-6),
                      (4e-6, 4e-6))),
        (gel.PhaseMask.sampled(lat, (n, n), (d, d)),
         oel.PhaseMask.sampled(lat, (n, n), (d, d))),
        (gel.PhaseMask.sampled(lat[:20, :30], (30, 20), (3e-6, 4e-6), 0.2,
                               gel.ClearAperture.rectangle(60e-6, 40e-6), (2e-6, 0.0)),
         oel.PhaseMask.sampled(lat[:20, :30], (30, 20), (3e-6, 4e-6), 0.2,
                               oel.ClearAperture.rectangle(60e-6, 40e-6), (2e-6, 0.0))),
        (gel.BlazedGrating(23e-6, 5.0, 0.0, gel.ClearAperture.circle(90e-6)),
         oel.BlazedGrating(23e-6, 5.0, 0.0, oel.ClearAperture.circle(90e-6))),
        (gel.BlazedGrating.kinoform(31e-6, 0.7), oel.BlazedGrating(31e-6, 2 * np.pi, 0.7)),
    ]


@pytest.mark.parametrize("prec,tol", [("f64", 1e-14), ("f32", 2e-6)])
def test_elements_match_oracle(prec, tol):
    n = 41
    ob = ofield.BandField(rng_field(n, n, 11), 5e-6, 5e-6, 550e-9)
    for ge, oe in element_pairs(n):
        ref = oe.apply(ob).samples
        out = ge.apply(to_gpu_band(ob), prec).samples
        assert np.array_equal(out == 0, ref == 0), type(ge).__name__
        assert np.max(np.abs(out - ref)) <= tol * np.max(np.abs(ref)), type(ge).__name__


def test_element_errors():
    b = BandField(np.ones((11, 11), complex), 1.0, 1.0, 500e-9)
    with pytest.raises(og.OsgpuError) as e:
        gel.EllipticalAperture.circle(6.0).apply(b)
    assert e.value.variant == "OutsideField"
    with pytest.raises(og.OsgpuError) as e:
        gel.ThinLens.fixed(0.0).apply(b)
    assert e.value.variant == "InvalidFocal"


@pytest.mark.parametrize("prec,tol", [("f64", TOL64), ("f32", TOL32)])
def test_beamline_trace_fused_matches_oracle(prec, tol):
    """DOE -> z1 -> aperture + lens -> z2 (elements fused into the FFT pass)."""
    n, d, lam = 96, 4e-6, 532e-9
    lat = np.floor(np.random.default_rng(4).uniform(0, 8, (n, n))) * (2 * np.pi / 8)
    ob = ofield.plane_wave(0.0, 0.0, 1.0, n, n, d, d, lam)
    obl_ = obl.Beamline()
    obl_.push(oel.PhaseMask.sampled(lat, (n, n), (d, d)), 2e-3)
    obl_.push(oel.RectangularAperture((150e-6, 120e-6)), 0.0)
    obl_.push(oel.ThinLens.fixed(0.05), 5e-3)
    cfg = oasm.AsmConfig()
    ref = obl_.trace(ob, obl.asm_engine(cfg))
    gbl = Beamline()
    gbl.push(gel.PhaseMask.sampled(lat, (n, n), (d, d)), 2e-3)
    gbl.push(gel.RectangularAperture((150e-6, 120e-6)), 0.0)
    gbl.push(gel.ThinLens.fixed(0.05), 5e-3)
    out = gbl.trace(to_gpu_band(ob), AsmEngine(gasm.AsmConfig(), prec))
    assert rel_l2(out.samples, ref.samples) <= tol


REG_CASES = [
    # ny, nx, dx, lam, z, cfg  (sub-FFT lengths 256..2048: the register-FFT passes)
    (256, 256, 3e-6, 500e-9, 0.02, oasm.AsmConfig()),
    (256, 512, 2e-6, 633e-9, -4e-3, oasm.AsmConfig(2.0, True, True, 8.0, 1.3)),
    (512, 512, 3e-6, 450e-9, 0.05, oasm.AsmConfig(2.0, False, False, 8.0, 1.0)),
    (1024, 1024, 4e-6, 532e-9, 0.03, oasm.AsmConfig()),
]


@pytest.mark.parametrize("case", REG_CASES)
def test_asm_f32_register_fft_sizes(case):
    ny, nx, dx, lam, z, cfg = case
    ob = ofield.BandField(rng_field(ny, nx, seed=nx + ny), dx, dx, lam)
    ref = oasm.propagate(ob, z, cfg)
    gcfg = gasm.AsmConfig(cfg.padding, cfg.band_limited, cfg.strict, cfg.max_padding, cfg.medium)
    out = gasm.propagate(to_gpu_band(ob), z, gcfg, "f32")
    assert rel_l2(out.samples, ref.samples) <= TOL32


def test_beamline_f32_register_fft_with_fused_fast_elements():
    """1024^2 DOE -> square aperture -> lens -> ASM, f32 engine: fast element
    tables fused into the register-FFT first pass."""
    n, d, lam = 1024, 4e-6, 532e-9
    lat = np.floor(np.random.default_rng(8).uniform(0, 16, (n, n))) * (2 * np.pi / 16)
    ob = ofield.plane_wave(0.0, 0.0, 1.0, n, n, d, d, lam)
    o = obl.Beamline()
    o.push(oel.PhaseMask.sampled(lat, (n, n), (d, d)), 0.0)
    o.push(oel.RectangularAperture((1.5e-3, 1.5e-3)), 0.0)
    o.push(oel.ThinLens.fixed(0.05), 0.02)
    ref = o.trace(ob, obl.asm_engine(oasm.AsmConfig()))
    g = Beamline()
    g.push(gel.PhaseMask.sampled(lat, (n, n), (d, d)), 0.0)
    g.push(gel.RectangularAperture((1.5e-3, 1.5e-3)), 0.0)
    g.push(gel.ThinLens.fixed(0.05), 0.02)
    out = g.trace(to_gpu_band(ob), AsmEngine(gasm.AsmConfig(), "f32"))
    assert rel_l2(out.samples, ref.samples) <= TOL32


@pytest.mark.parametrize("z", [5e-3, -3e-3])
def test_fresnel_f32_register_fft(z):
    ob = ofield.BandField(rng_field(256, 256, seed=21), 8e-6, 8e-6, 633e-9)
    cfg = ofr.FresnelConfig(strict=False)
    g = to_gpu_band(ob)
    gcfg = gfr.FresnelConfig(strict=False)
    assert rel_l2(gfr.propagate(g, z, gcfg, "f32").samples,
                  ofr.propagate(ob, z, cfg).samples) <= TOL32
    assert rel_l2(gfr.propagate_convolution(g, z, gcfg, "f32").samples,
                  ofr.propagate_convolution(ob, z, cfg).samples) <= TOL32


def screen_pairs():
    """Elements bound as grid screens (host-evaluated values): refractive
    surfaces (conic + asphere + tilt), wedges, an analytic phase mask and
    thick lenses, rotated and unrotated (unrotated ones take the f32 table
    path)."""
    prof = lambda x, y: 3e8 * x * y + 2e4 * x - 1e9 * y * y
    return [
        (gel.RefractiveSurface(2e-3, -0.5, (1e3, -2e6), 1.0, 1.52, (1e-3, -2e-3), 0.3,
                               gel.ClearAperture.circle(80e-6), (10e-6, -5e-6)),
         oel.RefractiveSurface(2e-3, -0.5, (1e3, -2e6), 1.0, 1.52, (1e-3, -2e-3), 0.3,
                               oel.ClearAperture.circle(80e-6), (10e-6, -5e-6))),
        (gel.RefractiveSurface(-3e-3, 0.0, (), 1.33, 1.0, (0.0, 0.0), None,
                               gel.ClearAperture.rectangle(70e-6, 60e-6)),
         oel.RefractiveSurface(-3e-3, 0.0, (), 1.33, 1.0, (0.0, 0.0), None,
                               oel.ClearAperture.rectangle(70e-6, 60e-6))),
        (gel.Wedge(0.01, 1.45, 1e-4, 0.7, gel.ClearAperture.ellipse(70e-6, 50e-6), (0.0, 8e-6)),
         oel.Wedge(0.01, 1.45, 1e-4, 0.7, oel.ClearAperture.ellipse(70e-6, 50e-6), (0.0, 8e-6))),
        (gel.Wedge(-0.02, 1.6, 5e-5, 0.0), oel.Wedge(-0.02, 1.6, 5e-5, 0.0)),
        (gel.PhaseMask.new(prof, 0.2, gel.ClearAperture.circle(85e-6)),
         oel.PhaseMask(prof, 0.2, oel.ClearAperture.circle(85e-6))),
        # thick lenses (element.rs:2159-2360): biconvex spheres, and an asphere
        # against a conic, rotated, off-centre, elliptical stop, dispersive glass
        (gel.ThickLens(gel.SurfaceProfile.spherical(2e-3), gel.SurfaceProfile.spherical(-3e-3),
                       1.52, 40e-6, None, gel.ClearAperture.circle(80e-6)),
         oel.ThickLens(oel.SurfaceProfile.spherical(2e-3), oel.SurfaceProfile.spherical(-3e-3),
                       1.52, 40e-6, None, oel.ClearAperture.circle(80e-6))),
        (gel.ThickLens(gel.SurfaceProfile(1.5e-3, -0.6, (2e3, -1e6)),
                       gel.SurfaceProfile(-4e-3, 0.3), lambda lam: 1.45 + 4e-15 / lam ** 2, 25e-6,
                       0.4, gel.ClearAperture.ellipse(70e-6, 50e-6), (3e-6, -4e-6)),
         oel.ThickLens(oel.SurfaceProfile(1.5e-3, -0.6, (2e3, -1e6)),
                       oel.SurfaceProfile(-4e-3, 0.3), lambda lam: 1.45 + 4e-15 / lam ** 2, 25e-6,
                       0.4, oel.ClearAperture.ellipse(70e-6, 50e-6), (3e-6, -4e-6))),
    ]


@pytest.mark.parametrize("prec,tol", [("f64", 1e-14), ("f32", 2e-6)])
def test_grid_screens_match_oracle(prec, tol):
    n = 48
    ob = ofield.BandField(rng_field(n, n, 12), 4e-6, 4e-6, 600e-9)
    for ge, oe in screen_pairs():
        ref = oe.apply(ob).samples
        out = ge.apply(to_gpu_band(ob), prec).samples
        assert np.array_equal(out == 0, ref == 0), type(ge).__name__
        assert np.max(np.abs(out - ref)) <= tol * np.max(np.abs(ref)), type(ge).__name__


@pytest.mark.parametrize("prec,tol", [("f64", TOL64), ("f32", TOL32)])
def test_refractive_surface_fused_in_beamline(prec, tol):
    n, d, lam = 96, 4e-6, 532e-9
    ob = ofield.plane_wave(0.0, 0.0, 1.0, n, n, d, d, lam)
    obl_ = obl.Beamline()
    obl_.push(oel.RefractiveSurface(5e-3, -1.0, (), 1.0, 1.5, (0.0, 0.0), None,
                                    oel.ClearAperture.circle(150e-6)), 3e-3)
    ref = obl_.trace(ob, obl.asm_engine(oasm.AsmConfig()))
    gbl = Beamline()
    gbl.push(gel.RefractiveSurface(5e-3, -1.0, (), 1.0, 1.5, (0.0, 0.0), None,
                                   gel.ClearAperture.circle(150e-6)), 3e-3)
    out = gbl.trace(to_gpu_band(ob), AsmEngine(gasm.AsmConfig(), prec))
    assert rel_l2(out.samples, ref.samples) <= tol


@pytest.mark.parametrize("shape", [(8, 8), (37, 45), (64, 128), (101, 97), (256, 256),
                                   (512, 384)])
def test_fft2_matches_numpy_convention(shape):
    """fft::fft2 / ifft2 (fft.rs:40-108): NumPy scaling and sign, any sizes."""
    from optics_studio_gb300.propagation import fft as gfft
    rng = np.random.default_rng(sum(shape))
    u = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    for prec, tol in (("f64", 1e-13), ("f32", 1e-6)):
        assert rel_l2(gfft.fft2(u, prec), np.fft.fft2(u)) <= tol
        assert rel_l2(gfft.ifft2(u, prec), np.fft.ifft2(u)) <= tol
        assert rel_l2(gfft.ifft2(gfft.fft2(u, prec), prec), u) <= 2 * tol


def test_fft2_device_and_delta():
    """Device entry point on resident buffers; a delta transforms to ones."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    from optics_studio_gb300 import _ffi as ffi
    n = 128
    d = torch.zeros((n, n), dtype=torch.complex64, device="cuda")
    d[0, 0] = 1.0
    out = torch.empty_like(d)
    ffi.check(og.lib().osgpu_fft2_device(d.data_ptr(), out.data_ptr(), ffi.C64, n, n, 0, None))
    torch.cuda.synchronize()
    assert torch.allclose(out, torch.ones_like(out), atol=1e-6)


def test_device_sources_match_oracle():
    """sources::gaussian (sources.rs:259-296), BandField::plane_wave / uniform
    (field.rs:315-386) written on the device."""
    torch = pytest.importorskip("torch")
    from optics_studio_gb300 import sources as gsrc
    n, m, d, lam = 96, 80, 3e-6, 633e-9
    cases = [
        (gsrc.gaussian(60e-6, 1.3, (12e-6, -7e-6), 2e-3, lam, n, m, d, d),
         ofield.gaussian(60e-6, 1.3, (12e-6, -7e-6), 2e-3, lam, n, m, d, d).samples),
        (gsrc.gaussian(40e-6, 1.0, (0.0, 0.0), 0.0, lam, n, m, d, d),
         ofield.gaussian(40e-6, 1.0, (0.0, 0.0), 0.0, lam, n, m, d, d).samples),
        (gsrc.plane_wave(0.01, -0.02, 0.7, n, m, d, d, lam),
         ofield.plane_wave(0.01, -0.02, 0.7, n, m, d, d, lam).samples),
        (gsrc.uniform(2.0, 0.3, n, m, d, d, lam),
         ofield.uniform(2.0, 0.3, n, m, d, d, lam).samples),
    ]
    for got, want in cases:
        assert rel_l2(got.cpu().numpy(), want) <= 1e-14
    g32 = gsrc.gaussian(60e-6, 1.3, (12e-6, -7e-6), 2e-3, lam, n, m, d, d, torch.complex64)
    assert rel_l2(g32.cpu().numpy().astype(np.complex128), cases[0][1]) <= 1e-7
    with pytest.raises(og.OsgpuError) as e:
        gsrc.gaussian(-1.0, 1.0, (0.0, 0.0), 0.0, lam, n, m, d, d)
    assert e.value.variant == "BadArgument"
