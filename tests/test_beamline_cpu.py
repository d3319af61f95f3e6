"""Beamline composition (src/beamline.rs:52-145) on the CPU: the reference's
beamline unit tests restated for the oracle's Beamline and for the
product's host-side Beamline driven by an engine closure (the step order,
zero-distance skips, the medium handed to the closure, error pass-through).
Element application runs on the device, so the product's cases here use
gaps only; the element paths are covered by the GPU parity tests."""

import math

import numpy as np
import pytest

from oracle import asm as oasm, beamline as obl, element as oel, field as ofield

LAMBDA = 500e-9


class Boom(Exception):
    pass


def band(n=64, d=1e-3):
    return ofield.uniform(1.0, 0.0, n, n, d, d, LAMBDA)


def product_band(n=64, d=1e-3):
    from optics_studio_gb300.field import BandField
    b = band(n, d)
    return BandField(b.samples, b.dx, b.dy, b.lam)


def boom(*_):
    raise Boom()


@pytest.mark.parametrize("side", ["oracle", "product"])
def test_empty_gap_only_and_engine_errors(side):
    """beamline.rs empty_beamline_is_the_identity, gap_only_beamline_and_len,
    engine_errors_surface_untouched, zero_spacing_skips_the_engine."""
    if side == "oracle":
        make, b = obl.Beamline, band()
    else:
        from optics_studio_gb300.beamline import Beamline as make
        b = product_band()
    out = make().trace(b, boom)
    np.testing.assert_array_equal(out.samples, b.samples)
    bl = make()
    bl.gap(0.0, 2.0)
    calls = []
    out = bl.trace(b, lambda x, z, m: calls.append((z, m)) or x)
    assert calls == [] and len(bl.steps) == 1
    np.testing.assert_array_equal(out.samples, b.samples)
    bl = make()
    bl.gap(0.1, 1.0)
    with pytest.raises(Boom):
        bl.trace(b, boom)
    bl = make()
    bl.gap(0.0, 1.0).gap(0.05, 1.0)
    calls = []
    bl.trace(b, lambda x, z, m: calls.append((z, m)) or x)
    assert calls == [(0.05, 1.0)]


@pytest.mark.parametrize("side", ["oracle", "product"])
def test_medium_reaches_the_engine_closure_per_step(side):
    """beamline.rs medium_reaches_the_engine_closure_per_step: the closure sees
    (1 mm, 1.5) then (0.5 mm, 1.0); zero gaps are skipped."""
    if side == "oracle":
        make, b = obl.Beamline, band(16, 20e-6)
    else:
        from optics_studio_gb300.beamline import Beamline as make
        b = product_band(16, 20e-6)
    seen = []
    bl = make()
    bl.gap(1e-3, 1.5).gap(0.5e-3, 1.0).gap(0.0, 1.5)
    bl.trace(b, lambda x, z, m: seen.append((z, m)) or x)
    assert seen == [(1e-3, 1.5), (0.5e-3, 1.0)]


def test_oracle_trace_matches_manual_chain_and_slab_piston():
    """beamline.rs trace_matches_manual_chain_bit_for_bit,
    medium_reaches_the_engine_closure_per_step (the slab piston
    e^{i k (1.5 * 1 mm + 0.5 mm)} to 1e-9), element_errors_surface_typed."""
    stop = oel.EllipticalAperture.circle(4e-3)
    lens = oel.ThinLens.fixed(0.2)
    rect = oel.RectangularAperture((3e-3, 2e-3))
    cfg = oasm.AsmConfig()
    bl = obl.Beamline()
    bl.push(stop, 0.1).push(lens, 0.2).push(rect, 0.0)
    traced = bl.trace(band(), lambda b, z, m: oasm.propagate(b, z, cfg)).samples
    m = stop.apply(band())
    m = oasm.propagate(m, 0.1, cfg)
    m = lens.apply(m)
    m = oasm.propagate(m, 0.2, cfg)
    m = rect.apply(m)
    np.testing.assert_array_equal(traced, m.samples)

    b = band(16, 20e-6)
    bl = obl.Beamline()
    bl.gap(1e-3, 1.5).gap(0.5e-3, 1.0).push_medium(oel.EllipticalAperture.circle(120e-6), 0.0,
                                                    1.5)
    out = bl.trace(b, lambda x, z, m: oasm.propagate(x, z, oasm.AsmConfig(padding=1.0, medium=m)))
    k = 2.0 * math.pi / LAMBDA
    want = np.exp(1j * k * (1.5 * 1e-3 + 1.0 * 0.5e-3))
    assert abs(out.samples[9, 3] / b.samples[9, 3] - want) < 1e-9

    bl = obl.Beamline()
    bl.push(oel.EllipticalAperture.circle(40e-3), 0.0)
    with pytest.raises(Exception) as e:
        bl.trace(band(), lambda x, z, m: x)
    assert "OutsideField" in str(e.value) or getattr(e.value, "variant", "") == "OutsideField"


def test_sum_intensity_matches_reference_tests():
    """field.rs sum_intensity_adds_powers_without_cross_terms (|1|^2 + |2|^2 = 5
    per sample, powers add, phases do not matter) and sum_intensity_validation."""
    from optics_studio_gb300.field import BandField, sum_intensity

    def band_at(a, phase, lam, d=1e-3):
        return BandField(np.full((4, 4), a * np.exp(1j * phase)), d, d, lam)

    red, blue = band_at(1.0, 0.0, 650e-9), band_at(2.0, math.pi / 3.0, 450e-9)
    s = sum_intensity([red, blue])
    assert float(np.max(np.abs(s.samples - 5.0))) < 1e-15
    assert abs(s.total_power() - (red.power() + blue.power())) < 1e-15
    np.testing.assert_array_equal(s.samples,
                                  sum_intensity([red, band_at(2.0, -1.2, 450e-9)]).samples)
    assert abs(sum_intensity([red, red]).total_power() - 2.0 * red.power()) < 1e-15
    with pytest.raises(ValueError, match="EmptyGrid"):
        sum_intensity([])
    with pytest.raises(ValueError, match="GeometryMismatch"):
        sum_intensity([red, band_at(1.0, 0.0, 650e-9, 2e-3)])
    bad = band_at(1.0, 0.0, 650e-9)
    bad.samples[1, 1] = complex(math.nan, 0.0)
    with pytest.raises(ValueError, match="NonFiniteSample"):
        sum_intensity([bad])
