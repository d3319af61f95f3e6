"""The reference's physical validation suites, on the oracle and on the device.

Each test restates one analytic check of tests/phase2.rs (Gaussian beam width
and Gouy phase, straight-edge Fresnel integrals, rectangular-aperture sinc^2,
Airy pattern across three engines), tests/phase3.rs (blazed-grating orders)
or tests/phase4.rs (Rayleigh-Sommerfeld against direct quadrature, ASM,
back-propagation, Fresnel divergence, power), with the reference's
geometries and tolerances.  The ``oracle`` parameter pins the f64
restatement on the CPU; ``f64`` and ``f32`` run the same geometry through
the product's engines and elements on the GPU.  The analytic helpers follow
tests/common/mod.rs (J1 and the Fresnel integrals from scipy.special).
"""

import math

import numpy as np
import pytest
from scipy import signal, special

from oracle import asm as oasm, fraunhofer as ofh, fresnel as ofr, rs as ors
from oracle import element as oel, field as ofield

from _util import to_gpu_band

LAMBDA = 500e-9
BACKENDS = ["oracle", pytest.param("f64", marks=pytest.mark.gpu),
            pytest.param("f32", marks=pytest.mark.gpu)]


def _engines(backend):
    if backend == "oracle":
        return {"asm": (oasm.propagate, oasm.AsmConfig),
                "fresnel": (ofr.propagate, ofr.FresnelConfig),
                "fresnel_conv": (ofr.propagate_convolution, ofr.FresnelConfig),
                "fraunhofer": (ofh.propagate, ofh.FraunhoferConfig),
                "rs": (ors.propagate, ors.RayleighSommerfeldConfig)}
    from optics_studio_gb300.propagation import asm, fraunhofer, fresnel, rayleigh_sommerfeld
    return {"asm": (asm.propagate, asm.AsmConfig),
            "fresnel": (fresnel.propagate, fresnel.FresnelConfig),
            "fresnel_conv": (fresnel.propagate_convolution, fresnel.FresnelConfig),
            "fraunhofer": (fraunhofer.propagate, fraunhofer.FraunhoferConfig),
            "rs": (rayleigh_sommerfeld.propagate, rayleigh_sommerfeld.RayleighSommerfeldConfig)}


def prop(backend, engine, band, z, **cfg):
    """Propagates the oracle band `band` with `engine` on `backend`; the
    result has .samples, .dx, .dy."""
    fn, conf = _engines(backend)[engine]
    if backend == "oracle":
        return fn(band, z, conf(**cfg))
    return fn(to_gpu_band(band), z, conf(**cfg), backend)


def apply(backend, make, band):
    """Applies the element make(module) (module: the oracle's or the
    product's element module, which share constructor names) to `band`."""
    if backend == "oracle":
        return make(oel).apply(band)
    from optics_studio_gb300 import element
    out = make(element).apply(to_gpu_band(band), backend)
    return ofield.BandField(out.samples, out.dx, out.dy, out.lam)


def gaussian_band(n, d, sigma):
    """common/mod.rs:21-33: exp(-(x^2 + y^2) / 2 sigma^2) on a centred grid."""
    c = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * d
    u = np.exp(-(c[None, :] ** 2 + c[:, None] ** 2) / (2.0 * sigma * sigma))
    return ofield.BandField(u.astype(np.complex128), d, d, LAMBDA)


def wrap_phase(d):
    return (d + math.pi) % (2.0 * math.pi) - math.pi


def rel_frobenius(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def coords(n, d):
    return (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * d


# ---- tests/phase2.rs -------------------------------------------------------------

@pytest.mark.parametrize("backend", BACKENDS)
def test_gaussian_beam_width_and_gouy_match_analytics(backend):
    """phase2.rs:56-132: width w(z), on-axis amplitude w0/w(z) and Gouy phase
    (1e-3) for ASM and Fresnel TF, and the two engines within 1e-3."""
    n, d, sigma, z = 255, 1e-5, 0.15e-3, 0.1
    band = gaussian_band(n, d, sigma)
    w0 = math.sqrt(2.0) * sigma
    z_r = math.pi * w0 * w0 / LAMBDA
    w_z = w0 * math.sqrt(1.0 + (z / z_r) ** 2)
    gouy = math.atan(z / z_r)
    k = 2.0 * math.pi / LAMBDA
    outs = {"asm": prop(backend, "asm", band, z), "fresnel": prop(backend, "fresnel", band, z)}
    x = coords(n, d)[None, :]
    for label, out in outs.items():
        i = np.abs(out.samples) ** 2
        s0, s2 = float(np.sum(i)), float(np.sum(i * x * x))
        sigma_meas = math.sqrt(2.0 * s2 / s0)
        sigma_exp = w_z / math.sqrt(2.0)
        assert abs(sigma_meas - sigma_exp) / sigma_exp < 1e-3, label
        c = out.samples[n // 2, n // 2]
        amp_exp = w0 / w_z
        assert abs(abs(c) - amp_exp) / amp_exp < 1e-3, label
        assert abs(wrap_phase(np.angle(c) - (k * z - gouy))) < 1e-3, label
    assert rel_frobenius(outs["asm"].samples, outs["fresnel"].samples) < 1e-3


@pytest.mark.parametrize("backend", BACKENDS)
def test_straight_edge_matches_fresnel_integrals(backend):
    """phase2.rs:134-172: a half plane after 2 mm (Fresnel TF) against the
    Fresnel-integral profile, within 2.5 % of I0 over |x| <= 0.2 mm."""
    n, d, z = 2048, 1e-6, 2e-3
    x = coords(n, d)
    u0 = np.ones((n, n), dtype=np.complex128)
    u0[:, x > 0.0] = 0.0
    out = prop(backend, "fresnel", ofield.BandField(u0, d, d, LAMBDA), z)
    sel = np.abs(x) <= 0.2e-3
    u = x[sel] * math.sqrt(2.0 / (LAMBDA * z))
    s, c = special.fresnel(u)
    i_exp = 0.5 * ((0.5 - c) ** 2 + (0.5 - s) ** 2)
    i_num = np.abs(out.samples[n // 2, sel]) ** 2
    assert float(np.max(np.abs(i_num - i_exp))) < 0.025


@pytest.mark.parametrize("backend", BACKENDS)
def test_rectangular_aperture_sinc2_far_field(backend):
    """phase2.rs:185-251: a 0.2 mm square in the Fraunhofer far field at 1 m
    against sinc^2, within 3 % of the peak out to |X| <= 4 mm."""
    n, d, a, z = 2048, 1e-5, 1e-4, 1.0
    x = coords(n, d)
    inside = (np.abs(x)[None, :] <= a) & (np.abs(x)[:, None] <= a)
    u0 = np.where(inside, 1.0 + 0.0j, 0.0j)
    out = prop(backend, "fraunhofer", ofield.BandField(u0, d, d, LAMBDA), z, aperture_extent=a)
    dxo = LAMBDA * z / (n * d)
    assert out.dx == pytest.approx(dxo, rel=1e-12)
    i = np.abs(out.samples) ** 2
    peak = float(np.max(i))
    xo = coords(n, dxo)
    sel = np.abs(xo) <= 4.0e-3
    arg = math.pi * 2.0 * a * xo[sel] / (LAMBDA * z)
    sinc = np.where(np.abs(arg) < 1e-12, 1.0, np.sin(arg) / np.where(arg == 0, 1.0, arg))
    assert float(np.max(np.abs(i[n // 2, sel] / peak - sinc ** 2))) < 0.03


def airy(v):
    v = np.asarray(v, dtype=np.float64)
    safe = np.where(np.abs(v) < 1e-8, 1.0, v)
    return np.where(np.abs(v) < 1e-8, 1.0 - v * v / 3.0, (2.0 * special.j1(safe) / safe) ** 2)


def row_profile(samples, dx, x_max, half_rows, analytic):
    """phase2.rs:23-44: mean |U|^2 over 2 half_rows + 1 centre rows, |x| <= x_max."""
    ny, nx = samples.shape
    iy0 = ny // 2
    x = coords(nx, dx)
    sel = np.abs(x) <= x_max
    rows = np.abs(samples[iy0 - half_rows:iy0 + half_rows + 1, :][:, sel]) ** 2
    r = np.abs(x[sel])
    return r, rows.mean(axis=0), analytic(r)


@pytest.mark.parametrize("backend", BACKENDS)
def test_airy_pattern_across_all_three_engines(backend):
    """phase2.rs:253-323: a 1 mm circular aperture at 40 m through Fraunhofer
    (3 %), Fresnel convolution at padding 1 (2 %) and ASM (2 %) against
    [2 J1(v)/v]^2; the Fresnel TF chirp is undersampled here while the
    convolution kernel is not."""
    n, d, a, z = 2048, 2e-5, 1e-3, 40.0
    band = ofield.uniform(1.0, 0.0, n, n, d, d, LAMBDA)
    masked = apply(backend, lambda m: m.EllipticalAperture.circle(a), band)
    k = 2.0 * math.pi / LAMBDA
    if backend == "oracle":
        rep = ofr.sampling_report(masked, z, ofr.FresnelConfig())
    else:
        from optics_studio_gb300.propagation import fresnel
        rep = fresnel.sampling_report(to_gpu_band(masked), z, fresnel.FresnelConfig())
    assert not bool(rep.nyquist_ok) and bool(rep.kernel_nyquist_ok)
    runs = [("fraunhofer", prop(backend, "fraunhofer", masked, z, aperture_extent=a), 0.03),
            ("fresnel_conv", prop(backend, "fresnel_conv", masked, z, padding=1.0, strict=True,
                                  max_padding=1.0), 0.02),
            ("asm", prop(backend, "asm", masked, z), 0.02)]
    for label, out, tol in runs:
        r, i, a_exp = row_profile(out.samples, out.dx, 12.6e-3, 2, lambda r: airy(k * a * r / z))
        err = np.abs(i / np.max(i) - a_exp / np.max(a_exp))
        assert float(np.max(err)) < tol, (label, float(np.max(err)))


# ---- tests/phase3.rs -------------------------------------------------------------
N3, PITCH3, PERIOD3, STOP3, Z3 = 512, 20e-6, 102.4e-6, 512e-6, 0.6
BINS_PER_ORDER = N3 * PITCH3 / PERIOD3  # 100 output bins between orders


def order_bins(m):
    return (N3 - 1.0) / 2.0 + m * BINS_PER_ORDER


def blaze_profile(backend, depth):
    """phase3.rs:41-69: the column-integrated far field of a uniform band
    behind a blazed grating with a circular stop (Fraunhofer, 0.6 m)."""
    band = ofield.uniform(1.0, 0.0, N3, N3, PITCH3, PITCH3, LAMBDA)
    masked = apply(backend, lambda m: m.BlazedGrating(PERIOD3, depth, 0.0,
                                                      m.ClearAperture.circle(STOP3)), band)
    out = prop(backend, "fraunhofer", masked, Z3, aperture_extent=STOP3)
    return out, np.sum(np.abs(out.samples) ** 2, axis=0)


def power_in_window(profile, center, half):
    lo = max(0, int(math.ceil(center - half)))
    hi = min(len(profile) - 1, int(math.floor(center + half)))
    return float(np.sum(profile[lo:hi + 1]))


@pytest.mark.parametrize("backend", BACKENDS)
def test_blazed_grating_orders(backend):
    """phase3.rs:78-150: depth 2 pi steers > 85 % into order +1 at
    lambda z / period (peak within 2 bins, orders 0 and -1 below 3 %);
    depth 4 pi puts > 80 % into order +2; depth pi splits orders 0 and +1
    (each 30-55 %, within 5 % of each other, order -1 below 10 %)."""
    out, prof = blaze_profile(backend, 2.0 * math.pi)
    peak = int(np.argmax(prof))
    assert abs(peak - order_bins(1.0)) <= 2.0
    x_peak = coords(N3, out.dx)[peak]
    x_1 = LAMBDA * Z3 / PERIOD3
    assert abs(x_peak - x_1) <= 2.0 * (x_1 / BINS_PER_ORDER)
    frac = lambda p, m: power_in_window(p, order_bins(m), 40.0) / float(np.sum(p))
    assert frac(prof, 1.0) > 0.85 and frac(prof, 0.0) < 0.03 and frac(prof, -1.0) < 0.03

    _, prof2 = blaze_profile(backend, 4.0 * math.pi)
    assert abs(int(np.argmax(prof2)) - order_bins(2.0)) <= 2.0
    assert frac(prof2, 2.0) > 0.8

    _, profh = blaze_profile(backend, math.pi)
    f0, f1, fm1 = frac(profh, 0.0), frac(profh, 1.0), frac(profh, -1.0)
    assert 0.30 < f0 < 0.55 and 0.30 < f1 < 0.55
    assert abs(f0 - f1) < 0.05 and fm1 < 0.10


# ---- tests/phase4.rs -------------------------------------------------------------

def rs_direct(band, z):
    """common/mod.rs:35-90: the linear convolution of the band with the RS-I
    impulse response (|z| / 2 pi r^2)(1/r - i sgn(z) k) e^{i sgn(z) k r} dx dy,
    summed directly over the window."""
    ny, nx = band.samples.shape
    k = 2.0 * math.pi / band.lam
    s = 1.0 if z >= 0.0 else -1.0
    az = abs(z)
    xx = (np.arange(2 * nx - 1) - (nx - 1.0)) * band.dx
    yy = (np.arange(2 * ny - 1) - (ny - 1.0)) * band.dy
    r = np.sqrt(xx[None, :] ** 2 + yy[:, None] ** 2 + az * az)
    obliq = az / (2.0 * math.pi * r ** 3) - 1j * s * k * az / (2.0 * math.pi * r * r)
    tab = obliq * np.exp(1j * s * k * r) * (band.dx * band.dy)
    full = signal.convolve2d(band.samples, tab, mode="full")
    return full[ny - 1:2 * ny - 1, nx - 1:2 * nx - 1]


ZA, ZB = 2e-3, 3e-3


def band_a():
    return gaussian_band(48, 2e-6, 10e-6)


def band_b(backend):
    flat = ofield.uniform(1.0, 0.0, 32, 32, 4e-6, 4e-6, LAMBDA)
    return apply(backend, lambda m: m.EllipticalAperture.circle(20e-6), flat)


def rs_report(backend, band, z):
    if backend == "oracle":
        return ors.sampling_report(band, z, ors.RayleighSommerfeldConfig(2.0, True))
    from optics_studio_gb300.propagation import rayleigh_sommerfeld as rs
    return rs.sampling_report(to_gpu_band(band), z, rs.RayleighSommerfeldConfig(2.0, True))


@pytest.mark.parametrize("backend", BACKENDS)
def test_rs_matches_direct_quadrature_asm_and_back_propagation(backend):
    """phase4.rs:63-125, 185-208: on a paraxial Gaussian (48^2, 2 um, z 2 mm)
    the RS engine is within 1e-2 of direct quadrature, RS and direct within
    2e-2 of ASM, +z then -z recovers the field within 3e-2, and RS and ASM
    conserve power within 1e-3."""
    band = band_a()
    assert bool(rs_report(backend, band, ZA).kernel_nyquist_ok)
    rs = prop(backend, "rs", band, ZA, padding=2.0, strict=True).samples
    asm = prop(backend, "asm", band, ZA).samples
    direct = rs_direct(band, ZA)
    assert rel_frobenius(rs, direct) < 1e-2
    assert rel_frobenius(rs, asm) < 2e-2
    assert rel_frobenius(direct, asm) < 2e-2
    fwd = prop(backend, "rs", band, ZA, padding=2.0, strict=True)
    fwd_o = ofield.BandField(fwd.samples, fwd.dx, fwd.dy, LAMBDA)
    rt = prop(backend, "rs", fwd_o, -ZA, padding=2.0, strict=True).samples
    assert rel_frobenius(rt, band.samples) < 3e-2
    p0 = float(np.sum(np.abs(band.samples) ** 2))
    assert abs(float(np.sum(np.abs(rs) ** 2)) - p0) / p0 < 1e-3
    assert abs(float(np.sum(np.abs(asm) ** 2)) - p0) / p0 < 1e-3


@pytest.mark.parametrize("backend", BACKENDS)
def test_fresnel_diverges_where_reported_error_says(backend):
    """phase4.rs:144-183: behind a 20 um circular aperture at 3 mm the
    Fresnel report flags the paraxial truncation (0.1-0.6 rad); RS stays
    within 2e-2 of direct quadrature while Fresnel TF errs by more than 4x
    that, but below 0.3."""
    band = band_b(backend)
    assert bool(rs_report(backend, band, ZB).kernel_nyquist_ok)
    truth = rs_direct(band, ZB)
    if backend == "oracle":
        rep = ofr.sampling_report(band, ZB, ofr.FresnelConfig(2.0, True, 8.0))
    else:
        from optics_studio_gb300.propagation import fresnel
        rep = fresnel.sampling_report(to_gpu_band(band), ZB, fresnel.FresnelConfig(2.0, True, 8.0))
    assert not bool(rep.paraxial_ok)
    assert 0.1 < rep.max_phase_error_vs_asm < 0.6
    rs = prop(backend, "rs", band, ZB, padding=2.0, strict=True).samples
    fr = prop(backend, "fresnel", band, ZB, padding=2.0, strict=True, max_padding=8.0).samples
    e_rs, e_fr = rel_frobenius(rs, truth), rel_frobenius(fr, truth)
    assert e_rs < 2e-2
    assert e_fr > 4.0 * e_rs
    assert e_fr < 0.3


# ---- tests/phase5.rs -------------------------------------------------------------

def trace(backend, steps, band, engine, **cfg):
    """A Beamline of steps [(make(module) | None, z_after)] traced with the
    ASM engine (fused on the device) or a Fraunhofer closure."""
    if backend == "oracle":
        from oracle import beamline as obl
        bl = obl.Beamline()
        for make, z in steps:
            bl.push(make(oel) if make else None, z)
        if engine == "asm":
            return bl.trace(band, obl.asm_engine(oasm.AsmConfig(**cfg)))
        return bl.trace(band, lambda b, z, m: ofh.propagate(b, z, ofh.FraunhoferConfig(**cfg)))
    from optics_studio_gb300 import beamline as gbl, element
    from optics_studio_gb300.propagation import asm, fraunhofer
    bl = gbl.Beamline()
    for make, z in steps:
        bl.push(make(element) if make else None, z)
    if engine == "asm":
        return bl.trace(to_gpu_band(band), gbl.AsmEngine(asm.AsmConfig(**cfg), backend))
    return bl.trace(to_gpu_band(band), lambda b, z, m: fraunhofer.propagate(
        b, z, fraunhofer.FraunhoferConfig(**cfg), backend))


def centroid(out):
    """Psf::centroid: the intensity-weighted mean of the centred coordinates."""
    i = np.abs(out.samples) ** 2
    ny, nx = i.shape
    s = float(np.sum(i))
    return (float(np.sum(i * coords(nx, out.dx)[None, :])) / s,
            float(np.sum(i * coords(ny, out.dy)[:, None])) / s)


@pytest.mark.parametrize("backend", BACKENDS)
def test_psf_of_circular_aperture_is_airy(backend):
    """phase5.rs:21-86: a 0.5 mm stop, Fraunhofer to 2 m: output pitch
    lambda z / (n d), centre row within 3 % of the Airy profile (2 % on the
    central lobe), first dark ring within 2 bins of 1.22 lambda z / 2a."""
    a, z, n, d = 0.5e-3, 2.0, 256, 25e-6
    band = ofield.uniform(1.0, 0.0, n, n, d, d, LAMBDA)
    out = trace(backend, [(lambda m: m.EllipticalAperture.circle(a), z)], band, "fraunhofer",
                aperture_extent=a)
    psf = np.abs(out.samples) ** 2
    assert psf.shape == (n, n)
    assert abs(out.dx - LAMBDA * z / (n * d)) < 1e-12
    iy = n // 2
    row = psf[iy] / psf[iy, n // 2]
    x = coords(n, out.dx)
    prof = airy(2.0 * math.pi * a * np.abs(x) / (LAMBDA * z))
    assert float(np.max(np.abs(row - prof))) < 0.03
    r1 = 1.22 * LAMBDA * z / (2.0 * a)
    win = np.nonzero((x > 0.6 * r1) & (x < 1.6 * r1))[0]
    xd = x[win[int(np.argmin(psf[iy, win]))]]
    assert abs(xd - r1) < 2.0 * out.dx
    lobe = np.abs(x) <= r1
    assert float(np.max(np.abs(row[lobe] - prof[lobe]))) < 0.02


@pytest.mark.parametrize("backend", BACKENDS)
def test_psf_peak_follows_field_angle(backend):
    """phase5.rs:88-121: a 1 mrad plane wave through a 1.25 mm stop and a
    f = 0.5 m lens (ASM) focuses with its centroid at f tan(theta) (2e-5 m),
    on axis in y (1e-6 m); the untilted wave focuses at the origin."""
    a, f, theta, n, d = 1.25e-3, 0.5, 0.001, 256, 25e-6
    steps = [(lambda m: m.EllipticalAperture.circle(a), 0.0),
             (lambda m: m.ThinLens.fixed(f), f)]
    out = trace(backend, steps, ofield.plane_wave(theta, 0.0, 1.0, n, n, d, d, LAMBDA), "asm")
    cx, cy = centroid(out)
    assert abs(cx - f * math.tan(theta)) < 2e-5
    assert abs(cy) < 1e-6
    out0 = trace(backend, steps, ofield.plane_wave(0.0, 0.0, 1.0, n, n, d, d, LAMBDA), "asm")
    c0x, c0y = centroid(out0)
    assert abs(c0x) < 1e-6 and abs(c0y) < 1e-6


def spherical(src, distance, amplitude, n, d):
    """sources.rs:627-666: A e^{ikr} / r from a point at (src, -distance)."""
    k = 2.0 * math.pi / LAMBDA
    x = coords(n, d)[None, :] - src[0]
    y = coords(n, d)[:, None] - src[1]
    r = np.sqrt(x * x + y * y + distance * distance)
    return ofield.BandField(amplitude * np.exp(1j * k * r) / r, d, d, LAMBDA)


@pytest.mark.parametrize("backend", BACKENDS)
def test_point_source_focuses_at_geometric_image(backend):
    """phase5.rs:123-159: a point 0.5 mm off axis, 0.3 m before a f = 0.1 m
    lens with a 1 mm stop, images at d_i = 0.15 m with the centroid at
    -x_s d_i / d_o (2e-5 m; y within 2e-6 m) and a peak above 10x the mean."""
    x_s, d_o, f, stop, n, d = 0.5e-3, 0.3, 0.1, 1.0e-3, 256, 1e-5
    d_i = f * d_o / (d_o - f)
    src = spherical((x_s, 0.0), d_o, 1e-3, n, d)
    out = trace(backend, [(lambda m: m.ThinLens.fixed(f, None, m.ClearAperture.circle(stop)),
                           d_i)], src, "asm")
    cx, cy = centroid(out)
    assert abs(cx + x_s * d_i / d_o) < 2e-5
    assert abs(cy) < 2e-6
    psf = np.abs(out.samples) ** 2
    assert float(np.max(psf)) > 10.0 * float(np.mean(psf))


# ---- tests/phase6.rs -------------------------------------------------------------
L0 = 550e-9


def radial_phase(samples, kmax):
    """phase6.rs:35-49: unwrapped phase along +x from the sample (n/2, n/2)."""
    c = samples.shape[1] // 2
    a = np.angle(samples[c, c:c + kmax + 1])
    steps = (np.diff(a) + math.pi) % (2.0 * math.pi) - math.pi
    return np.cumsum(steps)


def fit_power(phases, d, k):
    """phase6.rs:51-60: least-squares Phi of phi = -k Phi rho^2 / 2 through 0."""
    x = ((np.arange(len(phases)) + 1.0) * d) ** 2
    return -2.0 * float(np.sum(x * phases) / np.sum(x * x)) / k


@pytest.mark.parametrize("backend", BACKENDS)
def test_thick_stack_focuses_at_back_focal_length(backend):
    """phase6.rs:62-128: two spherical surfaces (R1 = 25 mm, R2 = -100 mm,
    n = 1.5) 5 mm apart in glass, traced with the medium-aware ASM on the
    odd 1021^2 grid (a prime length), focus at the thick-lens back focal
    length within 1 % and measurably away from the thin-lens law."""
    c1, c2, t, n = 40.0, -10.0, 5e-3, 1.5
    phi1, phi2 = (n - 1.0) * c1, (1.0 - n) * c2
    big_phi = phi1 + phi2 - t / n * phi1 * phi2
    bfl = (1.0 - t / n * phi1) / big_phi
    thin = 1.0 / (phi1 + phi2)
    ng, d, a = 1021, 4e-6, 1e-3
    band = ofield.uniform(1.0, 0.0, ng, ng, d, d, L0)
    s1 = lambda m: m.RefractiveSurface(1.0 / c1, n_front=1.0, n_back=n,
                                       aperture=m.ClearAperture.circle(a))
    s2 = lambda m: m.RefractiveSurface(1.0 / c2, n_front=n, n_back=1.0,
                                       aperture=m.ClearAperture.circle(a))
    if backend == "oracle":
        from oracle import beamline as obl
        bl = obl.Beamline()
        bl.push_medium(s1(oel), t, n).push(s2(oel), 0.0)
        out = bl.trace(band, obl.asm_engine(oasm.AsmConfig()))
    else:
        from optics_studio_gb300 import beamline as gbl, element
        from optics_studio_gb300.propagation import asm
        bl = gbl.Beamline()
        bl.push_medium(s1(element), t, n).push(s2(element), 0.0)
        out = bl.trace(to_gpu_band(band), gbl.AsmEngine(asm.AsmConfig(), backend))
    measured = 1.0 / fit_power(radial_phase(out.samples, 24), d, 2.0 * math.pi / L0)
    assert abs(measured - bfl) < 0.01 * bfl
    assert abs(measured - thin) > 0.5 * (thin - bfl)


@pytest.mark.parametrize("backend", BACKENDS)
def test_hybrid_achromat_cancels_first_order_color(backend):
    """phase6.rs:130-188: a dispersive thin lens plus a diffractive screen of
    opposite chromatic slope: total power within 1 % over 500-600 nm, the
    refractive lens alone shifting by more than 4 %, the corrected shift
    below a quarter of the uncorrected one."""
    c_r, a = 0.25, 400e-6
    n_of = lambda lam: 1.4 + 4e-14 / (lam * lam)
    phi_r = lambda lam: (n_of(lam) - 1.0) * c_r
    dphi_r = -2.0 * c_r * 4e-14 / L0 ** 3
    phi_d0 = -L0 * dphi_r
    assert phi_d0 > 0.0
    prof = lambda x, y: -(math.pi * phi_d0 / L0) * (x * x + y * y)

    def doe(m):
        ap = m.ClearAperture.circle(a)
        return m.PhaseMask.new(prof, None, ap) if hasattr(m.PhaseMask, "new") \
            else m.PhaseMask(prof, None, ap)

    def measure(lam, with_doe):
        band = ofield.uniform(1.0, 0.0, 128, 128, 8e-6, 8e-6, lam)
        f = apply(backend, lambda m: m.ThinLens(lambda l: 1.0 / phi_r(l)), band)
        if with_doe:
            f = apply(backend, doe, f)
        return fit_power(radial_phase(f.samples, 50), 8e-6, 2.0 * math.pi / lam)

    p0, p500, p600 = measure(L0, True), measure(500e-9, True), measure(600e-9, True)
    r500, r0 = measure(500e-9, False), measure(L0, False)
    shift = lambda x, y: abs((x - y) / y)
    assert shift(p500, p0) < 0.01 and shift(p600, p0) < 0.01
    assert shift(r500, r0) > 0.04
    assert shift(p500, p0) < 0.25 * shift(r500, r0)


@pytest.mark.parametrize("backend", BACKENDS)
def test_wedge_deflects_toward_the_base(backend):
    """phase6.rs:190-226: a 1 mrad wedge (n = 1.5) behind a 400 um stop,
    Fraunhofer at 2 m: centroid at -(n - 1) tan(alpha) z within 1e-4 m, y
    within 1e-6 m."""
    alpha, z, a = 1e-3, 2.0, 400e-6
    band = ofield.uniform(1.0, 0.0, 128, 128, 20e-6, 20e-6, L0)
    out = trace(backend, [(lambda m: m.Wedge(alpha, 1.5, 1e-3, 0.0, m.ClearAperture.circle(a)),
                           z)], band, "fraunhofer", aperture_extent=a)
    cx, cy = centroid(out)
    assert abs(cx + (1.5 - 1.0) * math.tan(alpha) * z) < 1e-4
    assert abs(cy) < 1e-6
