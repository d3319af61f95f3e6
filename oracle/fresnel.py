"""Fresnel propagation, transfer-function and convolution forms (oracle; test
infrastructure only).

Restates ``src/propagation/fresnel.rs``: FresnelConfig defaults (113-123),
``transfer_value`` (258-262), ``worst_axis_step`` (267-274),
``worst_paraxial_error`` (280-287), ``worst_kernel_axis_step`` (293-298),
``impulse_response`` (312-338), ``analyze`` (342-373), ``validate``
(395-411), ``propagate`` (430-509), ``propagate_convolution`` (531-590).
"""

import math
from dataclasses import dataclass

import numpy as np

from .fft import fft2, ifft2, fftfreq, padded_len, embed_centered, crop_centered

PI = math.pi


@dataclass(frozen=True)
class FresnelConfig:
    padding: float = 2.0
    strict: bool = True
    max_padding: float = 8.0


@dataclass(frozen=True)
class FresnelSamplingReport:
    lam: float
    z: float
    input_dims: tuple
    pitch: tuple
    requested_padding: float
    used_padding: float
    padded_dims: tuple
    max_phase_step_x: float
    max_phase_step_y: float
    nyquist_ok: bool
    max_kernel_step_x: float
    max_kernel_step_y: float
    kernel_nyquist_ok: bool
    max_phase_error_vs_asm: float
    paraxial_ok: bool


class FresnelError(Exception):
    def __init__(self, variant, value=None, report=None):
        super().__init__(f"{variant}({value if report is None else report})")
        self.variant = variant
        self.value = value
        self.report = report


def worst_axis_step(n_pad, d, lam, z):
    df = 1.0 / (float(n_pad) * d)
    f_nyq = float(n_pad // 2) * df
    hi = max(math.floor(f_nyq / df), 0.0) * df
    lo = max(hi - df, 0.0)
    return PI * lam * abs(z) * (hi * hi - lo * lo)


def worst_paraxial_error(dx, dy, lam, z):
    fx = 1.0 / (2.0 * dx)
    fy = 1.0 / (2.0 * dy)
    s = (lam * fx) * (lam * fx) + (lam * fy) * (lam * fy)
    k = 2.0 * PI / lam
    return k * abs(z) * (1.0 - 0.5 * s - math.sqrt(max(1.0 - s, 0.0)))


def worst_kernel_axis_step(n_pad, d, lam, z):
    hi = float(n_pad // 2) * d
    lo = hi - d
    return PI * (hi * hi - lo * lo) / (lam * abs(z))


def analyze(band, z, cfg, padding):
    nx, ny = band.nx, band.ny
    dx, dy = band.dx, band.dy
    lam = band.lam
    nx_pad = padded_len(nx, padding)
    ny_pad = padded_len(ny, padding)
    sx = worst_axis_step(nx_pad, dx, lam, z)
    sy = worst_axis_step(ny_pad, dy, lam, z)
    kx = worst_kernel_axis_step(nx_pad, dx, lam, z)
    ky = worst_kernel_axis_step(ny_pad, dy, lam, z)
    err = worst_paraxial_error(dx, dy, lam, z)
    return FresnelSamplingReport(lam, z, (nx, ny), (dx, dy), cfg.padding, padding,
                                 (nx_pad, ny_pad), sx, sy, sx < PI and sy < PI, kx, ky,
                                 kx < PI and ky < PI, err, err < 0.01)


def sampling_report(band, z, cfg):
    return analyze(band, z, cfg, cfg.padding)


def validate(band, z):
    if not math.isfinite(z):
        raise FresnelError("InvalidDistance", z)
    if not math.isfinite(band.lam) or band.lam <= 0.0:
        raise FresnelError("InvalidWavelength", band.lam)
    if band.nx == 0 or band.ny == 0:
        raise FresnelError("EmptyGrid")
    if not np.all(np.isfinite(band.samples)):
        raise FresnelError("NonFiniteSample")


def resolve_report_tf(band, z, cfg):
    """Validation + densification ladder of ``propagate`` (fresnel.rs:430-451)."""
    validate(band, z)
    if z == 0.0:
        return None
    report = analyze(band, z, cfg, cfg.padding)
    if cfg.strict and not report.nyquist_ok:
        padding = cfg.padding
        while not report.nyquist_ok and padding < cfg.max_padding:
            padding = min(padding * 2.0, cfg.max_padding)
            report = analyze(band, z, cfg, padding)
        if not report.nyquist_ok:
            raise FresnelError("AliasingRisk", report=report)
    return report


def resolve_report_conv(band, z, cfg):
    """Validation + kernel gate of ``propagate_convolution`` (fresnel.rs:531-552)."""
    validate(band, z)
    if z == 0.0:
        return None
    report = analyze(band, z, cfg, cfg.padding)
    if cfg.strict and not report.kernel_nyquist_ok:
        raise FresnelError("AliasingRisk", report=report)
    return report


def transfer_function(nx_pad, ny_pad, dx, dy, lam, z):
    """H_F = e^{i(kz - pi lam z (fx^2 + fy^2))} (fresnel.rs:258-262)."""
    fx = fftfreq(nx_pad, dx)[None, :]
    fy = fftfreq(ny_pad, dy)[:, None]
    k = 2.0 * PI / lam
    phase = k * z - PI * lam * z * (fx * fx + fy * fy)
    return np.exp(1j * phase)


def dft_order_coords(n, d):
    """``coord`` closure of fresnel.rs:322-328: i*d for i <= n/2, else (i-n)*d."""
    i = np.arange(n, dtype=np.float64)
    return np.where(np.arange(n) <= n // 2, i * d, (i - float(n)) * d)


def impulse_response(nx_pad, ny_pad, dx, dy, lam, z):
    """Sampled paraxial kernel in DFT order with dx dy folded in (fresnel.rs:312-338)."""
    k = 2.0 * PI / lam
    pref = complex(math.cos(k * z), math.sin(k * z)) / (1j * lam * z) * (dx * dy)
    x = dft_order_coords(nx_pad, dx)[None, :]
    y = dft_order_coords(ny_pad, dy)[:, None]
    return pref * np.exp(1j * (PI * (x * x + y * y) / (lam * z)))


def propagate(band, z, cfg=FresnelConfig()):
    """``fresnel::propagate`` (fresnel.rs:430-509)."""
    report = resolve_report_tf(band, z, cfg)
    if report is None:
        return band.with_samples(band.samples.copy())
    nx_pad, ny_pad = report.padded_dims
    buf, ox, oy = embed_centered(band.samples, nx_pad, ny_pad)
    spec = fft2(buf) * transfer_function(nx_pad, ny_pad, band.dx, band.dy, band.lam, z)
    res = crop_centered(ifft2(spec), band.nx, band.ny, ox, oy)
    if not np.all(np.isfinite(res)):
        raise FresnelError("NonFiniteSample")
    return band.with_samples(res)


def propagate_convolution(band, z, cfg=FresnelConfig()):
    """``fresnel::propagate_convolution`` (fresnel.rs:531-590)."""
    report = resolve_report_conv(band, z, cfg)
    if report is None:
        return band.with_samples(band.samples.copy())
    nx_pad, ny_pad = report.padded_dims
    buf, ox, oy = embed_centered(band.samples, nx_pad, ny_pad)
    h = impulse_response(nx_pad, ny_pad, band.dx, band.dy, band.lam, z)
    spec = fft2(buf) * fft2(h)
    res = crop_centered(ifft2(spec), band.nx, band.ny, ox, oy)
    if not np.all(np.isfinite(res)):
        raise FresnelError("NonFiniteSample")
    return band.with_samples(res)
