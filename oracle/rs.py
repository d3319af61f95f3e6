"""Rayleigh-Sommerfeld first-kind propagation (oracle; test infrastructure only).

Restates ``src/propagation/rayleigh_sommerfeld.rs``: config defaults
(107-116), ``kernel_value`` (228-235), ``worst_kernel_axis_step``
(240-249), ``worst_paraxial_excess`` (254-270), ``impulse_response``
(277-301), ``analyze`` (304-329), ``validate`` (345-362), ``propagate``
(384-442).
"""

import math
from dataclasses import dataclass

import numpy as np

from .fft import fft2, ifft2, padded_len, embed_centered, crop_centered
from .fresnel import dft_order_coords

PI = math.pi


@dataclass(frozen=True)
class RayleighSommerfeldConfig:
    padding: float = 2.0
    strict: bool = True


@dataclass(frozen=True)
class RsSamplingReport:
    lam: float
    z: float
    input_dims: tuple
    pitch: tuple
    padding: float
    padded_dims: tuple
    max_kernel_step_x: float
    max_kernel_step_y: float
    kernel_nyquist_ok: bool
    max_phase_error_vs_fresnel: float
    paraxial_ok: bool


class RayleighSommerfeldError(Exception):
    def __init__(self, variant, value=None, report=None):
        super().__init__(f"{variant}({value if report is None else report})")
        self.variant = variant
        self.value = value
        self.report = report


def kernel_value(x, y, lam, z):
    """rayleigh_sommerfeld.rs:228-235 (vectorised)."""
    k = 2.0 * PI / lam
    s = 1.0 if z > 0.0 else -1.0
    r = np.sqrt(x * x + y * y + z * z)
    amp = abs(z) / (2.0 * PI * r * r)
    obliq = (1.0 / r) + 1j * (-s * k)
    return amp * obliq * np.exp(1j * (s * k * r))


def worst_kernel_axis_step(n_pad, d, lam, z):
    k = 2.0 * PI / lam
    x_hi = float(n_pad // 2) * d
    x_lo = x_hi - d
    r_hi = math.sqrt(x_hi * x_hi + z * z)
    r_lo = math.sqrt(x_lo * x_lo + z * z)
    return k * (r_hi - r_lo) + k * d / (1.0 + k * k * z * z)


def worst_paraxial_excess(nx_pad, ny_pad, dx, dy, lam, z):
    k = 2.0 * PI / lam
    x = float(nx_pad // 2) * dx
    y = float(ny_pad // 2) * dy
    az = abs(z)
    r = math.sqrt(x * x + y * y + az * az)
    return max(k * (r - az - (x * x + y * y) / (2.0 * az)), 0.0)


def analyze(band, z, padding):
    nx, ny = band.nx, band.ny
    dx, dy = band.dx, band.dy
    lam = band.lam
    nx_pad = padded_len(nx, padding)
    ny_pad = padded_len(ny, padding)
    kx = worst_kernel_axis_step(nx_pad, dx, lam, z)
    ky = worst_kernel_axis_step(ny_pad, dy, lam, z)
    err = worst_paraxial_excess(nx_pad, ny_pad, dx, dy, lam, z)
    return RsSamplingReport(lam, z, (nx, ny), (dx, dy), padding, (nx_pad, ny_pad), kx, ky,
                            kx < PI and ky < PI, err, err < 0.01)


def sampling_report(band, z, cfg):
    return analyze(band, z, cfg.padding)


def validate(band, z):
    if not math.isfinite(z) or z == 0.0:
        raise RayleighSommerfeldError("InvalidDistance", z)
    if not math.isfinite(band.lam) or band.lam <= 0.0:
        raise RayleighSommerfeldError("InvalidWavelength", band.lam)
    if band.nx == 0 or band.ny == 0:
        raise RayleighSommerfeldError("EmptyGrid")
    if not np.all(np.isfinite(band.samples)):
        raise RayleighSommerfeldError("NonFiniteSample")


def resolve_report(band, z, cfg):
    validate(band, z)
    report = analyze(band, z, cfg.padding)
    if cfg.strict and not report.kernel_nyquist_ok:
        raise RayleighSommerfeldError("AliasingRisk", report=report)
    return report


def impulse_response(nx_pad, ny_pad, dx, dy, lam, z):
    x = dft_order_coords(nx_pad, dx)[None, :]
    y = dft_order_coords(ny_pad, dy)[:, None]
    return kernel_value(x, y, lam, z) * (dx * dy)


def propagate(band, z, cfg=RayleighSommerfeldConfig()):
    """``rayleigh_sommerfeld::propagate`` (rayleigh_sommerfeld.rs:384-442)."""
    report = resolve_report(band, z, cfg)
    nx_pad, ny_pad = report.padded_dims
    buf, ox, oy = embed_centered(band.samples, nx_pad, ny_pad)
    h = impulse_response(nx_pad, ny_pad, band.dx, band.dy, band.lam, z)
    res = crop_centered(ifft2(fft2(buf) * fft2(h)), band.nx, band.ny, ox, oy)
    if not np.all(np.isfinite(res)):
        raise RayleighSommerfeldError("NonFiniteSample")
    return band.with_samples(res)
