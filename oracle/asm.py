"""Exact angular-spectrum propagation (oracle; test infrastructure only).

Restates ``src/propagation/asm.rs``: AsmConfig defaults (124-137),
``axis_band_limit`` (258-265), ``transfer_value`` (273-281),
``worst_phase_steps`` (307-368), ``analyze`` (373-412),
``sampling_report`` (418-420) and ``propagate`` (438-538).
"""

import math
from dataclasses import dataclass, replace

import numpy as np

from .fft import fft2, ifft2, fftfreq, padded_len, embed_centered, crop_centered

PI = math.pi


@dataclass(frozen=True)
class AsmConfig:
    padding: float = 2.0
    band_limited: bool = True
    strict: bool = True
    max_padding: float = 8.0
    medium: float = 1.0


@dataclass(frozen=True)
class SamplingReport:
    lam: float
    medium: float
    z: float
    input_dims: tuple
    pitch: tuple
    requested_padding: float
    used_padding: float
    padded_dims: tuple
    band_limit_fx: float
    band_limit_fy: float
    max_phase_step_x: float
    max_phase_step_y: float
    nyquist_ok: bool


class PropagationError(Exception):
    """Mirror of ``PropagationError`` (asm.rs:219-250)."""

    def __init__(self, variant, value=None, report=None):
        super().__init__(f"{variant}({value if report is None else report})")
        self.variant = variant
        self.value = value
        self.report = report


def axis_band_limit(lam, z, grid_width, band_limited, medium):
    """asm.rs:258-265."""
    lam_n = lam / medium
    if band_limited:
        return 1.0 / (lam_n * math.sqrt((2.0 * z / grid_width) ** 2 + 1.0))
    return 1.0 / lam_n


def _worst_phase_steps(lam, medium, z, nx_pad, ny_pad, dx, dy, lim_x, lim_y, band_limited):
    """asm.rs:307-368."""
    lam_n = lam / medium
    kz = (2.0 * PI / lam_n) * abs(z)

    def step_along(n_pad, d, f_other, lim_other, lim_self):
        df = 1.0 / (float(n_pad) * d)
        nyq = float(n_pad // 2) * df
        f_circle = math.sqrt(max((1.0 / lam_n) ** 2 - f_other ** 2, 0.0))
        f_edge = min(f_circle, nyq)
        if band_limited:
            if abs(f_other) > lim_other:
                return 0.0
            f_edge = min(f_edge, lim_self)
        hi = max(math.floor(f_edge / df), 0.0) * df
        lo = max(hi - df, 0.0)

        def root(f):
            return math.sqrt(max(1.0 - lam_n * lam_n * (f * f + f_other * f_other), 0.0))

        return kz * abs(root(hi) - root(lo))

    step_x = step_along(nx_pad, dx, 0.0, lim_y, lim_x)
    step_y = step_along(ny_pad, dy, 0.0, lim_x, lim_y)
    if band_limited:
        step_x = max(step_x, step_along(nx_pad, dx, lim_y, lim_y, lim_x))
        step_y = max(step_y, step_along(ny_pad, dy, lim_x, lim_x, lim_y))
    return step_x, step_y


def analyze(band, z, cfg, padding):
    """asm.rs:373-412."""
    nx, ny = band.nx, band.ny
    dx, dy = band.dx, band.dy
    lam = band.lam
    nx_pad = padded_len(nx, padding)
    ny_pad = padded_len(ny, padding)
    lim_x = axis_band_limit(lam, z, float(nx_pad) * dx, cfg.band_limited, cfg.medium)
    lim_y = axis_band_limit(lam, z, float(ny_pad) * dy, cfg.band_limited, cfg.medium)
    sx, sy = _worst_phase_steps(lam, cfg.medium, z, nx_pad, ny_pad, dx, dy, lim_x, lim_y,
                                cfg.band_limited)
    return SamplingReport(lam, cfg.medium, z, (nx, ny), (dx, dy), cfg.padding, padding,
                          (nx_pad, ny_pad), lim_x, lim_y, sx, sy, sx < PI and sy < PI)


def sampling_report(band, z, cfg):
    """asm.rs:418-420."""
    return analyze(band, z, cfg, cfg.padding)


def resolve_report(band, z, cfg):
    """Validation + strict densification ladder of ``propagate`` (asm.rs:438-479).

    Returns the report whose ``padded_dims`` the propagation runs on, or
    ``None`` for the z == 0 identity.
    """
    if not math.isfinite(z):
        raise PropagationError("InvalidDistance", z)
    lam = band.lam
    if not math.isfinite(lam) or lam <= 0.0:
        raise PropagationError("InvalidWavelength", lam)
    if not math.isfinite(cfg.medium) or cfg.medium <= 0.0:
        raise PropagationError("InvalidMedium", cfg.medium)
    if band.nx == 0 or band.ny == 0:
        raise PropagationError("EmptyGrid")
    if not np.all(np.isfinite(band.samples)):
        raise PropagationError("NonFiniteSample")
    if z == 0.0:
        return None
    report = analyze(band, z, cfg, cfg.padding)
    if cfg.strict and not report.nyquist_ok:
        padding = cfg.padding
        while not report.nyquist_ok and padding < cfg.max_padding:
            padding = min(padding * 2.0, cfg.max_padding)
            report = analyze(band, z, cfg, padding)
        if not report.nyquist_ok:
            raise PropagationError("AliasingRisk", report=report)
    return report


def transfer_function(nx_pad, ny_pad, dx, dy, lam, z, medium, band_limited, lim_x, lim_y):
    """The masked transfer function H over the padded grid (asm.rs:273-281, 505-522)."""
    fx = fftfreq(nx_pad, dx)[None, :]
    fy = fftfreq(ny_pad, dy)[:, None]
    lam_n = lam / medium
    s = 1.0 - (lam_n * fx) ** 2 - (lam_n * fy) ** 2
    k = 2.0 * PI / lam_n
    ok = s >= 0.0
    if band_limited:
        ok = ok & ~((np.abs(fx) > lim_x) | (np.abs(fy) > lim_y))
    ph = k * z * np.sqrt(np.where(ok, s, 0.0))
    return np.where(ok, np.exp(1j * ph), 0.0)


def propagate(band, z, cfg=AsmConfig()):
    """``asm::propagate`` (asm.rs:438-538)."""
    report = resolve_report(band, z, cfg)
    if report is None:
        return band.with_samples(band.samples.copy())
    nx_pad, ny_pad = report.padded_dims
    buf, ox, oy = embed_centered(band.samples, nx_pad, ny_pad)
    spec = fft2(buf)
    spec *= transfer_function(nx_pad, ny_pad, band.dx, band.dy, band.lam, z, cfg.medium,
                              cfg.band_limited, report.band_limit_fx, report.band_limit_fy)
    out = ifft2(spec)
    res = crop_centered(out, band.nx, band.ny, ox, oy)
    if not np.all(np.isfinite(res)):
        raise PropagationError("NonFiniteSample")
    return band.with_samples(res)


def with_medium(cfg, medium):
    return replace(cfg, medium=medium)
