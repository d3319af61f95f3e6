"""Fraunhofer far-field propagation (oracle; test infrastructure only).

Restates ``src/propagation/fraunhofer.rs``: FraunhoferConfig defaults
(159-171), ``validate`` (284-302), ``regime_report`` (306-347) and
``propagate`` (364-443).
"""

import math
from dataclasses import dataclass
from typing import Optional, Tuple

import numpy as np

from .fft import fft2

PI = math.pi


@dataclass(frozen=True)
class FraunhoferConfig:
    strict: bool = True
    max_n_f: float = 1.0
    source_pos: Optional[Tuple[float, float]] = None
    aperture_extent: Optional[float] = None


@dataclass(frozen=True)
class FraunhoferReport:
    lam: float
    z: float
    input_dims: tuple
    input_pitch: tuple
    output_dims: tuple
    output_pitch: tuple
    n_f_x: float
    n_f_y: float
    source_pos: tuple
    extent_used: float
    extent_is_aperture: bool
    quad_phase_error_rad: float
    max_n_f: float
    regime_ok: bool


class FraunhoferError(Exception):
    def __init__(self, variant, value=None, report=None):
        super().__init__(f"{variant}({value if report is None else report})")
        self.variant = variant
        self.value = value
        self.report = report


def validate(band, z):
    if not math.isfinite(z) or z == 0.0:
        raise FraunhoferError("InvalidDistance", z)
    if not math.isfinite(band.lam) or band.lam <= 0.0:
        raise FraunhoferError("InvalidWavelength", band.lam)
    if band.nx == 0 or band.ny == 0:
        raise FraunhoferError("EmptyGrid")
    if not np.all(np.isfinite(band.samples)):
        raise FraunhoferError("NonFiniteSample")


def regime_report(band, z, cfg):
    """fraunhofer.rs:306-347."""
    nx, ny = band.nx, band.ny
    dx, dy = band.dx, band.dy
    lam = band.lam
    az = abs(z)
    xs, ys = cfg.source_pos if cfg.source_pos is not None else (0.0, 0.0)
    hx = (float(nx) - 1.0) / 2.0 * dx
    hy = (float(ny) - 1.0) / 2.0 * dy
    ap = cfg.aperture_extent
    if ap is not None and math.isfinite(ap) and ap > 0.0:
        rx, ry, from_ap = ap, ap, True
    else:
        rx, ry, from_ap = hx + abs(xs), hy + abs(ys), False
    extent = max(rx, ry)
    n_f_x = rx * rx / (lam * az)
    n_f_y = ry * ry / (lam * az)
    n_f = max(n_f_x, n_f_y)
    return FraunhoferReport(lam, z, (nx, ny), (dx, dy), (nx, ny),
                            (lam * az / (float(nx) * dx), lam * az / (float(ny) * dy)),
                            n_f_x, n_f_y, (xs, ys), extent, from_ap, PI * n_f, cfg.max_n_f,
                            n_f <= cfg.max_n_f)


def _cis(p):
    return np.exp(1j * p)


def propagate(band, z, cfg=FraunhoferConfig()):
    """``fraunhofer::propagate`` (fraunhofer.rs:364-443)."""
    validate(band, z)
    report = regime_report(band, z, cfg)
    if cfg.strict and not report.regime_ok:
        raise FraunhoferError("RegimeViolation", report=report)
    lam = band.lam
    nx, ny = band.nx, band.ny
    dx, dy = band.dx, band.dy
    dxo, dyo = report.output_pitch
    xs, ys = report.source_pos
    k = 2.0 * PI / lam
    f_s = xs / (lam * z)
    g_s = ys / (lam * z)
    cx = (float(nx) - 1.0) / 2.0
    cy = (float(ny) - 1.0) / 2.0
    ix = np.arange(nx, dtype=np.float64)
    iy = np.arange(ny, dtype=np.float64)
    eta = (iy - cy) * dy
    xi = (ix - cx) * dx
    pre_y = _cis(2.0 * PI * cy * iy / float(ny))
    ramp_y = _cis(2.0 * PI * g_s * eta)
    pre_x = _cis(2.0 * PI * (cx * ix / float(nx) + f_s * xi))
    pre = (pre_y * ramp_y)[:, None] * pre_x[None, :]
    buf = fft2(band.samples * pre)
    sgn = 1.0 if z > 0.0 else -1.0
    quad = complex(math.cos(k * z), math.sin(k * z)) / (1j * lam * z)
    dyp = (iy - cy) * dyo - ys
    dxp = (ix - cx) * dxo - xs
    my = np.rint(sgn * (iy - cy) + cy).astype(np.int64)
    mx = np.rint(sgn * (ix - cx) + cx).astype(np.int64)
    post_y = _cis(2.0 * PI * cy * (my.astype(np.float64) - cy) / float(ny))
    post_x = _cis(2.0 * PI * cx * (mx.astype(np.float64) - cx) / float(nx))
    chirp = _cis(PI * (dxp[None, :] * dxp[None, :] + dyp[:, None] * dyp[:, None]) / (lam * z))
    sel = buf[my[:, None], mx[None, :]]
    out = quad * chirp * (post_y[:, None] * post_x[None, :]) * sel * (dx * dy)
    if not np.all(np.isfinite(out)):
        raise FraunhoferError("NonFiniteSample")
    return band.with_samples(out, dxo, dyo)
