"""Detector-plane metrics (oracle; test infrastructure only): numpy f64
restatement of src/analysis.rs.

Each function cites the reference lines it follows.  Psf grids are real
(ny, nx) arrays with pitch (dx, dy); coordinates are the centred pixel
coordinates of field.rs:490-495.
"""

import math

import numpy as np


def _coords(nx, ny, dx, dy):
    x = (np.arange(nx, dtype=np.float64) - (nx - 1.0) / 2.0) * dx
    y = (np.arange(ny, dtype=np.float64) - (ny - 1.0) / 2.0) * dy
    return x[None, :], y[:, None]


def total_power(img, pitch):
    """field.rs:499-501: sum I dx dy."""
    return float(np.sum(img)) * pitch[0] * pitch[1]


class EncircledEnergy:
    """analysis.rs:37-78: cumulative curve with linear interpolation."""

    def __init__(self, radii, fraction):
        self.radii = np.asarray(radii)
        self.fraction = np.asarray(fraction)

    @staticmethod
    def _interp(xs, ys, x):
        if xs.size == 0 or x <= xs[0]:
            return float(ys[0]) if ys.size else 0.0
        if x >= xs[-1]:
            return float(ys[-1])
        k = int(np.searchsorted(xs, x, side="left"))
        if xs[k] == x:
            return float(ys[k])
        x0, x1, y0, y1 = xs[k - 1], xs[k], ys[k - 1], ys[k]
        if x1 == x0:
            return float(y1)
        return float(y0 + (y1 - y0) * (x - x0) / (x1 - x0))

    def value_at(self, r):
        return self._interp(self.radii, self.fraction, r)

    def radius_for_fraction(self, f):
        return self._interp(self.fraction, self.radii, min(max(f, 0.0), 1.0))


def encircled_energy(img, pitch):
    """analysis.rs:81-108: radius-sorted walk, one entry per distinct radius."""
    ny, nx = img.shape
    x, y = _coords(nx, ny, pitch[0], pitch[1])
    r = np.sqrt(x * x + y * y).reshape(-1)
    v = np.asarray(img, dtype=np.float64).reshape(-1)
    order = np.argsort(r, kind="stable")
    r, v = r[order], v[order]
    total = float(np.sum(v))
    if not total > 0.0:
        return EncircledEnergy([], [])
    acc = np.cumsum(v)
    last = np.ones(r.size, dtype=bool)
    last[:-1] = r[1:] != r[:-1]
    return EncircledEnergy(r[last], acc[last] / total)


def spot_rms_radius(img, pitch):
    """analysis.rs:111-124."""
    ny, nx = img.shape
    x, y = _coords(nx, ny, pitch[0], pitch[1])
    sw = float(np.sum(img))
    swr2 = float(np.sum(img * (x * x + y * y)))
    return math.sqrt(swr2 / sw) if sw > 0.0 else 0.0


def mtf(img, pitch):
    """analysis.rs:136-150: row fy = 0 of fft2(I), normalised by DC, capped at 1."""
    ny, nx = img.shape
    buf = np.fft.fft2(np.asarray(img, dtype=np.complex128))
    dc = max(abs(buf[0, 0]), np.finfo(np.float64).tiny)
    half = nx // 2
    freqs = [k / (nx * pitch[0]) for k in range(half + 1)]
    values = [min(abs(buf[0, k]) / dc, 1.0) for k in range(half + 1)]
    return freqs, values


def strehl(measured, pm_pitch, reference, pr_pitch):
    """analysis.rs:159-168."""
    pm, pr = total_power(measured, pm_pitch), total_power(reference, pr_pitch)
    if pm <= 0.0 or pr <= 0.0:
        return 0.0
    peak = lambda a: max(0.0, float(np.max(a)))
    return (peak(measured) / pm) / (peak(reference) / pr)


def marechal_strehl(rms_waves):
    """analysis.rs:174-177."""
    t = 2.0 * math.pi * rms_waves
    return math.exp(-t * t)
