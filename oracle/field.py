"""Field / BandField data and closed-form sources (oracle; test infrastructure only).

Restates ``src/field.rs`` (Field, BandField, plane_wave, uniform, power,
intensities) and ``src/sources.rs:259-296`` (``gaussian``).
"""

import math
from dataclasses import dataclass

import numpy as np


class FieldError(ValueError):
    """Mirror of ``FieldError`` (field.rs): variant name in ``.variant``."""

    def __init__(self, variant, msg=""):
        super().__init__(f"{variant}: {msg}")
        self.variant = variant


def _valid_pitch(d):
    return math.isfinite(d) and d > 0.0


def _valid_wavelength(lam):
    return math.isfinite(lam) and lam > 0.0


@dataclass
class BandField:
    """A row-major complex grid (shape (ny, nx)) bound to a wavelength.

    Mirrors ``Field`` (field.rs:99-105) + ``BandField`` (field.rs:287-290).
    """

    samples: np.ndarray
    dx: float
    dy: float
    lam: float

    def __post_init__(self):
        s = np.asarray(self.samples, dtype=np.complex128)
        if s.ndim != 2 or s.shape[0] == 0 or s.shape[1] == 0:
            raise FieldError("EmptyGrid")
        if not (_valid_pitch(self.dx) and _valid_pitch(self.dy)):
            raise FieldError("NonPositivePitch")
        if not np.all(np.isfinite(s)):
            raise FieldError("NonFiniteSample")
        if not _valid_wavelength(self.lam):
            raise FieldError("NonPositiveWavelength")
        self.samples = s

    @property
    def nx(self):
        return self.samples.shape[1]

    @property
    def ny(self):
        return self.samples.shape[0]

    def coords(self):
        """Origin-centred coordinates x[ix], y[iy] (field.rs:216-221)."""
        return axis_coords(self.nx, self.dx), axis_coords(self.ny, self.dy)

    def intensities(self):
        return np.abs(self.samples) ** 2  # field.rs:256

    def power(self):
        return float(np.sum(self.intensities()) * self.dx * self.dy)  # field.rs:266

    def with_samples(self, s, dx=None, dy=None):
        return BandField(s, self.dx if dx is None else dx, self.dy if dy is None else dy, self.lam)


def axis_coords(n, d):
    """``(i - (n-1)/2) * d`` with the reference's operation order (field.rs:216-221)."""
    c = (float(n) - 1.0) / 2.0
    return (np.arange(n, dtype=np.float64) - c) * d


def uniform(amplitude, phase, nx, ny, dx, dy, lam):
    """``BandField::uniform`` (field.rs:315-330): u = A e^{i phase}."""
    if not _valid_wavelength(lam):
        raise FieldError("NonPositiveWavelength")
    v = amplitude * complex(math.cos(phase), math.sin(phase))
    return BandField(np.full((ny, nx), v, dtype=np.complex128), dx, dy, lam)


def plane_wave(theta_x, theta_y, amplitude, nx, ny, dx, dy, lam):
    """``BandField::plane_wave`` (field.rs:360-386)."""
    if not _valid_wavelength(lam):
        raise FieldError("NonPositiveWavelength")
    k = 2.0 * math.pi / lam
    alpha = math.sin(theta_x)
    beta = math.sin(theta_y)
    x = axis_coords(nx, dx)
    y = axis_coords(ny, dy)
    ph = k * (alpha * x[None, :] + beta * y[:, None])
    return BandField(amplitude * np.exp(1j * ph), dx, dy, lam)


def gaussian(w0, amplitude, center, z, lam, nx, ny, dx, dy):
    """``sources::gaussian`` q-form beam sampled at distance z from the waist
    (sources.rs:259-296)."""
    cx, cy = center
    if not (math.isfinite(w0) and w0 > 0 and math.isfinite(amplitude)
            and math.isfinite(cx) and math.isfinite(cy)):
        raise FieldError("InvalidBeam")
    if not math.isfinite(z):
        raise FieldError("InvalidPlane")
    if not _valid_wavelength(lam):
        raise FieldError("NonPositiveWavelength")
    z_r = math.pi * w0 * w0 / lam
    w_z = w0 * math.sqrt(1.0 + (z / z_r) ** 2)
    k = 2.0 * math.pi / lam
    inv_r = z / (z * z + z_r * z_r)
    carrier = k * z - math.atan(z / z_r)
    amp = amplitude * w0 / w_z
    x = axis_coords(nx, dx) - cx
    y = axis_coords(ny, dy) - cy
    rho2 = x[None, :] * x[None, :] + y[:, None] * y[:, None]
    env = amp * np.exp(-rho2 / (w_z * w_z))
    phase = carrier + 0.5 * k * rho2 * inv_r
    return BandField(env * np.exp(1j * phase), dx, dy, lam)
