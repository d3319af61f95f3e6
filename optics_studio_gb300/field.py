"""BandField: a row-major complex grid bound to a wavelength.

Mirrors ``Field`` + ``BandField`` of the reference (src/field.rs:99-105,
287-290): samples are complex128, index ``[iy, ix]`` (flat ``iy*nx + ix``),
pitch (dx, dy) in meters, wavelength in meters.
"""

import math

import numpy as np

from . import _ffi


class BandField:
    def __init__(self, samples, dx, dy, lam):
        s = np.ascontiguousarray(samples, dtype=np.complex128)
        if s.ndim != 2:
            raise ValueError("samples must be a 2-D (ny, nx) array")
        if not (math.isfinite(dx) and dx > 0 and math.isfinite(dy) and dy > 0):
            raise ValueError("NonPositivePitch")
        if not (math.isfinite(lam) and lam > 0):
            raise ValueError("NonPositiveWavelength")
        self.samples = s
        self.dx = float(dx)
        self.dy = float(dy)
        self.lam = float(lam)

    @property
    def nx(self):
        return self.samples.shape[1]

    @property
    def ny(self):
        return self.samples.shape[0]

    def grid(self):
        return _ffi.Grid(self.nx, self.ny, self.dx, self.dy, self.lam)

    def with_samples(self, s, dx=None, dy=None):
        return BandField(s, self.dx if dx is None else dx, self.dy if dy is None else dy, self.lam)

    def intensities(self):
        """|u|^2 as re^2 + im^2 (Complex64::norm_sqr, field.rs)."""
        return self.samples.real ** 2 + self.samples.imag ** 2

    def power(self):
        return float(np.sum(self.intensities()) * self.dx * self.dy)


class Psf:
    """A real intensity grid with its pitch (field.rs:404-420): ``samples`` is
    (ny, nx) float64."""

    def __init__(self, samples, dx, dy):
        self.samples = np.ascontiguousarray(samples, dtype=np.float64)
        self.dx = float(dx)
        self.dy = float(dy)

    def total_power(self):
        """field.rs:499-501: sum I dx dy."""
        return float(np.sum(self.samples)) * self.dx * self.dy


def sum_intensity(bands):
    """field.rs:554-578: the incoherent sum of the bands' intensities on their
    shared grid (the results of host-buffer propagations, already on the
    host).  Raises ValueError("EmptyGrid") for no band,
    ValueError("GeometryMismatch") for differing dims or pitch and
    ValueError("NonFiniteSample") for a non-finite sum."""
    if not bands:
        raise ValueError("EmptyGrid")
    first = bands[0]
    geom = (first.nx, first.ny, first.dx, first.dy)
    for b in bands[1:]:
        if (b.nx, b.ny, b.dx, b.dy) != geom:
            raise ValueError("GeometryMismatch")
    acc = first.intensities().copy()
    for b in bands[1:]:
        acc += b.intensities()
    if not np.all(np.isfinite(acc)):
        raise ValueError("NonFiniteSample")
    return Psf(acc, first.dx, first.dy)


def ptr(a):
    return a.ctypes.data_as(_ffi.c_double_p)


def precision_code(precision):
    if precision in ("f64", _ffi.F64, None):
        return _ffi.F64
    if precision in ("f32", _ffi.F32):
        return _ffi.F32
    raise ValueError(f"precision must be 'f64' or 'f32', got {precision!r}")
