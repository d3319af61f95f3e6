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
        return np.abs(self.samples) ** 2

    def power(self):
        return float(np.sum(self.intensities()) * self.dx * self.dy)


def ptr(a):
    return a.ctypes.data_as(_ffi.c_double_p)


def precision_code(precision):
    if precision in ("f64", _ffi.F64, None):
        return _ffi.F64
    if precision in ("f32", _ffi.F32):
        return _ffi.F32
    raise ValueError(f"precision must be 'f64' or 'f32', got {precision!r}")
