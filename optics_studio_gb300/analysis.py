"""Detector-plane metrics on device intensity grids (mirror of src/analysis.rs).

``spot_rms_radius``, ``mtf``, ``strehl`` and ``encircled_energy`` run on the
device through osgpu_psf_*_device (FP64 sums); ``marechal_strehl`` is the
reference's closed form of a scalar and the encircled-energy curve is
interpolated on the host, as in the reference.  Intensity grids are real torch tensors
(ny, nx) on the GPU, float64 or float32, with pitch (dx, dy) in meters.
"""

import ctypes as C
import math

from . import _ffi


def _args(img, pitch):
    import torch
    if not img.is_cuda or img.dim() != 2:
        raise _ffi.OsgpuError(102)
    img = img.contiguous()
    code = {torch.float64: _ffi.F64, torch.float32: _ffi.F32}.get(img.dtype)
    if code is None:
        raise _ffi.OsgpuError(102)
    ny, nx = img.shape
    return img, code, _ffi.Grid(nx, ny, float(pitch[0]), float(pitch[1]), 0.0)


def _stream(stream):
    from .inverse import _stream_handle
    return _stream_handle(stream)


def spot_rms_radius(img, pitch, stream=None):
    """analysis.rs:111-124: sqrt(sum I rho^2 / sum I) (m)."""
    img, code, g = _args(img, pitch)
    out = C.c_double()
    _ffi.check(_ffi.lib().osgpu_psf_spot_rms_device(img.data_ptr(), code, C.byref(g),
                                                    _stream(stream), C.byref(out)))
    return out.value


class EncircledEnergy:
    """analysis.rs:37-78: cumulative curve (radii ascending, fractions) with the
    reference's linear interpolation (evaluated on the host)."""

    def __init__(self, radii, fraction):
        self.radii = list(radii)
        self.fraction = list(fraction)

    def curve(self):
        return self.radii, self.fraction

    @staticmethod
    def _interp(xs, ys, x):
        import bisect
        if not xs or x <= xs[0]:
            return ys[0] if ys else 0.0
        if x >= xs[-1]:
            return ys[-1]
        k = bisect.bisect_left(xs, x)
        if xs[k] == x:
            return ys[k]
        x0, x1, y0, y1 = xs[k - 1], xs[k], ys[k - 1], ys[k]
        if x1 == x0:
            return y1
        return y0 + (y1 - y0) * (x - x0) / (x1 - x0)

    def value_at(self, r):
        return self._interp(self.radii, self.fraction, r)

    def radius_for_fraction(self, f):
        return self._interp(self.fraction, self.radii, min(max(f, 0.0), 1.0))


def encircled_energy(img, pitch, stream=None):
    """analysis.rs:81-108: the radius-sorted walk (gather + FP64 prefix sum on
    the device, the geometry's radius order sorted once on the host)."""
    img, code, g = _args(img, pitch)
    cap = g.nx * g.ny
    radii = (C.c_double * cap)()
    frac = (C.c_double * cap)()
    n = C.c_uint64()
    _ffi.check(_ffi.lib().osgpu_psf_encircled_energy_device(
        img.data_ptr(), code, C.byref(g), _stream(stream), radii, frac, cap, C.byref(n)))
    k = n.value
    return EncircledEnergy(radii[:k], frac[:k])


def mtf(img, pitch, stream=None):
    """analysis.rs:136-150: (freqs, values) along +fx, k = 0..nx/2."""
    img, code, g = _args(img, pitch)
    half = g.nx // 2
    freqs = (C.c_double * (half + 1))()
    vals = (C.c_double * (half + 1))()
    _ffi.check(_ffi.lib().osgpu_psf_mtf_device(img.data_ptr(), code, C.byref(g), _stream(stream),
                                               freqs, vals))
    return list(freqs), list(vals)


def strehl(measured, measured_pitch, reference, reference_pitch, stream=None):
    """analysis.rs:159-168: peak ratio after equalising total power."""
    m, code, gm = _args(measured, measured_pitch)
    r, code_r, gr = _args(reference, reference_pitch)
    if code != code_r:
        raise _ffi.OsgpuError(102)
    out = C.c_double()
    _ffi.check(_ffi.lib().osgpu_psf_strehl_device(m.data_ptr(), C.byref(gm), r.data_ptr(),
                                                  C.byref(gr), code, _stream(stream),
                                                  C.byref(out)))
    return out.value


def marechal_strehl(rms_waves):
    """analysis.rs:174-177: exp(-(2 pi sigma)^2), sigma in waves."""
    t = 2.0 * math.pi * rms_waves
    return math.exp(-t * t)
