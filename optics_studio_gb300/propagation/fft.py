"""2D DFT in the NumPy convention (mirror of optics-core ``propagation::fft``,
src/propagation/fft.rs:40-108): ``fft2`` unnormalised with kernel
e^{-2 pi i k n / N}, ``ifft2`` scaled by 1 / (nx ny), unshifted bins, on the
GPU through ``osgpu_fft2``."""

import numpy as np

from .. import _ffi
from ..field import ptr, precision_code


def _transform(samples, inverse, precision):
    a = np.ascontiguousarray(samples, dtype=np.complex128)
    if a.ndim != 2:
        raise ValueError("samples must be a 2-D (ny, nx) array")
    out = np.empty_like(a)
    ny, nx = a.shape
    _ffi.check(_ffi.lib().osgpu_fft2(ptr(a), ptr(out), nx, ny, 1 if inverse else 0,
                                     precision_code(precision)))
    return out


def fft2(samples, precision="f64"):
    return _transform(samples, False, precision)


def ifft2(samples, precision="f64"):
    return _transform(samples, True, precision)
