"""Thin elements (mirror of optics-core ``element``, src/element.rs).

Each element builds its ``osgpu_element`` descriptor; ``apply`` runs the
pointwise transmission on the GPU.  Host closures of the reference
(``ThinLens`` f(lambda), analytic ``PhaseMask``) are evaluated here, on the
host, before upload: ``focal`` is called with the band wavelength, and an
analytic profile is sampled on the field grid into a lattice.
"""

import math
from dataclasses import dataclass

import numpy as np

from . import _ffi
from .field import ptr, precision_code

EL_ELLIPSE, EL_RECT, EL_LENS, EL_PHASE, EL_GRATING = 1, 2, 3, 4, 5
STOP_FIELD, STOP_CIRCLE, STOP_ELLIPSE, STOP_RECT = 0, 1, 2, 3


@dataclass(frozen=True)
class ClearAperture:
    """ClearAperture (element.rs:384-408): kind in field/circle/ellipse/rect."""

    kind: int = STOP_FIELD
    a: float = 0.0
    b: float = 0.0

    @staticmethod
    def field():
        return ClearAperture(STOP_FIELD)

    @staticmethod
    def circle(r):
        return ClearAperture(STOP_CIRCLE, r, r)

    @staticmethod
    def ellipse(a, b):
        return ClearAperture(STOP_ELLIPSE, a, b)

    @staticmethod
    def rectangle(half_x, half_y):
        return ClearAperture(STOP_RECT, half_x, half_y)


class Element:
    def descriptor(self, band):
        """(osgpu_element, keep-alive objects) for this element on ``band``."""
        raise NotImplementedError

    def apply(self, band, precision="f64"):
        return apply_elements(band, [self], precision)


def apply_elements(band, elements, precision="f64"):
    """``Element::apply`` of each element in order, on the GPU."""
    descs, keep = [], []
    for e in elements:
        d, k = e.descriptor(band)
        descs.append(d)
        keep.append(k)
    arr = (_ffi.ElementC * max(len(descs), 1))(*descs)
    out = np.empty_like(band.samples)
    _ffi.check(_ffi.lib().osgpu_apply_elements(ptr(band.samples), ptr(out), band.grid(), arr,
                                               len(descs), precision_code(precision)))
    return band.with_samples(out)


def _desc(kind, stop=STOP_FIELD, a=0.0, b=0.0, psi=0.0, center=(0.0, 0.0), focal=0.0, period=0.0,
          depth=0.0, lattice=None, lnx=0, lny=0, ldx=0.0, ldy=0.0):
    lp = ptr(lattice) if lattice is not None else None
    return _ffi.ElementC(kind, stop, a, b, psi, center[0], center[1], focal, period, depth, lp,
                         lnx, lny, ldx, ldy, 0)


class EllipticalAperture(Element):
    """element.rs:635-790."""

    def __init__(self, semi_axes, orientation=None, center=(0.0, 0.0)):
        self.a, self.b = semi_axes
        self.psi = 0.0 if orientation is None else orientation
        self.center = center

    @staticmethod
    def circle(radius, center=(0.0, 0.0)):
        return EllipticalAperture((radius, radius), None, center)

    def descriptor(self, band):
        return _desc(EL_ELLIPSE, STOP_FIELD, self.a, self.b, self.psi, self.center), None


class RectangularAperture(Element):
    """element.rs:817-929."""

    def __init__(self, half_width, orientation=None, center=(0.0, 0.0)):
        self.a, self.b = half_width
        self.psi = 0.0 if orientation is None else orientation
        self.center = center

    def descriptor(self, band):
        return _desc(EL_RECT, STOP_FIELD, self.a, self.b, self.psi, self.center), None


class ThinLens(Element):
    """element.rs:965-1154; ``focal`` is a constant or a callable f(lambda)."""

    def __init__(self, focal, orientation=None, aperture=ClearAperture.field(), center=(0.0, 0.0)):
        self.focal = focal
        self.psi = 0.0 if orientation is None else orientation
        self.aperture = aperture
        self.center = center

    @staticmethod
    def fixed(f0, orientation=None, aperture=ClearAperture.field(), center=(0.0, 0.0)):
        return ThinLens(f0, orientation, aperture, center)

    def focal_at(self, lam):
        return self.focal(lam) if callable(self.focal) else float(self.focal)

    def descriptor(self, band):
        ap = self.aperture
        return _desc(EL_LENS, ap.kind, ap.a, ap.b, self.psi, self.center,
                     focal=self.focal_at(band.lam)), None


class PhaseMask(Element):
    """element.rs:1262-1484: sampled lattice (bilinear) or analytic closure."""

    def __init__(self, lattice=None, dims=None, pitch=None, profile=None, orientation=None,
                 aperture=ClearAperture.field(), center=(0.0, 0.0)):
        self.lattice = None if lattice is None else np.ascontiguousarray(lattice, dtype=np.float64)
        self.dims = dims
        self.pitch = pitch
        self.profile = profile
        self.psi = 0.0 if orientation is None else orientation
        self.aperture = aperture
        self.center = center

    @staticmethod
    def sampled(values, dims, pitch, orientation=None, aperture=ClearAperture.field(),
                center=(0.0, 0.0)):
        nx, ny = dims
        v = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        if nx == 0 or ny == 0 or v.size != nx * ny:
            raise _ffi.OsgpuError(26)
        return PhaseMask(v.reshape(ny, nx), dims, pitch, None, orientation, aperture, center)

    @staticmethod
    def new(profile, orientation=None, aperture=ClearAperture.field(), center=(0.0, 0.0)):
        return PhaseMask(None, None, None, profile, orientation, aperture, center)

    def descriptor(self, band):
        ap = self.aperture
        if self.lattice is not None:
            nx, ny = self.dims
            lat = self.lattice
            dx, dy = self.pitch
        else:
            # analytic closure: evaluate in the element frame on the field grid
            # and pass it as a lattice with identical geometry (element frame
            # coordinates of the field samples, sampled on the host).
            raise NotImplementedError("analytic PhaseMask: sample it with PhaseMask.sampled")
        return _desc(EL_PHASE, ap.kind, ap.a, ap.b, self.psi, self.center, lattice=lat,
                     lnx=nx, lny=ny, ldx=dx, ldy=dy), lat


class BlazedGrating(Element):
    """element.rs:1519-1703."""

    def __init__(self, period, phase_depth, orientation, aperture=ClearAperture.field(),
                 center=(0.0, 0.0)):
        self.period = period
        self.depth = phase_depth
        self.psi = orientation
        self.aperture = aperture
        self.center = center

    @staticmethod
    def kinoform(period, orientation, aperture=ClearAperture.field(), center=(0.0, 0.0)):
        return BlazedGrating(period, 2.0 * math.pi, orientation, aperture, center)

    def descriptor(self, band):
        ap = self.aperture
        return _desc(EL_GRATING, ap.kind, ap.a, ap.b, self.psi, self.center, period=self.period,
                     depth=self.depth), None
