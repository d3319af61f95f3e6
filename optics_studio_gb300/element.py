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

EL_ELLIPSE, EL_RECT, EL_LENS, EL_PHASE, EL_GRATING, EL_SCREEN = 1, 2, 3, 4, 5, 6
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
            # analytic closure: evaluated on the host at each field sample's
            # element-frame coordinates, passed as a grid screen (depth 1)
            _, _, fx, fy = frame_coords(band, self.center, self.psi)
            vals = np.ascontiguousarray(np.broadcast_to(self.profile(fx, fy), fx.shape),
                                        dtype=np.float64)
            vals = np.where(ap_contains(ap, fx, fy), vals, 0.0)
            return _screen_desc(vals, 1.0, ap, self.psi, self.center), vals
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


TAU = 2.0 * math.pi


def wrap_angle(radians):
    """``Angle::new``: rem_euclid into [0, 2 pi) (common.rs:36-40)."""
    r = math.fmod(radians, TAU)
    return r + TAU if r < 0.0 else r


def frame_coords(band, center, orientation):
    """Element-frame coordinates of every field sample: origin-centred grid
    coordinates (field.rs:216-221), shifted by the centre and rotated by the
    wrapped orientation (element.rs:557-560), in the reference's order."""
    psi = wrap_angle(orientation or 0.0)
    x = (np.arange(band.nx, dtype=np.float64) - (band.nx - 1.0) / 2.0) * band.dx
    y = (np.arange(band.ny, dtype=np.float64) - (band.ny - 1.0) / 2.0) * band.dy
    xr = x[None, :] - center[0]
    yr = y[:, None] - center[1]
    c, s = math.cos(psi), math.sin(psi)
    return xr, yr, c * xr + s * yr, -s * xr + c * yr


def ap_contains(ap, fx, fy):
    """ClearAperture::contains (element.rs:476-488), inclusive boundary."""
    if ap.kind == STOP_FIELD:
        return np.ones(fx.shape, dtype=bool)
    if ap.kind == STOP_CIRCLE:
        return fx * fx + fy * fy <= ap.a * ap.a
    if ap.kind == STOP_ELLIPSE:
        a2, b2 = ap.a * ap.a, ap.b * ap.b
        return b2 * fx * fx + a2 * fy * fy <= a2 * b2
    return (np.abs(fx) <= ap.a) & (np.abs(fy) <= ap.b)


def _screen_desc(values, depth, ap, psi, center):
    ny, nx = values.shape
    return _ffi.ElementC(EL_SCREEN, ap.kind, ap.a, ap.b, psi, center[0], center[1], 0.0, 0.0,
                         depth, ptr(values), nx, ny, 0.0, 0.0, 0)


def conic_sag(r, radius, conic, coeffs=()):
    """Conic + even-asphere sag z(r) (element.rs:1850-1862)."""
    c = 1.0 / radius
    r2 = r * r
    root = np.sqrt(np.maximum(1.0 - (1.0 + conic) * c * c * r2, 0.0))
    z = c * r2 / (1.0 + root)
    poly = 0.0
    for a in reversed(list(coeffs)):
        poly = poly * r2 + a
    return z + poly * r2 * r2


def _index(n, lam):
    return float(n(lam)) if callable(n) else float(n)


class SurfaceProfile:
    """SurfaceProfile (element.rs:1760-1870): spherical / conic / even asphere
    (vertex radius, conic constant, coefficients of r^4, r^6, ...) or an
    analytic sag callable z(r), evaluated on the host."""

    def __init__(self, radius=None, conic=0.0, coeffs=(), analytic=None):
        self.radius, self.conic, self.coeffs, self.analytic = radius, conic, tuple(coeffs), analytic

    @staticmethod
    def spherical(radius):
        return SurfaceProfile(radius)

    def validate(self):
        """element.rs:1800-1822: finite parameters and a nonzero vertex radius."""
        if self.analytic is not None:
            return
        if (not math.isfinite(self.radius) or self.radius == 0.0 or not math.isfinite(self.conic)
                or any(not math.isfinite(a) for a in self.coeffs)):
            raise _ffi.OsgpuError(31)

    def check_domain(self, r_max):
        """element.rs:1828-1845: the conic square root must stay real over the stop."""
        if self.analytic is None:
            c = 1.0 / self.radius
            if (1.0 + self.conic) * c * c * r_max * r_max > 1.0:
                raise _ffi.OsgpuError(31)

    def sag(self, r):
        if self.analytic is not None:
            return np.asarray(self.analytic(r), dtype=np.float64)
        return conic_sag(r, self.radius, self.conic, self.coeffs)

    def vertex_curvature(self):
        return None if self.analytic is not None else 1.0 / self.radius


class RefractiveSurface(Element):
    """element.rs:1910-2123: exp(i k (n1 - n2) z) inside the stop, z = conic /
    even-asphere sag plus a linear tilt.  The sag is evaluated on the host at
    the element-frame coordinate of every field sample and bound as a grid
    screen with depth k (n1 - n2); indices are constants or callables n(lam)."""

    def __init__(self, radius, conic=0.0, coeffs=(), n_front=1.0, n_back=1.5, tilt=(0.0, 0.0),
                 orientation=None, aperture=ClearAperture.field(), center=(0.0, 0.0)):
        SurfaceProfile(radius, conic, coeffs).validate()
        self.radius, self.conic, self.coeffs = radius, conic, tuple(coeffs)
        self.n_front, self.n_back, self.tilt = n_front, n_back, tilt
        self.psi = 0.0 if orientation is None else orientation
        self.aperture, self.center = aperture, center

    def values(self, band):
        _, _, fx, fy = frame_coords(band, self.center, self.psi)
        z = (conic_sag(np.sqrt(fx * fx + fy * fy), self.radius, self.conic, self.coeffs)
             + self.tilt[0] * fx + self.tilt[1] * fy)
        inside = ap_contains(self.aperture, fx, fy)
        if not np.all(np.isfinite(z[inside])):
            raise _ffi.OsgpuError(29)
        return np.ascontiguousarray(np.where(inside, z, 0.0))

    def descriptor(self, band):
        k = 2.0 * math.pi / band.lam
        dn = _index(self.n_front, band.lam) - _index(self.n_back, band.lam)
        v = self.values(band)
        return _screen_desc(v, k * dn, self.aperture, self.psi, self.center), v


class Wedge(Element):
    """element.rs:2383-2540: exp(i k (n - 1) t) inside the stop with the
    thickness t = t0 - tan(angle) (x' cos o + y' sin o) evaluated on the host
    per field sample and bound as a grid screen with depth k (n - 1)."""

    def __init__(self, angle, n, base_thickness, orientation, aperture=ClearAperture.field(),
                 center=(0.0, 0.0)):
        self.angle, self.n, self.t0 = angle, n, base_thickness
        self.psi = orientation
        self.aperture, self.center = aperture, center

    def values(self, band):
        _, _, fx, fy = frame_coords(band, self.center, self.psi)
        o = wrap_angle(self.psi)
        g = fx * math.cos(o) + fy * math.sin(o)
        t = self.t0 - math.tan(self.angle) * g
        return np.ascontiguousarray(np.where(ap_contains(self.aperture, fx, fy), t, 0.0))

    def descriptor(self, band):
        k = 2.0 * math.pi / band.lam
        v = self.values(band)
        return _screen_desc(v, k * (_index(self.n, band.lam) - 1.0), self.aperture, self.psi,
                            self.center), v


def _validate_stop(ap, center):
    """ClearAperture::validate (element.rs:415-430) on the host: a finite centre
    for the full field, else positive finite semi-axes and a finite centre."""
    cx, cy = center
    if ap.kind == STOP_FIELD:
        if not (math.isfinite(cx) and math.isfinite(cy)):
            raise _ffi.OsgpuError(22)
    elif not (math.isfinite(ap.a) and ap.a > 0.0 and math.isfinite(ap.b) and ap.b > 0.0
              and math.isfinite(cx) and math.isfinite(cy)):
        raise _ffi.OsgpuError(20)


def _check_footprint(ap, psi, center, band):
    """The OutsideField check of Element::apply (element.rs:2310-2322): the
    stop's rotated footprint plus the centre offset within the grid's half
    extents."""
    if ap.kind == STOP_FIELD:
        return
    if ap.kind == STOP_CIRCLE:
        fx, fy = ap.a, ap.b
    else:
        o = wrap_angle(psi)
        c, s = abs(math.cos(o)), abs(math.sin(o))
        fx, fy = ap.a * c + ap.b * s, ap.a * s + ap.b * c
    gx = (float(band.nx) - 1.0) / 2.0 * band.dx
    gy = (float(band.ny) - 1.0) / 2.0 * band.dy
    if abs(center[0]) + fx > gx or abs(center[1]) + fy > gy:
        raise _ffi.OsgpuError(21)


class ThickLens(Element):
    """element.rs:2159-2360: exp(i k (n - 1) t(rho)) inside the stop, with the
    glass thickness t = t0 - z_front(rho) + z_back(rho) at the element-frame
    radius (no tilt term: a common tilt cancels in the difference).  The
    thickness is evaluated on the host per field sample and bound as a grid
    screen with depth k (n - 1); the index is a number or a callable n(lam).
    Construction raises InvalidOrientation, InvalidSurface, InvalidThickness
    and the aperture errors in the reference's order; apply raises
    OutsideField, InvalidMedium and InvalidSag."""

    def __init__(self, front, back, n, thickness, orientation=None,
                 aperture=ClearAperture.field(), center=(0.0, 0.0)):
        if orientation is not None and not math.isfinite(orientation):
            raise _ffi.OsgpuError(24)
        front.validate()
        back.validate()
        if not math.isfinite(thickness) or thickness < 0.0:
            raise _ffi.OsgpuError(30)
        _validate_stop(aperture, center)
        if aperture.kind != STOP_FIELD:
            r_max = max(aperture.a, aperture.b)  # ClearAperture::extent_radius
            front.check_domain(r_max)
            back.check_domain(r_max)
        self.front, self.back, self.n, self.t0 = front, back, n, thickness
        self.psi = 0.0 if orientation is None else orientation
        self.aperture, self.center = aperture, center

    def thickness_profile(self, r):
        """element.rs:2215-2217."""
        return self.t0 - self.front.sag(r) + self.back.sag(r)

    def power_at(self, lam):
        """element.rs:2221-2225: (n(lam) - 1)(c1 - c2); None for analytic profiles."""
        c1, c2 = self.front.vertex_curvature(), self.back.vertex_curvature()
        if c1 is None or c2 is None:
            return None
        return (_index(self.n, lam) - 1.0) * (c1 - c2)

    def focal_at(self, lam):
        p = self.power_at(lam)
        return None if p is None or p == 0.0 else 1.0 / p

    def values(self, band):
        _, _, fx, fy = frame_coords(band, self.center, self.psi)
        inside = ap_contains(self.aperture, fx, fy)
        t = self.thickness_profile(np.hypot(fx, fy))
        if not np.all(np.isfinite(t[inside])):
            raise _ffi.OsgpuError(29)
        return np.ascontiguousarray(np.where(inside, t, 0.0))

    def descriptor(self, band):
        _check_footprint(self.aperture, self.psi, self.center, band)
        n = _index(self.n, band.lam)
        if not math.isfinite(n) or n <= 0.0:
            raise _ffi.OsgpuError(3)
        k = 2.0 * math.pi / band.lam
        v = self.values(band)
        return _screen_desc(v, k * (n - 1.0), self.aperture, self.psi, self.center), v

