"""Thin-element transmissions (oracle; test infrastructure only).

Restates ``src/element.rs``: ``ClearAperture`` (384-517), helpers
``grid_half_extents`` / ``to_element_frame`` / ``rotated_box`` /
``resolve_orientation`` / ``validate_footprint`` (548-603),
``EllipticalAperture::apply`` (754-790), ``RectangularAperture::apply``
(900-929), ``ThinLens::apply`` (1115-1154), ``SampledPhase::at``
(1189-1207), ``PhaseMask::sampled`` (1321-1368) and ``apply``
(1443-1484), ``BlazedGrating::apply`` (1668-1703), and ``Angle``
wrapping (``src/common.rs:25-40``).
"""

import math
from dataclasses import dataclass
from typing import Callable

import numpy as np

from .field import axis_coords

TAU = 2.0 * math.pi


class OpticsError(ValueError):
    def __init__(self, variant, **kw):
        super().__init__(f"{variant}{kw}")
        self.variant = variant
        self.info = kw


def wrap_angle(radians):
    """``Angle::new``: rem_euclid into [0, 2 pi) (common.rs:36-40)."""
    r = math.fmod(radians, TAU)
    if r < 0.0:
        r += TAU
    return r


def resolve_orientation(orientation):
    o = 0.0 if orientation is None else wrap_angle(orientation)
    if not math.isfinite(o):
        raise OpticsError("InvalidOrientation", radians=o)
    return o


def validate_footprint(hx, hy, center):
    cx, cy = center
    if (not math.isfinite(hx) or hx <= 0.0 or not math.isfinite(hy) or hy <= 0.0
            or not math.isfinite(cx) or not math.isfinite(cy)):
        raise OpticsError("InvalidAperture", half_x=hx, half_y=hy, center_x=cx, center_y=cy)


def rotated_box(hx, hy, psi):
    c, s = abs(math.cos(psi)), abs(math.sin(psi))
    return hx * c + hy * s, hx * s + hy * c


def to_element_frame(x, y, psi):
    c, s = math.cos(psi), math.sin(psi)
    return c * x + s * y, -s * x + c * y


def grid_half_extents(band):
    return ((float(band.nx) - 1.0) / 2.0 * band.dx, (float(band.ny) - 1.0) / 2.0 * band.dy)


@dataclass(frozen=True)
class ClearAperture:
    """kind in {'field', 'circle', 'ellipse', 'rect'}; a/b = semi-axes or half-widths."""

    kind: str = "field"
    a: float = 0.0
    b: float = 0.0

    @staticmethod
    def field():
        return ClearAperture("field")

    @staticmethod
    def circle(r):
        return ClearAperture("circle", r, r)

    @staticmethod
    def ellipse(a, b):
        return ClearAperture("ellipse", a, b)

    @staticmethod
    def rectangle(half_x, half_y):
        return ClearAperture("rect", half_x, half_y)

    def validate(self, center):
        if self.kind == "field":
            cx, cy = center
            if not math.isfinite(cx) or not math.isfinite(cy):
                raise OpticsError("InvalidAxis", center_x=cx, center_y=cy)
        else:
            validate_footprint(self.a, self.b, center)

    def footprint_at(self, psi):
        if self.kind == "field":
            return None
        if self.kind == "circle":
            return (self.a, self.b)
        return rotated_box(self.a, self.b, psi)

    def contains(self, x, y):
        """Boundary-inclusive containment in the stop frame (element.rs:476-488)."""
        if self.kind == "field":
            return np.ones(np.broadcast(x, y).shape, dtype=bool)
        if self.kind == "circle":
            r = self.a
            return x * x + y * y <= r * r
        if self.kind == "ellipse":
            a2, b2 = self.a * self.a, self.b * self.b
            return b2 * x * x + a2 * y * y <= a2 * b2
        return (np.abs(x) <= self.a) & (np.abs(y) <= self.b)


def _check_footprint(fp, center, band):
    if fp is None:
        return
    fx, fy = fp
    cx, cy = center
    gx, gy = grid_half_extents(band)
    if abs(cx) + fx > gx or abs(cy) + fy > gy:
        raise OpticsError("OutsideField", half_x=fx, half_y=fy, center_x=cx, center_y=cy,
                          grid_half_x=gx, grid_half_y=gy)


def _frame_coords(band, center, psi):
    x = axis_coords(band.nx, band.dx)[None, :]
    y = axis_coords(band.ny, band.dy)[:, None]
    xr = x - center[0]
    yr = y - center[1]
    c, s = math.cos(psi), math.sin(psi)
    fx = c * xr + s * yr
    fy = -s * xr + c * yr
    return xr, yr, fx, fy


class Element:
    def transmission(self, band):
        """Pointwise t(x, y) on ``band``'s grid (apply of a unit field)."""
        raise NotImplementedError

    def apply(self, band):
        return band.with_samples(band.samples * self.transmission(band))


class EllipticalAperture(Element):
    """element.rs:635-790."""

    def __init__(self, semi_axes, orientation=None, center=(0.0, 0.0)):
        self.psi = resolve_orientation(orientation)
        validate_footprint(semi_axes[0], semi_axes[1], center)
        self.a, self.b = semi_axes
        self.center = center

    @staticmethod
    def circle(radius, center=(0.0, 0.0)):
        return EllipticalAperture((radius, radius), None, center)

    def transmission(self, band):
        a, b = self.a, self.b
        bx, by = (a, b) if a == b else rotated_box(a, b, self.psi)
        _check_footprint((bx, by), self.center, band)
        _, _, fx, fy = _frame_coords(band, self.center, self.psi)
        a2, b2 = a * a, b * b
        inside = ~(b2 * fx * fx + a2 * fy * fy > a2 * b2)
        return inside.astype(np.complex128)


class RectangularAperture(Element):
    """element.rs:817-929."""

    def __init__(self, half_width, orientation=None, center=(0.0, 0.0)):
        self.psi = resolve_orientation(orientation)
        validate_footprint(half_width[0], half_width[1], center)
        self.a, self.b = half_width
        self.center = center

    def transmission(self, band):
        bx, by = rotated_box(self.a, self.b, self.psi)
        _check_footprint((bx, by), self.center, band)
        _, _, fx, fy = _frame_coords(band, self.center, self.psi)
        inside = ~((np.abs(fx) > self.a) | (np.abs(fy) > self.b))
        return inside.astype(np.complex128)


class ThinLens(Element):
    """element.rs:965-1154; ``focal`` is f(lambda) or a constant."""

    def __init__(self, focal, orientation=None, aperture=ClearAperture.field(), center=(0.0, 0.0)):
        self.psi = resolve_orientation(orientation)
        aperture.validate(center)
        self.focal = focal if callable(focal) else (lambda _lam, f0=focal: f0)
        self.aperture = aperture
        self.center = center

    @staticmethod
    def fixed(f0, orientation=None, aperture=ClearAperture.field(), center=(0.0, 0.0)):
        return ThinLens(f0, orientation, aperture, center)

    def transmission(self, band):
        lam = band.lam
        f = self.focal(lam)
        if not math.isfinite(f) or f == 0.0:
            raise OpticsError("InvalidFocal", lam=lam, f=f)
        _check_footprint(self.aperture.footprint_at(self.psi), self.center, band)
        k = TAU / lam
        xr, yr, fx, fy = _frame_coords(band, self.center, self.psi)
        inside = self.aperture.contains(fx, fy)
        phase = -k * (xr * xr + yr * yr) / (2.0 * f)
        return np.where(inside, np.exp(1j * phase), 0.0)


class PhaseMask(Element):
    """element.rs:1262-1484: analytic closure or sampled lattice (bilinear)."""

    def __init__(self, profile: Callable, orientation=None, aperture=ClearAperture.field(),
                 center=(0.0, 0.0), lattice=None):
        self.psi = resolve_orientation(orientation)
        aperture.validate(center)
        self.profile = profile
        self.aperture = aperture
        self.center = center
        self.lattice = lattice

    @staticmethod
    def sampled(values, dims, pitch, orientation=None, aperture=ClearAperture.field(),
                center=(0.0, 0.0)):
        """element.rs:1321-1368; ``values`` row-major flat or (ny, nx)."""
        psi = resolve_orientation(orientation)
        nx, ny = dims
        v = np.asarray(values, dtype=np.float64).reshape(-1)
        if nx == 0 or ny == 0 or v.size != nx * ny:
            raise OpticsError("InvalidGrid", nx=nx, ny=ny, len=v.size)
        dx, dy = pitch
        if not math.isfinite(dx) or dx <= 0 or not math.isfinite(dy) or dy <= 0:
            raise OpticsError("InvalidGridPitch", dx=dx, dy=dy)
        bad = np.flatnonzero(~np.isfinite(v))
        if bad.size:
            kk = int(bad[0])
            raise OpticsError("InvalidPhase", x=(kk % nx - (nx - 1) / 2.0) * dx,
                              y=(kk // nx - (ny - 1) / 2.0) * dy, phase=float(v[kk]))
        aperture.validate(center)
        lat = (v.reshape(ny, nx), nx, ny, dx, dy)
        m = PhaseMask(lambda x, y: sampled_at(lat, x, y), None, aperture, center, lattice=lat)
        m.psi = psi
        return m

    def transmission(self, band):
        _check_footprint(self.aperture.footprint_at(self.psi), self.center, band)
        _, _, fx, fy = _frame_coords(band, self.center, self.psi)
        inside = self.aperture.contains(fx, fy)
        phi = np.broadcast_to(self.profile(fx, fy), inside.shape)
        bad = inside & ~np.isfinite(phi)
        if np.any(bad):
            raise OpticsError("InvalidPhase")
        return np.where(inside, np.exp(1j * np.where(inside, phi, 0.0)), 0.0)


def sampled_at(lat, x, y):
    """``SampledPhase::at`` bilinear lookup, zero outside the span (element.rs:1189-1207)."""
    vals, nx, ny, dx, dy = lat
    x, y = np.broadcast_arrays(np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64))
    fx = x / dx + (float(nx) - 1.0) / 2.0
    fy = y / dy + (float(ny) - 1.0) / 2.0
    last_x = float(nx) - 1.0
    last_y = float(ny) - 1.0
    outside = (fx < 0.0) | (fx > last_x) | (fy < 0.0) | (fy > last_y)
    fxc = np.where(outside, 0.0, fx)
    fyc = np.where(outside, 0.0, fy)
    i0 = np.floor(fxc).astype(np.int64)
    j0 = np.floor(fyc).astype(np.int64)
    i1 = np.minimum(i0 + 1, nx - 1)
    j1 = np.minimum(j0 + 1, ny - 1)
    tx = fxc - i0
    ty = fyc - j0
    v00 = vals[j0, i0]
    v10 = vals[j0, i1]
    v01 = vals[j1, i0]
    v11 = vals[j1, i1]
    a = v00 + (v10 - v00) * tx
    b = v01 + (v11 - v01) * tx
    return np.where(outside, 0.0, a + (b - a) * ty)


class BlazedGrating(Element):
    """element.rs:1519-1703."""

    def __init__(self, period, phase_depth, orientation, aperture=ClearAperture.field(),
                 center=(0.0, 0.0)):
        psi = wrap_angle(orientation)
        if (not math.isfinite(period) or period <= 0 or not math.isfinite(phase_depth)
                or not math.isfinite(psi)):
            raise OpticsError("InvalidGrating", period=period, depth=phase_depth)
        aperture.validate(center)
        self.period, self.depth, self.psi = period, phase_depth, psi
        self.aperture = aperture
        self.center = center

    def transmission(self, band):
        _check_footprint(self.aperture.footprint_at(self.psi), self.center, band)
        _, _, fx, fy = _frame_coords(band, self.center, self.psi)
        inside = self.aperture.contains(fx, fy)
        u = fx * (1.0 / self.period)
        phi = self.depth * (u - np.floor(u))
        return np.where(inside, np.exp(1j * phi), 0.0)


def transmission(element, band):
    """``adjoint::transmission``: t = apply(1) on ``band``'s grid (adjoint.rs:102-108)."""
    return element.transmission(band)


def conic_sag(r, radius, conic, coeffs=()):
    """Conic + even-asphere sag (element.rs:1850-1862)."""
    c = 1.0 / radius
    r2 = r * r
    root = np.sqrt(np.maximum(1.0 - (1.0 + conic) * c * c * r2, 0.0))
    z = c * r2 / (1.0 + root)
    poly = 0.0
    for a in reversed(list(coeffs)):
        poly = poly * r2 + a
    return z + poly * r2 * r2


class RefractiveSurface(Element):
    """element.rs:1910-2123 with constant indices: t = stop * exp(i (k (n1 - n2)) z),
    z(x', y') = sag(sqrt(x'^2 + y'^2)) + tau_x x' + tau_y y'."""

    def __init__(self, radius, conic=0.0, coeffs=(), n_front=1.0, n_back=1.5, tilt=(0.0, 0.0),
                 orientation=None, aperture=ClearAperture.field(), center=(0.0, 0.0)):
        self.radius, self.conic, self.coeffs = radius, conic, tuple(coeffs)
        self.n1, self.n2, self.tilt = n_front, n_back, tilt
        self.psi = resolve_orientation(orientation)
        aperture.validate(center)
        self.aperture, self.center = aperture, center

    def surface_z(self, fx, fy):
        return (conic_sag(np.sqrt(fx * fx + fy * fy), self.radius, self.conic, self.coeffs)
                + self.tilt[0] * fx + self.tilt[1] * fy)

    def transmission(self, band):
        _check_footprint(self.aperture.footprint_at(self.psi), self.center, band)
        _, _, fx, fy = _frame_coords(band, self.center, self.psi)
        inside = self.aperture.contains(fx, fy)
        k = 2.0 * math.pi / band.lam
        dn = self.n1 - self.n2
        z = self.surface_z(fx, fy)
        return np.where(inside, np.exp(1j * ((k * dn) * z)), 0.0)


class Wedge(Element):
    """element.rs:2383-2540 with a constant index: t = stop * exp(i (k (n - 1)) t(x', y')),
    t = t0 - tan(angle) (x' cos(o) + y' sin(o))."""

    def __init__(self, angle, n, base_thickness, orientation, aperture=ClearAperture.field(),
                 center=(0.0, 0.0)):
        self.angle, self.n, self.t0 = angle, n, base_thickness
        self.psi = resolve_orientation(orientation)
        aperture.validate(center)
        self.aperture, self.center = aperture, center

    def thickness_at(self, fx, fy):
        g = fx * math.cos(self.psi) + fy * math.sin(self.psi)
        return self.t0 - math.tan(self.angle) * g

    def transmission(self, band):
        _check_footprint(self.aperture.footprint_at(self.psi), self.center, band)
        _, _, fx, fy = _frame_coords(band, self.center, self.psi)
        inside = self.aperture.contains(fx, fy)
        k = 2.0 * math.pi / band.lam
        dn = self.n - 1.0
        return np.where(inside, np.exp(1j * ((k * dn) * self.thickness_at(fx, fy))), 0.0)


class SurfaceProfile:
    """SurfaceProfile (element.rs:1760-1870): spherical / conic / even asphere
    (vertex radius, conic constant, coefficients of r^4, r^6, ...) or an
    analytic sag callable z(r)."""

    def __init__(self, radius=None, conic=0.0, coeffs=(), analytic=None):
        self.radius, self.conic, self.coeffs, self.analytic = radius, conic, tuple(coeffs), analytic

    @staticmethod
    def spherical(radius):
        return SurfaceProfile(radius)

    def validate(self):
        """element.rs:1800-1822."""
        if self.analytic is not None:
            return
        r, k = self.radius, self.conic
        if (not math.isfinite(r) or r == 0.0 or not math.isfinite(k)
                or any(not math.isfinite(a) for a in self.coeffs)):
            raise OpticsError("InvalidSurface", radius=r, conic=k, r=math.nan)

    def check_domain(self, r_max):
        """element.rs:1828-1845: 1 - (1 + k) c^2 r^2 >= 0 over the stop."""
        if self.analytic is not None:
            return
        c = 1.0 / self.radius
        if (1.0 + self.conic) * c * c * r_max * r_max > 1.0:
            raise OpticsError("InvalidSurface", radius=self.radius, conic=self.conic, r=r_max)

    def sag(self, r):
        if self.analytic is not None:
            return self.analytic(r)
        return conic_sag(r, self.radius, self.conic, self.coeffs)

    def vertex_curvature(self):
        return None if self.analytic is not None else 1.0 / self.radius


class ThickLens(Element):
    """element.rs:2159-2360: exp(i (k (n - 1)) t(rho)) inside the stop,
    t = t0 - z_front(rho) + z_back(rho) at the element-frame radius; the glass
    index ``n`` is a number or a callable n(lam)."""

    def __init__(self, front, back, n, thickness, orientation=None,
                 aperture=ClearAperture.field(), center=(0.0, 0.0)):
        self.psi = resolve_orientation(orientation)
        front.validate()
        back.validate()
        if not math.isfinite(thickness) or thickness < 0.0:
            raise OpticsError("InvalidThickness", thickness=thickness)
        aperture.validate(center)
        if aperture.kind != "field":
            r_max = max(aperture.a, aperture.b)
            front.check_domain(r_max)
            back.check_domain(r_max)
        self.front, self.back, self.n, self.t0 = front, back, n, thickness
        self.aperture, self.center = aperture, center

    def index_at(self, lam):
        return float(self.n(lam)) if callable(self.n) else float(self.n)

    def thickness_profile(self, r):
        """element.rs:2215-2217."""
        return self.t0 - self.front.sag(r) + self.back.sag(r)

    def power_at(self, lam):
        """element.rs:2221-2225: (n - 1)(c1 - c2), None for analytic profiles."""
        c1, c2 = self.front.vertex_curvature(), self.back.vertex_curvature()
        if c1 is None or c2 is None:
            return None
        return (self.index_at(lam) - 1.0) * (c1 - c2)

    def focal_at(self, lam):
        p = self.power_at(lam)
        return None if p is None or p == 0.0 else 1.0 / p

    def transmission(self, band):
        """element.rs:2305-2358."""
        _check_footprint(self.aperture.footprint_at(self.psi), self.center, band)
        n = self.index_at(band.lam)
        if not math.isfinite(n) or n <= 0.0:
            raise OpticsError("InvalidMedium", n_front=n, n_back=n)
        _, _, fx, fy = _frame_coords(band, self.center, self.psi)
        inside = self.aperture.contains(fx, fy)
        k = 2.0 * math.pi / band.lam
        dn = n - 1.0
        t = self.thickness_profile(np.hypot(fx, fy))
        bad = inside & ~np.isfinite(t)
        if np.any(bad):
            raise OpticsError("InvalidSag", r=float(np.hypot(fx, fy)[bad][0]),
                              sag=float(t[bad][0]))
        return np.where(inside, np.exp(1j * ((k * dn) * t)), 0.0)

