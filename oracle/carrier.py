"""Design and grid-phase carrier (oracle; test infrastructure only).

Restates ``crates/optics-inverse/src/carrier.rs``: ``Design`` (49-123),
``GridSpec::build_mask`` (169-185), ``Carrier::grid_phase`` (219-242),
``Carrier::analytic`` (204-212), ``slot_bounds`` (303-305),
``grid_geom`` (311-322) and ``build`` (328-356).
"""

import math
from dataclasses import dataclass

import numpy as np

from .beamline import Beamline
from .element import ClearAperture, PhaseMask


class InverseError(ValueError):
    def __init__(self, variant, msg=""):
        super().__init__(f"{variant}: {msg}")
        self.variant = variant


class Design:
    def __init__(self):
        self.elements = []
        self.steps = []  # (element index | None, z_after, medium)

    def push(self, element, z_after, medium=1.0):
        self.elements.append(element)
        self.steps.append((len(self.elements) - 1, z_after, medium))
        return self

    def gap(self, z_after, medium=1.0):
        self.steps.append((None, z_after, medium))
        return self

    def beamline(self):
        bl = Beamline()
        for ei, z, m in self.steps:
            if ei is None:
                bl.gap(z, m)
            else:
                bl.push_medium(self.elements[ei], z, m)
        return bl


@dataclass
class GridGeom:
    dims: tuple
    pitch: tuple
    aperture: ClearAperture
    center: tuple


class Carrier:
    """kind 'grid_phase' or 'analytic'."""

    def __init__(self, kind, dim, lo, hi, geom=None, build_fn=None):
        self.kind = kind
        self.dim = dim
        self.lo = lo
        self.hi = hi
        self.geom = geom
        self.build_fn = build_fn

    @staticmethod
    def grid_phase(dims, pitch, aperture, center, lo, hi):
        nx, ny = dims
        if nx == 0 or ny == 0:
            raise InverseError("Carrier", "grid dims must be positive")
        return Carrier("grid_phase", nx * ny, lo, hi, GridGeom(dims, pitch, aperture, center))

    @staticmethod
    def analytic(dim, lo, hi, build_fn):
        return Carrier("analytic", dim, lo, hi, build_fn=build_fn)

    def slot_bounds(self):
        return (self.lo, self.hi)

    def validate_values(self, values):
        v = np.asarray(values, dtype=np.float64).reshape(-1)
        if v.size != self.dim:
            raise InverseError("WrongDimension", f"{v.size} != {self.dim}")
        if not np.all(np.isfinite(v)):
            raise InverseError("NotFinite")
        if np.any(v < self.lo) or np.any(v > self.hi):
            raise InverseError("OutOfBounds")
        return v

    def build(self, values, lam):
        v = self.validate_values(values)
        if self.kind == "analytic":
            return self.build_fn(v, lam)
        g = self.geom
        mask = PhaseMask.sampled(v, g.dims, g.pitch, None, g.aperture, g.center)
        d = Design()
        d.push(mask, 0.0, 1.0)
        return d


def rem_euclid(a, m):
    r = math.fmod(a, m)
    return r + m if r < 0 else r
