"""Beamline composition (mirror of optics-core ``beamline``, src/beamline.rs:52-145).

``trace`` with the built-in ASM engine runs the whole beamline through one
C-ABI call (``osgpu_beamline_trace``): the elements of each plane are fused
into the first FFT pass of the propagation that follows them.  Any other
engine closure is driven step by step (element apply, then closure),
exactly as the reference's ``trace``.
"""

import numpy as np

from . import _ffi
from .field import ptr, precision_code
from .propagation.asm import AsmConfig


class AsmEngine:
    """The ASM closure of optics-inverse (observe.rs:195-210): medium injected."""

    def __init__(self, cfg=AsmConfig(), precision="f64"):
        self.cfg = cfg
        self.precision = precision

    def __call__(self, band, z, medium):
        from .propagation import asm
        from dataclasses import replace
        return asm.propagate(band, z, replace(self.cfg, medium=medium), self.precision)


class Beamline:
    def __init__(self):
        self.steps = []  # (element | None, z_after, medium)

    def push(self, element, z_after):
        return self.push_medium(element, z_after, 1.0)

    def push_medium(self, element, z_after, medium):
        self.steps.append((element, z_after, medium))
        return self

    def gap(self, z, medium):
        self.steps.append((None, z, medium))
        return self

    def __len__(self):
        return len(self.steps)

    def trace(self, band, engine):
        if isinstance(engine, AsmEngine):
            return self._trace_fused(band, engine)
        cur = band
        for element, z, medium in self.steps:
            if element is not None:
                cur = element.apply(cur)
            if z != 0.0:
                cur = engine(cur, z, medium)
        return cur

    def psf(self, band, engine):
        return self.trace(band, engine).intensities()

    def _trace_fused(self, band, engine):
        keep = []
        steps = []
        for element, z, medium in self.steps:
            if element is not None:
                d, k = element.descriptor(band)
                keep.append(k)
                arr = (_ffi.ElementC * 1)(d)
                keep.append(arr)
                steps.append(_ffi.StepC(arr, 1, z, medium))
            else:
                steps.append(_ffi.StepC(None, 0, z, medium))
        sarr = (_ffi.StepC * max(len(steps), 1))(*steps)
        reps = (_ffi.AsmReportC * max(len(steps), 1))()
        out = np.empty_like(band.samples)
        _ffi.check(_ffi.lib().osgpu_beamline_trace(ptr(band.samples), ptr(out), band.grid(), sarr,
                                                   len(steps), engine.cfg.c(),
                                                   precision_code(engine.precision), reps))
        res = band.with_samples(out)
        res.reports = list(reps)[: len(steps)]
        return res
