"""Exact angular-spectrum propagation on the GPU.

Mirrors ``optics_core::propagation::asm`` (src/propagation/asm.rs):
``AsmConfig`` (101-137), ``SamplingReport`` (145-179),
``sampling_report`` (418), ``propagate`` (438).  The host analysis and the
strict densification ladder run in the C library exactly as in the
reference; the transform runs in the sm_103a kernels.
"""

from dataclasses import dataclass

import numpy as np

from .. import _ffi
from ..field import ptr, precision_code


@dataclass(frozen=True)
class AsmConfig:
    padding: float = 2.0
    band_limited: bool = True
    strict: bool = True
    max_padding: float = 8.0
    medium: float = 1.0

    def c(self):
        return _ffi.AsmConfigC(self.padding, int(self.band_limited), int(self.strict),
                               self.max_padding, self.medium)


PropagationError = _ffi.OsgpuError


def _report(r):
    return r


def sampling_report(band, z, cfg=AsmConfig()):
    rep = _ffi.AsmReportC()
    _ffi.check(_ffi.lib().osgpu_asm_sampling_report(band.grid(), z, cfg.c(), rep))
    return rep


def propagate(band, z, cfg=AsmConfig(), precision="f64"):
    """``asm::propagate``; ``precision`` selects the plain f64 or the f32 engine."""
    out = np.empty_like(band.samples)
    rep = _ffi.AsmReportC()
    code = _ffi.lib().osgpu_asm_propagate(ptr(band.samples), ptr(out), band.grid(), z, cfg.c(),
                                          precision_code(precision), rep)
    _ffi.check(code, rep)
    res = band.with_samples(out)
    res.report = rep
    return res
