"""Rayleigh-Sommerfeld first-kind propagation on the GPU.

Mirrors ``optics_core::propagation::rayleigh_sommerfeld``
(src/propagation/rayleigh_sommerfeld.rs): config (95-116),
``sampling_report``, ``propagate`` (384).
"""

from dataclasses import dataclass

import numpy as np

from .. import _ffi
from ..field import ptr, precision_code


@dataclass(frozen=True)
class RayleighSommerfeldConfig:
    padding: float = 2.0
    strict: bool = True

    def c(self):
        return _ffi.RsConfigC(self.padding, int(self.strict))


RayleighSommerfeldError = _ffi.OsgpuError


def sampling_report(band, z, cfg=RayleighSommerfeldConfig()):
    rep = _ffi.RsReportC()
    _ffi.check(_ffi.lib().osgpu_rs_sampling_report(band.grid(), z, cfg.c(), rep))
    return rep


def propagate(band, z, cfg=RayleighSommerfeldConfig(), precision="f64"):
    out = np.empty_like(band.samples)
    rep = _ffi.RsReportC()
    _ffi.check(_ffi.lib().osgpu_rs_propagate(ptr(band.samples), ptr(out), band.grid(), z,
                                             cfg.c(), precision_code(precision), rep), rep)
    res = band.with_samples(out)
    res.report = rep
    return res
