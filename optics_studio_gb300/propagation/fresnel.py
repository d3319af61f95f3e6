"""Fresnel propagation on the GPU, transfer-function and convolution forms.

Mirrors ``optics_core::propagation::fresnel`` (src/propagation/fresnel.rs):
``FresnelConfig`` (99-123), ``sampling_report``, ``propagate`` (430),
``propagate_convolution`` (531).
"""

from dataclasses import dataclass

import numpy as np

from .. import _ffi
from ..field import ptr, precision_code


@dataclass(frozen=True)
class FresnelConfig:
    padding: float = 2.0
    strict: bool = True
    max_padding: float = 8.0

    def c(self):
        return _ffi.FresnelConfigC(self.padding, int(self.strict), self.max_padding)


FresnelError = _ffi.OsgpuError


def sampling_report(band, z, cfg=FresnelConfig()):
    rep = _ffi.FresnelReportC()
    _ffi.check(_ffi.lib().osgpu_fresnel_sampling_report(band.grid(), z, cfg.c(), rep))
    return rep


def _run(fn, band, z, cfg, precision):
    out = np.empty_like(band.samples)
    rep = _ffi.FresnelReportC()
    _ffi.check(fn(ptr(band.samples), ptr(out), band.grid(), z, cfg.c(),
                  precision_code(precision), rep), rep)
    res = band.with_samples(out)
    res.report = rep
    return res


def propagate(band, z, cfg=FresnelConfig(), precision="f64"):
    return _run(_ffi.lib().osgpu_fresnel_propagate, band, z, cfg, precision)


def propagate_convolution(band, z, cfg=FresnelConfig(), precision="f64"):
    return _run(_ffi.lib().osgpu_fresnel_propagate_convolution, band, z, cfg, precision)
