"""Fraunhofer far-field propagation on the GPU.

Mirrors ``optics_core::propagation::fraunhofer`` (src/propagation/fraunhofer.rs):
``FraunhoferConfig`` (118-171), ``regime_report`` (306), ``propagate`` (364).
The output band lives on the far-field grid (pitch lambda |z| / (n d)).
"""

from dataclasses import dataclass
from typing import Optional, Tuple

import numpy as np

from .. import _ffi
from ..field import ptr, precision_code


@dataclass(frozen=True)
class FraunhoferConfig:
    strict: bool = True
    max_n_f: float = 1.0
    source_pos: Optional[Tuple[float, float]] = None
    aperture_extent: Optional[float] = None

    def c(self):
        sp = self.source_pos
        ae = self.aperture_extent
        return _ffi.FraunhoferConfigC(int(self.strict), self.max_n_f, int(sp is not None),
                                      sp[0] if sp else 0.0, sp[1] if sp else 0.0,
                                      int(ae is not None), ae if ae is not None else 0.0)


FraunhoferError = _ffi.OsgpuError


def regime_report(band, z, cfg=FraunhoferConfig()):
    rep = _ffi.FraunhoferReportC()
    _ffi.check(_ffi.lib().osgpu_fraunhofer_regime_report(band.grid(), z, cfg.c(), rep))
    return rep


def propagate(band, z, cfg=FraunhoferConfig(), precision="f64"):
    out = np.empty_like(band.samples)
    rep = _ffi.FraunhoferReportC()
    _ffi.check(_ffi.lib().osgpu_fraunhofer_propagate(ptr(band.samples), ptr(out), band.grid(), z,
                                                     cfg.c(), precision_code(precision), rep),
               rep)
    res = band.with_samples(out, rep.dx_out, rep.dy_out)
    res.report = rep
    return res
