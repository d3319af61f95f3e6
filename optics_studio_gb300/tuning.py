"""Measured schedules of the f32 FFT passes (osgpu_autotune_*).

The reference builds an ``FftPlanner`` on every call (src/propagation/
fft.rs:41,53) and lets rustfft pick its algorithm.  Here each of the three
passes of an f32 propagation has interchangeable kernel variants (row-tile
heights, persistent TMA / bulk-copy kernels, sub-transform groups per CTA,
mirror-column pairs); the tuner times a synthetic batch of a geometry under
each variant of pass A, then B, then C, keeps the fastest, and later f32
propagations of that geometry use it.  ``lanes`` is 1 for single
propagations and 2 for the device batch, which runs items on two lanes.
Off by default (the built-in defaults apply); ``enable()`` makes the device
batch tune every new geometry before its first run.
"""

import ctypes as C

from . import _ffi


def enable():
    _ffi.check(_ffi.lib().osgpu_autotune_config(1))


def disable():
    _ffi.check(_ffi.lib().osgpu_autotune_config(0))


def clear():
    """Forget every measured schedule."""
    _ffi.check(_ffi.lib().osgpu_autotune_clear())


def _info(o):
    return {"m": (o.mx, o.my), "r": (o.rx, o.ry), "n": (o.nx, o.ny), "lanes": o.lanes,
            "pass_a": o.pass_a.decode(), "pass_b": o.pass_b.decode(),
            "pass_c": o.pass_c.decode(), "ms_default": o.ms_default, "ms_best": o.ms_best}


def tune(grid, z, cfg, lanes=1):
    """Measure (once) the schedule of an f32 ASM propagation of ``grid`` (an
    ``osgpu_grid``) over ``z`` with ``cfg`` (an ``AsmConfig``); returns it."""
    out = _ffi.ScheduleInfoC()
    _ffi.check(_ffi.lib().osgpu_autotune_asm(C.byref(grid), float(z), C.byref(cfg.c()),
                                             int(lanes), C.byref(out)))
    return _info(out)


def schedules():
    """Every measured schedule, as dicts (sizes, lanes, variant per pass, the
    synthetic batch's time under the defaults and under the choice)."""
    n = C.c_int32()
    _ffi.check(_ffi.lib().osgpu_autotune_list(None, 0, C.byref(n)))
    arr = (_ffi.ScheduleInfoC * max(n.value, 1))()
    _ffi.check(_ffi.lib().osgpu_autotune_list(arr, n.value, C.byref(n)))
    return [_info(arr[i]) for i in range(n.value)]
