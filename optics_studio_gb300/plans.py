"""Kernel-spectrum plans for repeated f32 ASM propagation (osgpu_plan_cache_*).

No counterpart in the reference, whose ``asm::propagate`` recomputes H on
every call (src/propagation/asm.rs:505-522).  When a padded grid exceeds twice
the field (strict densification often pads 2048^2 to 8192^2), the output
only reaches kernel offsets |d| < n, so the same propagation is a circular
convolution of period 2n.  With plans enabled, the first f32 ASM propagation
of a geometry builds that kernel's spectrum once (the kernel by the f32
engine on the padded path, its spectrum folded in FP64) and later ones,
forward or adjoint, run at 2n: worth it when one geometry is propagated
many times (an optimisation loop, a renderer over scenes).  Off by default.
"""

import ctypes as C

from . import _ffi


def enable(max_bytes=4 << 30):
    """Turns plans on, holding at most ``max_bytes`` of device tables."""
    _ffi.check(_ffi.lib().osgpu_plan_cache_config(1, int(max_bytes)))


def disable():
    """Later propagations take the padded path; the held tables are freed."""
    _ffi.check(_ffi.lib().osgpu_plan_cache_config(0, 0))


def clear():
    _ffi.check(_ffi.lib().osgpu_plan_cache_clear())


def stats():
    s = _ffi.PlanStatsC()
    _ffi.check(_ffi.lib().osgpu_plan_cache_stats(C.byref(s)))
    return {"plans": s.plans, "bytes": s.bytes, "hits": s.hits, "builds": s.builds}
