"""GB300-native (sm_103a) implementation of the optics-studio propagation hot path.

The public surface mirrors the reference Rust API (optics-core
``field``, ``propagation::{asm, fresnel, fraunhofer, rayleigh_sommerfeld}``,
``element``, ``beamline`` and optics-inverse ``gs`` / ``adjoint``); every
call goes through the C ABI of ``include/osgpu.h`` (``lib/libosgpu.so``).
There is no CPU fallback: if the library cannot be built or loaded, or no
GPU is visible, calls raise.
"""

from ._ffi import OsgpuError, lib  # noqa: F401
from . import field, element, beamline  # noqa: F401
from .propagation import asm, fresnel, fraunhofer, rayleigh_sommerfeld  # noqa: F401

F64 = "f64"
F32 = "f32"


def build(force=False):
    from . import _build
    return _build.build(force=force)
