"""Propagation engines (mirror of optics-core ``propagation``)."""
from . import asm, fresnel, fraunhofer, rayleigh_sommerfeld  # noqa: F401
