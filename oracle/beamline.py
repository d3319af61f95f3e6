"""Beamline composition (oracle; test infrastructure only).

Restates ``src/beamline.rs:52-145``: steps ``(element | None, z_after,
medium)``; ``trace`` applies each element, then calls the engine closure
for nonzero spacings; ``psf`` returns |u|^2.
"""

from dataclasses import replace

from . import asm


class Beamline:
    def __init__(self):
        self.steps = []

    def push(self, element, z_after):
        return self.push_medium(element, z_after, 1.0)

    def push_medium(self, element, z_after, medium):
        self.steps.append((element, z_after, medium))
        return self

    def gap(self, z, medium):
        self.steps.append((None, z, medium))
        return self

    def trace(self, band, propagate):
        """beamline.rs:109-127."""
        cur = band.with_samples(band.samples.copy())
        for element, z, medium in self.steps:
            if element is not None:
                cur = element.apply(cur)
            if z != 0.0:
                cur = propagate(cur, z, medium)
        return cur

    def psf(self, band, propagate):
        return self.trace(band, propagate).intensities()


def asm_engine(cfg=asm.AsmConfig()):
    """The ASM closure used by optics-inverse (observe.rs:195-210): medium injected."""
    return lambda band, z, medium: asm.propagate(band, z, replace(cfg, medium=medium))
