"""Renderer / Observation (oracle; test infrastructure only).

Restates ``crates/optics-inverse/src/observe.rs``: the flat
``[channel][band][scene][row][col]`` layout (64-147), ``render_frame``
(195-210) and ``render`` with the source-position / band central
differences (213-314).
"""

import math
from dataclasses import dataclass, field, replace
from typing import Callable, List

import numpy as np

from . import asm
from .carrier import InverseError

INTENSITY, DX, DY, DLAMBDA = "intensity", "dx", "dy", "dlambda"


@dataclass
class Observation:
    channels: list
    bands: list
    scenes: list
    dims: tuple
    pitch: tuple
    data: np.ndarray  # shape (C, B, S, ny, nx)
    fd_steps: tuple = (0.0, 0.0)

    def frame_len(self):
        return self.dims[0] * self.dims[1]

    def channel_index(self, ch):
        return self.channels.index(ch) if ch in self.channels else None


@dataclass
class Renderer:
    carrier: object
    source: Callable  # (x0, y0, lam) -> BandField
    bands: List[float] = field(default_factory=lambda: [500e-9])
    scenes: List[tuple] = field(default_factory=lambda: [(0.0, 0.0)])
    asm_cfg: asm.AsmConfig = asm.AsmConfig()
    deriv_x: bool = False
    deriv_y: bool = False
    deriv_lambda: bool = False
    scene_step: float = 1e-6
    lambda_step: float = 1e-9

    def render_frame(self, values, lam, x0, y0):
        """observe.rs:195-210."""
        design = self.carrier.build(values, lam)
        band = self.source(x0, y0, lam)
        out = design.beamline().trace(
            band, lambda b, z, m: asm.propagate(b, z, replace(self.asm_cfg, medium=m)))
        return out.intensities()

    def render(self, values):
        """observe.rs:213-314."""
        if not self.bands or not self.scenes:
            raise InverseError("Render", "renderer needs at least one band and one scene")
        if (self.deriv_x or self.deriv_y) and not (math.isfinite(self.scene_step)
                                                   and self.scene_step > 0.0):
            raise InverseError("Render", "scene_step must be positive and finite")
        if self.deriv_lambda and not (math.isfinite(self.lambda_step) and self.lambda_step > 0.0):
            raise InverseError("Render", "lambda_step must be positive and finite")
        chans = [INTENSITY]
        if self.deriv_x:
            chans.append(DX)
        if self.deriv_y:
            chans.append(DY)
        if self.deriv_lambda:
            chans.append(DLAMBDA)
        b0 = self.source(self.scenes[0][0], self.scenes[0][1], self.bands[0])
        ny, nx = b0.samples.shape
        data = np.zeros((len(chans), len(self.bands), len(self.scenes), ny, nx))
        h = self.scene_step
        hl = self.lambda_step
        for bi, lam in enumerate(self.bands):
            for si, (x0, y0) in enumerate(self.scenes):
                data[0, bi, si] = self.render_frame(values, lam, x0, y0)
                if self.deriv_x:
                    hi = self.render_frame(values, lam, x0 + h, y0)
                    lo = self.render_frame(values, lam, x0 - h, y0)
                    data[chans.index(DX), bi, si] = (hi - lo) / (2.0 * h)
                if self.deriv_y:
                    hi = self.render_frame(values, lam, x0, y0 + h)
                    lo = self.render_frame(values, lam, x0, y0 - h)
                    data[chans.index(DY), bi, si] = (hi - lo) / (2.0 * h)
                if self.deriv_lambda:
                    hi = self.render_frame(values, lam + hl, x0, y0)
                    lo = self.render_frame(values, lam - hl, x0, y0)
                    data[chans.index(DLAMBDA), bi, si] = (hi - lo) / (2.0 * hl)
        return Observation(chans, list(self.bands), list(self.scenes), (nx, ny),
                           (b0.dx, b0.dy), data, (h, hl))
