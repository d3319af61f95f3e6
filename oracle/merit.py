"""Merits over an Observation (oracle; test infrastructure only).

``MseToTarget`` restates ``crates/optics-inverse/src/merit.rs:112-164``
(Selector summing over bands/scenes, ``merit.rs:25-81``).

``SpotArrayEfficiency`` has no reference implementation: it is the
project-defined merit the inverse-design workload uses (negative summed
efficiency into a set of spot windows), written against the same ``Merit``
seam (``evaluate`` + ``obs_gradient``).
"""

import numpy as np


class MseToTarget:
    def __init__(self, target, band=None, scene=None):
        self.target = np.asarray(target, dtype=np.float64)
        self.band, self.scene = band, scene

    def _frames(self, obs):
        B, S = len(obs.bands), len(obs.scenes)
        bs = range(B) if self.band is None else [self.band]
        ss = range(S) if self.scene is None else [self.scene]
        return bs, ss

    def evaluate(self, obs):
        bs, ss = self._frames(obs)
        frame = sum(obs.data[0, b, s] for b in bs for s in ss)
        return float(np.sum((frame - self.target.reshape(frame.shape)) ** 2) / frame.size)

    def obs_gradient(self, obs):
        g = np.zeros_like(obs.data)
        n = obs.frame_len()
        bs, ss = self._frames(obs)
        t = self.target.reshape(obs.data.shape[-2:])
        for b in bs:
            for s in ss:
                g[0, b, s] = 2.0 * (obs.data[0, b, s] - t) / n
        return g


class SpotArrayEfficiency:
    """M = -sum_b sum_w (sum_{k in window w} I_b[k]) / P_in_b.

    ``windows`` is a boolean (ny, nx) mask of the spot windows; ``p_in`` the
    per-band input power normaliser (sum |u_in|^2), so each band contributes
    the fraction of input power landing in the spots.
    """

    def __init__(self, windows, p_in):
        self.windows = np.asarray(windows, dtype=bool)
        self.p_in = np.asarray(p_in, dtype=np.float64)

    def evaluate(self, obs):
        tot = 0.0
        for b in range(len(obs.bands)):
            for s in range(len(obs.scenes)):
                tot += np.sum(obs.data[0, b, s][self.windows]) / self.p_in[b]
        return -float(tot)

    def obs_gradient(self, obs):
        g = np.zeros_like(obs.data)
        for b in range(len(obs.bands)):
            for s in range(len(obs.scenes)):
                g[0, b, s] = np.where(self.windows, -1.0 / self.p_in[b], 0.0)
        return g


class EncircledEnergyMerit:
    """merit.rs:167-245: M = -S_in / S_tot over a centred circle of ``radius``."""

    def __init__(self, radius, band=None, scene=None):
        self.radius = radius
        self.band, self.scene = band, scene

    def _mask(self, obs):
        nx, ny = obs.dims
        dx, dy = obs.pitch
        y = (np.arange(ny, dtype=np.float64) - (ny - 1.0) / 2.0) * dy
        x = (np.arange(nx, dtype=np.float64) - (nx - 1.0) / 2.0) * dx
        return x[None, :] * x[None, :] + y[:, None] * y[:, None] <= self.radius * self.radius

    def _frame(self, obs):
        B, S = len(obs.bands), len(obs.scenes)
        bs = range(B) if self.band is None else [self.band]
        ss = range(S) if self.scene is None else [self.scene]
        return sum(obs.data[0, b, s] for b in bs for s in ss), bs, ss

    def evaluate(self, obs):
        frame, _, _ = self._frame(obs)
        total = float(np.sum(frame))
        if total <= 0.0:
            return 0.0
        return -float(np.sum(frame[self._mask(obs)])) / total

    def obs_gradient(self, obs):
        frame, bs, ss = self._frame(obs)
        total = float(np.sum(frame))
        if total <= 0.0:
            return None
        m = self._mask(obs)
        inside = float(np.sum(frame[m]))
        g = np.zeros_like(obs.data)
        for b in bs:
            for s in ss:
                g[0, b, s] = -((np.where(m, total, 0.0) - inside) / (total * total))
        return g
