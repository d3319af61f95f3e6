"""Merits over an Observation (oracle; test infrastructure only).

``MseToTarget`` restates ``crates/optics-inverse/src/merit.rs:112-164``
(Selector summing over bands/scenes, ``merit.rs:25-81``);
``EncircledEnergyMerit``, ``SpotRmsMerit``, ``StrehlMerit`` and ``MtfMerit``
restate ``merit.rs:167-400``.

``SpotArrayEfficiency`` has no reference implementation: it is the
project-defined merit the inverse-design workload uses (negative summed
efficiency into a set of spot windows), written against the same ``Merit``
seam (``evaluate`` + ``obs_gradient``).
"""

import math

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


class WeightedSpotEfficiency:
    """M = -sum_b sum_k w[k] I_b[k] / P_in_b (project-defined: the efficiency into
    a weighted spot-array target, e.g. a 9 x 9 array of Gaussian spots of peak
    1); dM/dI_b = -w / P_in_b."""

    def __init__(self, weights, p_in):
        self.weights = np.asarray(weights, dtype=np.float64)
        self.p_in = np.asarray(p_in, dtype=np.float64)

    def evaluate(self, obs):
        tot = 0.0
        for b in range(len(obs.bands)):
            for s in range(len(obs.scenes)):
                tot += math.fsum((self.weights * obs.data[0, b, s]).ravel()) / self.p_in[b]
        return -float(tot)

    def obs_gradient(self, obs):
        g = np.zeros_like(obs.data)
        for b in range(len(obs.bands)):
            for s in range(len(obs.scenes)):
                g[0, b, s] = -self.weights / self.p_in[b]
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


def _selected(obs, band, scene):
    """Selector::frame (merit.rs:47-80): the selected intensity frames summed
    band-major, scene-minor, from 0.0."""
    B, S = len(obs.bands), len(obs.scenes)
    bs = range(B) if band is None else [band]
    ss = range(S) if scene is None else [scene]
    for b in bs:
        if b >= B:
            raise ValueError(f"band index {b} out of range")
    for s in ss:
        if s >= S:
            raise ValueError(f"scene index {s} out of range")
    acc = np.zeros(obs.data.shape[-2:], dtype=np.float64)
    for b in bs:
        for s in ss:
            acc = acc + obs.data[0, b, s]
    return acc, bs, ss


class SpotRmsMerit:
    """merit.rs:248-321: R = sqrt(sum I rho^2 / sum I) over the centred pixel
    coordinates; dR/dI_k = (rho_k^2 - R^2) / (2 R sum I) on the selected
    frames."""

    def __init__(self, band=None, scene=None):
        self.band, self.scene = band, scene

    @staticmethod
    def _r2(obs):
        nx, ny = obs.dims
        dx, dy = obs.pitch
        y = (np.arange(ny, dtype=np.float64) - (ny - 1.0) / 2.0) * dy
        x = (np.arange(nx, dtype=np.float64) - (nx - 1.0) / 2.0) * dx
        return x[None, :] * x[None, :] + y[:, None] * y[:, None]

    def evaluate(self, obs):
        frame, _, _ = _selected(obs, self.band, self.scene)
        sw = float(np.sum(frame))
        if sw <= 0.0:
            return 0.0
        return math.sqrt(float(np.sum(frame * self._r2(obs))) / sw)

    def obs_gradient(self, obs):
        frame, bs, ss = _selected(obs, self.band, self.scene)
        sw = float(np.sum(frame))
        if sw <= 0.0:
            return None
        r2 = self._r2(obs)
        rr = float(np.sum(frame * r2)) / sw
        root = math.sqrt(rr)
        if root <= 0.0:
            return None
        g = np.zeros_like(obs.data)
        for b in bs:
            for s in ss:
                g[0, b, s] = (r2 - rr) / (2.0 * root * sw)
        return g


class StrehlMerit:
    """merit.rs:323-352: -((max I / sum I) / (max R / sum R)) against a
    reference frame R of the same grid (maxima folded from 0.0); no
    obs_gradient."""

    def __init__(self, reference, band=None, scene=None):
        self.reference = np.asarray(reference, dtype=np.float64)
        self.band, self.scene = band, scene

    def evaluate(self, obs):
        frame, _, _ = _selected(obs, self.band, self.scene)
        if frame.size != self.reference.size:
            raise ValueError("strehl reference length != frame length")
        pm, pr = float(np.sum(frame)), float(np.sum(self.reference))
        if pm <= 0.0 or pr <= 0.0:
            return 0.0
        peak = lambda v: max(0.0, float(np.max(v)))
        return -((peak(frame) / pm) / (peak(self.reference) / pr))

    def obs_gradient(self, obs):
        return None


class MtfMerit:
    """merit.rs:354-400: -|sum_k I_k e^{-2 pi i m ix_k / nx}| / sum I at the
    bin m = freq nx dx, which must be an integer below Nyquist; no
    obs_gradient."""

    def __init__(self, freq, band=None, scene=None):
        self.freq = freq
        self.band, self.scene = band, scene

    def evaluate(self, obs):
        frame, _, _ = _selected(obs, self.band, self.scene)
        nx, dx = obs.dims[0], obs.pitch[0]
        if self.freq < 0.0 or 2.0 * self.freq * dx >= 1.0:
            raise ValueError(f"MTF frequency {self.freq} beyond Nyquist")
        k = self.freq * nx * dx
        m = int(round(k))
        if abs(k - m) > 1e-9:
            raise ValueError("MTF frequency must land on a DFT bin")
        ang = -2.0 * math.pi * m * np.arange(nx, dtype=np.float64) / nx
        re = float(np.sum(frame * np.cos(ang)[None, :]))
        im = float(np.sum(frame * np.sin(ang)[None, :]))
        dc = float(np.sum(frame))
        if dc <= 0.0:
            return 0.0
        return -(math.hypot(re, im) / dc)

    def obs_gradient(self, obs):
        return None
