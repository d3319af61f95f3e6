"""Shared helpers for the parity tests."""

import numpy as np

from optics_studio_gb300.field import BandField


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def to_gpu_band(ob):
    """oracle BandField -> product BandField (same samples / pitch / lambda)."""
    return BandField(ob.samples, ob.dx, ob.dy, ob.lam)


def rng_field(ny, nx, seed=0, smooth=True):
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(ny, nx)) + 1j * rng.normal(size=(ny, nx))
    if smooth:
        # mild low-pass so the spectrum is not flat to the band edge
        k = np.fft.fft2(u)
        fy = np.fft.fftfreq(ny)[:, None]
        fx = np.fft.fftfreq(nx)[None, :]
        k *= np.exp(-(fx ** 2 + fy ** 2) / (2 * 0.15 ** 2))
        u = np.fft.ifft2(k)
    return u


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
