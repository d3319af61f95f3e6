"""NumPy-convention 2D FFT helpers (oracle; test infrastructure only).

Restates ``src/propagation/fft.rs`` and ``src/propagation/mod.rs:58-64``.
Buffers are complex128 arrays of shape (ny, nx), row-major like the
reference's flat ``iy * nx + ix`` layout.
"""

import math

import numpy as np


def fft2(buf):
    """Unnormalised forward 2D DFT, kernel e^{-2 pi i k n / N} (fft.rs:40-45)."""
    return np.fft.fft2(buf)


def ifft2(buf):
    """Inverse 2D DFT scaled by 1/(nx ny) (fft.rs:52-64)."""
    return np.fft.ifft2(buf)


def fftfreq(n, d):
    """Bin frequencies k/(n d), negative wrap above (n-1)//2 (fft.rs:115-126).

    Written out element by element with the reference's expression
    ``kk / (n as f64 * d)`` so the values are bit-identical to it.
    """
    out = np.empty(n, dtype=np.float64)
    half = (n - 1) // 2
    nd = float(n) * d
    for k in range(n):
        kk = float(k) if k <= half else float(k) - float(n)
        out[k] = kk / nd
    return out


def padded_len(n, padding):
    """``ceil(n * padding)``, at least ``n`` (propagation/mod.rs:58-64)."""
    if padding <= 1.0:
        return n
    return int(math.ceil(float(n) * padding))


def embed_centered(u, nx_pad, ny_pad):
    """Zero-padded centred embed (asm.rs:483-498)."""
    ny, nx = u.shape
    ox = (nx_pad - nx) // 2
    oy = (ny_pad - ny) // 2
    buf = np.zeros((ny_pad, nx_pad), dtype=np.complex128)
    buf[oy:oy + ny, ox:ox + nx] = u
    return buf, ox, oy


def crop_centered(buf, nx, ny, ox, oy):
    """Central window extraction (asm.rs:529-534)."""
    return np.ascontiguousarray(buf[oy:oy + ny, ox:ox + nx])
