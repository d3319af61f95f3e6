"""Gerchberg-Saxton loop (oracle; test infrastructure only).

Restates ``crates/optics-inverse/src/gs.rs``: ``wrap_pi`` (108-110),
``encode_bounds`` (115-121), variants (125-179), ``run`` (347-597).

``run`` takes a ``propagate_half(samples, z) -> samples`` closure so the
same loop drives both the reference's ASM half-transforms
(``gs.rs:436-444, 493, 554``) and the Fraunhofer far-field variant of the
GS batch workload (no reference implementation: forward is
``fraunhofer::propagate``, back is its exact adjoint, see
``fraunhofer_adjoint`` below).  ``GsInit::Random`` draws from rand 0.8.8
``StdRng`` (ChaCha12) and cannot be reproduced outside Rust; parity runs
use ``GsInit::Given``.
"""

import math
from dataclasses import dataclass, field

import numpy as np

TAU = 2.0 * math.pi


def wrap_pi(v):
    """(v + pi).rem_euclid(2 pi) - pi  (gs.rs:108-110)."""
    r = np.fmod(v + math.pi, TAU)
    r = np.where(r < 0.0, r + TAU, r)
    return r - math.pi


def encode_bounds(phi, lo, hi):
    """gs.rs:115-121."""
    if hi - lo >= TAU:
        r = np.fmod(phi - lo, TAU)
        r = np.where(r < 0.0, r + TAU, r)
        return lo + r
    return np.clip(phi, lo, hi)


@dataclass
class GsRecord:
    iteration: int
    merit: float
    best_merit: float
    amplitude_mse: float
    target_error_rms: float
    phase_update_rms: float


@dataclass
class GsSolution:
    phase: np.ndarray
    merit: float
    best_iteration: int
    amplitude_mse: float
    converged: bool
    iterations: int
    history: list = field(default_factory=list)
    target_intensity: np.ndarray = None
    target_amplitude_error: np.ndarray = None
    phase_error: np.ndarray = None
    illumination_amplitude: np.ndarray = None
    last_phase: np.ndarray = None


def run(u_in, aperture_open, target_amplitude, lo, hi, init_phase, prop_fwd, prop_back,
        merit_fn, max_iterations=100, patience=10, merit_tolerance=1e-4, beta_f=1.0, beta_p=1.0,
        illum=None):
    """``gs::run`` main loop (gs.rs:425-597).

    ``prop_fwd(samples)`` is the input->DOE and DOE->target half-transform,
    ``prop_back(samples)`` the target->DOE back-propagation; ``merit_fn``
    maps the target-plane intensity frame to the merit (the Observation seam
    with one band and one scene).  ``illum`` overrides the DOE-plane
    illumination amplitude (default |prop_fwd(u_in)|, gs.rs:436-444).
    """
    n = target_amplitude.size
    shape = target_amplitude.shape
    if illum is None:
        illum = np.abs(prop_fwd(u_in))
    phase = encode_bounds(np.asarray(init_phase, dtype=np.float64).reshape(shape), lo, hi)
    best = None
    history = []
    last_te = np.zeros(shape)
    last_pe = np.zeros(shape)
    converged = False
    for it in range(max_iterations):
        mask = np.where(aperture_open, illum * np.exp(1j * phase), 0.0)
        u_t = prop_fwd(mask)
        amp_t = np.abs(u_t)
        intensity = amp_t * amp_t
        err = amp_t - target_amplitude
        amp_mse = float(np.sum(err * err) / n)
        merit = merit_fn(intensity)
        improved = best is None or merit < best[0]
        if improved:
            best = (merit, it, phase.copy(), intensity.copy())
        best_merit = best[0]
        history.append(GsRecord(it, merit, best_merit, amp_mse, math.sqrt(amp_mse), 0.0))
        last_te = err
        a = (1.0 - beta_f) * amp_t + beta_f * target_amplitude
        with np.errstate(divide="ignore", invalid="ignore"):
            proj = np.where(amp_t > 0.0, u_t * (a / np.where(amp_t > 0, amp_t, 1.0)), a + 0j)
        v = prop_back(proj)
        dphi = wrap_pi(np.angle(v) - phase)
        phase = encode_bounds(phase + beta_p * dphi, lo, hi)
        last_pe = dphi
        history[-1].phase_update_rms = math.sqrt(float(np.sum(dphi * dphi))) / math.sqrt(n)
        if it + 1 > patience:
            earlier = history[len(history) - 1 - patience].best_merit
            scale = max(abs(earlier), 1e-30)
            if (earlier - best_merit) / scale < merit_tolerance:
                converged = True
                break
    m, bi, bp, bint = best
    return GsSolution(bp, m, bi, history[bi].amplitude_mse, converged, len(history), history,
                      bint, last_te, last_pe, illum, phase)


def fraunhofer_adjoint(out_samples, nx, ny, dx, dy, lam, z):
    """Exact adjoint of ``fraunhofer::propagate`` (source_pos = None, z > 0).

    Forward: U = C * D * F(u * pre) with pre/post/chirp unit-modulus
    diagonals, F the unnormalised DFT, C = quad * dx * dy.  Adjoint:
    u = conj(pre) * F^H(conj(C) conj(post*chirp) U), F^H = N * ifft2.
    """
    from . import fraunhofer as fr
    PI = math.pi
    k = 2.0 * PI / lam
    cx = (nx - 1.0) / 2.0
    cy = (ny - 1.0) / 2.0
    ix = np.arange(nx, dtype=np.float64)
    iy = np.arange(ny, dtype=np.float64)
    dxo = lam * abs(z) / (nx * dx)
    dyo = lam * abs(z) / (ny * dy)
    quad = complex(math.cos(k * z), math.sin(k * z)) / (1j * lam * z)
    dxp = (ix - cx) * dxo
    dyp = (iy - cy) * dyo
    post_y = np.exp(1j * 2.0 * PI * cy * (iy - cy) / ny)
    post_x = np.exp(1j * 2.0 * PI * cx * (ix - cx) / nx)
    chirp = np.exp(1j * PI * (dxp[None, :] ** 2 + dyp[:, None] ** 2) / (lam * z))
    diag = quad * chirp * (post_y[:, None] * post_x[None, :]) * (dx * dy)
    w = np.conj(diag) * out_samples
    v = np.fft.ifft2(w) * (nx * ny)
    pre_y = np.exp(1j * 2.0 * PI * cy * iy / ny)
    pre_x = np.exp(1j * 2.0 * PI * cx * ix / nx)
    return np.conj(pre_y[:, None] * pre_x[None, :]) * v
