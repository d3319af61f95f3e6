"""Adam update (oracle; test infrastructure only).

Restates the per-epoch update of ``crates/optics-inverse/src/fd.rs:217-235``
(gradient-norm clip, bias-corrected moments, ``lr_frac * span`` step,
``clamp_into`` of ``solve.rs:74-78``) for one step ``t >= 1``.
"""

import numpy as np


def adam_step(x, g, m, v, t, lo, hi, lr_frac=0.02, beta1=0.9, beta2=0.999, eps=1.0e-8,
              clip_norm=1.0):
    """Returns (x, m, v) after step t (all float64 arrays, inputs unchanged)."""
    x = np.array(x, dtype=np.float64)
    m = np.array(m, dtype=np.float64)
    v = np.array(v, dtype=np.float64)
    g = np.asarray(g, dtype=np.float64)
    norm = float(np.sqrt(np.sum(g * g)))
    scale = clip_norm / norm if (clip_norm is not None and norm > clip_norm and norm > 0.0) else 1.0
    bc1 = 1.0 - beta1 ** float(t)
    bc2 = 1.0 - beta2 ** float(t)
    span = hi - lo
    gi = g * scale
    m = beta1 * m + (1.0 - beta1) * gi
    v = beta2 * v + (1.0 - beta2) * gi * gi
    mh = m / bc1
    vh = v / bc2
    denom = np.sqrt(vh) + eps
    step = np.where(denom > 0.0, lr_frac * span * mh / denom, 0.0)
    x = x - step
    x = np.minimum(np.maximum(x, lo), hi)
    return x, m, v
