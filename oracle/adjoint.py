"""Reverse-mode grid gradient through the render chain (oracle; test
infrastructure only).

Restates ``crates/optics-inverse/src/adjoint.rs``: ``asm_adjoint``
(90-92), ``transmission`` (102-108), ``push_back`` (140-246) and
``grid_gradient`` (268-340).
"""

from dataclasses import replace

import numpy as np

from . import asm
from .element import transmission


def asm_adjoint(band, z, cfg):
    """A(z)^dagger = A(-z) with the same config (adjoint.rs:90-92)."""
    return asm.propagate(band, -z, cfg)


def push_back(design, band_in, cfg, dmdi):
    """adjoint.rs:140-246: forward tape, seed w = dmdi * U, reverse sweep.

    Returns {element index: dM/dphi array (ny, nx)}.
    """
    tape = []
    cur = band_in
    for ei, z, medium in design.steps:
        t = v_after = None
        if ei is not None:
            el = design.elements[ei]
            t = transmission(el, cur)
            cur = el.apply(cur)
            v_after = cur.samples.copy()
        if z != 0.0:
            cur = asm.propagate(cur, z, replace(cfg, medium=medium))
        tape.append((ei, t, v_after, z, medium))
    co = np.asarray(dmdi).reshape(cur.samples.shape) * cur.samples
    acc = {}
    for ei, t, v_after, z, medium in reversed(tape):
        if z != 0.0:
            b = cur.with_samples(co)
            co = asm_adjoint(b, z, replace(cfg, medium=medium)).samples
        if ei is not None:
            g = acc.setdefault(ei, np.zeros(co.shape))
            g += -2.0 * np.imag(np.conj(co) * v_after)
            co = np.conj(t) * co
    return dict(sorted(acc.items()))


def grid_gradient(renderer, values, merit):
    """adjoint.rs:268-340: one render, then one push_back per frame, summed."""
    obs = renderer.render(values)
    seed = merit.obs_gradient(obs)
    acc = {}
    for bi, lam in enumerate(renderer.bands):
        design = renderer.carrier.build(values, lam)
        for si, (x0, y0) in enumerate(renderer.scenes):
            band = renderer.source(x0, y0, lam)
            for ei, g in push_back(design, band, renderer.asm_cfg, seed[0, bi, si]).items():
                if ei in acc:
                    acc[ei] = acc[ei] + g
                else:
                    acc[ei] = g
    return acc
