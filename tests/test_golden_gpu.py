"""The reference's hypercam golden render on the GPU.

crates/optics-inverse/tests/hypercam_forward.rs:89-207 renders a 32 x 32
thickness design [gap 0.5 mm] [phase mask, 5 mm] [lens f 5 mm with a 0.2 mm
stop, 10 mm] [lens, 5 mm] for five scene positions with the intensity channel
and the two source-position central differences, and checks it against
tests/data/hypercam/forward.npy (copied to tests/golden/hypercam by
tests/golden/make_hypercam.py) to 1e-6 of the peak.  The same render runs
here through the product's Renderer (device Gaussian sources, device phase
lattice, osgpu_render_batch_device): the FP64 engine to the reference's own
1e-6 of peak over all three channels, the f32 engine to 1e-5 of peak on the
intensity channel (its 1 um finite differences of f32 renders are checked to
1e-3 of their peak).
"""

import math
import pathlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from optics_studio_gb300 import inverse as inv, element as el, sources  # noqa: E402
from optics_studio_gb300.propagation.asm import AsmConfig  # noqa: E402

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "hypercam"


def meta():
    out = {}
    for line in (GOLDEN / "meta.txt").read_text().splitlines():
        line = line.strip()
        if line and not line.startswith("#"):
            k, v = line.split("=", 1)
            out[k] = float(v)
    return out


def render(precision):
    m = meta()
    n = int(m["n"])
    pitch, lam, index = m["pitch"], m["lambda"], m["index"]
    z_gap, f, ap_r, w0, h = m["z_gap"], m["f_relay"], m["aperture_r"], m["w0"], m["h_scene"]
    cdt = torch.complex128 if precision == "f64" else torch.complex64
    rdt = torch.float64 if precision == "f64" else torch.float32
    thick = torch.from_numpy(np.load(GOLDEN / "thickness.npy")).cuda()

    def carrier(values, lam_):
        # the reference's carrier: phase = 2 pi (index - 1) / lambda * thickness
        phase = (values * (2.0 * math.pi * (index - 1.0) / lam_)).to(rdt).contiguous()
        lens = lambda: el.ThinLens.fixed(f, None, el.ClearAperture.circle(ap_r))
        d = inv.Design()
        d.gap(z_gap)
        d.push(inv.DevicePhaseMask(phase, (n, n), (pitch, pitch)), f)
        d.push(lens(), 2 * f)
        d.push(lens(), f)
        return d

    def source(x0, y0, lam_):
        return sources.gaussian(w0, 1.0, (x0, y0), 0.0, lam_, n, n, pitch, pitch, cdt)

    rend = inv.Renderer(carrier, source, (pitch, pitch), bands=[lam],
                        scenes=[(0.0, 0.0), (h, 0.0), (-h, 0.0), (0.0, h), (0.0, -h)],
                        asm_cfg=AsmConfig(1.0, False, False, 1.0, 1.0), precision=precision,
                        deriv_x=True, deriv_y=True, scene_step=h)
    obs = rend.render(thick)
    torch.cuda.synchronize()
    return obs.data.cpu().numpy().astype(np.float64)


def test_hypercam_golden_fp64():
    ref = np.load(GOLDEN / "forward.npy")
    got = render("f64")
    assert got.shape == ref.shape == (3, 1, 5, 32, 32)
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 1e-6


def test_hypercam_golden_f32():
    ref = np.load(GOLDEN / "forward.npy")
    got = render("f32")
    assert np.max(np.abs(got[0] - ref[0])) / np.max(np.abs(ref[0])) < 1e-5
    for c in (1, 2):
        assert np.max(np.abs(got[c] - ref[c])) / np.max(np.abs(ref[c])) < 1e-3, c
