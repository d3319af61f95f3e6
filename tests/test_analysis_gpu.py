"""Detector metrics on the GPU (osgpu_psf_*_device) against the oracle
restatement of src/analysis.rs (oracle/analysis.py): FP64 grids to 1e-12
relative (MTF values to 1e-12 of the DC term), float32 grids to 1e-6."""


import numpy as np
import pytest

from oracle import analysis as oan

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from optics_studio_gb300 import analysis as gan  # noqa: E402


def gaussian_psf(w, n, d, centre=(0.0, 0.0)):
    c = (np.arange(n, dtype=np.float64) - (n - 1.0) / 2.0) * d
    return np.exp(-((c[None, :] - centre[0]) ** 2 + (c[:, None] - centre[1]) ** 2) / (w * w))


def grids():
    rng = np.random.default_rng(31)
    yield gaussian_psf(100e-6, 512, 10e-6), (10e-6, 10e-6)
    yield gaussian_psf(40e-6, 200, 4e-6, (30e-6, -12e-6)) + 0.01 * rng.random((200, 200)), (4e-6, 4e-6)
    yield rng.random((96, 130)) ** 3, (3e-6, 5e-6)


@pytest.mark.parametrize("k", [0, 1, 2])
def test_spot_rms_and_mtf_match_oracle(k):
    img, pitch = list(grids())[k]
    for dt, tol in ((torch.float64, 1e-12), (torch.float32, 1e-6)):
        t = torch.from_numpy(img).to("cuda", dt)
        ref_img = t.double().cpu().numpy()
        r = gan.spot_rms_radius(t, pitch)
        assert r == pytest.approx(oan.spot_rms_radius(ref_img, pitch), rel=tol)
        f, v = gan.mtf(t, pitch)
        fo, vo = oan.mtf(ref_img, pitch)
        assert len(f) == len(fo) == img.shape[1] // 2 + 1
        np.testing.assert_allclose(f, fo, rtol=1e-15)
        np.testing.assert_allclose(v, vo, rtol=0, atol=tol)


def test_strehl_and_anchors_match_oracle():
    d = 10e-6
    narrow, wide = gaussian_psf(80e-6, 256, d), gaussian_psf(160e-6, 256, d)
    tn = torch.from_numpy(narrow).cuda()
    tw = torch.from_numpy(wide).cuda()
    assert gan.strehl(tn, (d, d), tn, (d, d)) == pytest.approx(1.0, abs=1e-12)
    s = gan.strehl(tw, (d, d), tn, (d, d))
    assert s == pytest.approx(oan.strehl(wide, (d, d), narrow, (d, d)), rel=1e-12)
    assert 0.2 < s < 0.6
    other = torch.from_numpy(gaussian_psf(60e-6, 128, 7e-6)).cuda()
    assert gan.strehl(other, (7e-6, 7e-6), tn, (d, d)) == pytest.approx(
        oan.strehl(other.cpu().numpy(), (7e-6, 7e-6), narrow, (d, d)), rel=1e-12)
    assert gan.strehl(torch.zeros_like(tn), (d, d), tn, (d, d)) == 0.0
    assert gan.marechal_strehl(0.1) == oan.marechal_strehl(0.1)
    g = gaussian_psf(100e-6, 512, 10e-6)
    assert abs(gan.spot_rms_radius(torch.from_numpy(g).cuda(), (10e-6, 10e-6)) / 100e-6 - 1) < 0.01
    assert gan.spot_rms_radius(torch.zeros((8, 8), dtype=torch.float64, device="cuda"),
                               (1e-6, 1e-6)) == 0.0


@pytest.mark.parametrize("k", [0, 1, 2])
def test_encircled_energy_curve_matches_oracle(k):
    img, pitch = list(grids())[k]
    t = torch.from_numpy(img).cuda()
    got = gan.encircled_energy(t, pitch)
    want = oan.encircled_energy(img, pitch)
    assert len(got.radii) == want.radii.size
    np.testing.assert_array_equal(np.array(got.radii), want.radii)  # same sort, same groups
    np.testing.assert_allclose(got.fraction, want.fraction, rtol=1e-10, atol=1e-13)
    for r in (0.0, float(want.radii[len(want.radii) // 3]), 1.5 * float(want.radii[-1]) / 3):
        assert got.value_at(r) == pytest.approx(want.value_at(r), rel=1e-10, abs=1e-13)
    assert got.radius_for_fraction(0.5) == pytest.approx(want.radius_for_fraction(0.5), rel=1e-9)
    # again on the same geometry (cached radius order), float32 samples
    t32 = t.float()
    g32 = gan.encircled_energy(t32, pitch)
    w32 = oan.encircled_energy(t32.double().cpu().numpy(), pitch)
    np.testing.assert_allclose(g32.fraction, w32.fraction, rtol=1e-10, atol=1e-13)
    assert gan.encircled_energy(torch.zeros_like(t), pitch).radii == []


def test_encircled_energy_of_airy_on_device():
    """analysis.rs:444-474 on the device: EE(r1) = 0.84 +- 0.02."""
    from oracle import field as ofield, element as oel, fraunhofer as ofr
    lam, a, z = 500e-9, 0.5e-3, 0.5
    band = ofield.uniform(1.0, 0.0, 128, 128, 50e-6, 50e-6, lam)
    far = ofr.propagate(oel.EllipticalAperture.circle(a).apply(band), z,
                        ofr.FraunhoferConfig(aperture_extent=a))
    psf = torch.from_numpy(np.abs(far.samples) ** 2).cuda()
    ee = gan.encircled_energy(psf, (far.dx, far.dy))
    assert abs(ee.value_at(1.22 * lam * z / (2.0 * a)) - 0.84) < 0.02
