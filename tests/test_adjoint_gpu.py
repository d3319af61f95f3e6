"""Inverse loops on the GPU against the f64 oracle (oracle/adjoint.py,
observe.py, merit.py, adam.py restating crates/optics-inverse/src/
{adjoint,observe,merit,fd}.rs).

Tolerances: the FP64 engine matches the oracle to 1e-12 relative L2 (fields,
gradients) and 1e-12 relative (merit values); the f32 engine's gradients
match to 1e-4 relative L2 (the gradient bound of the inverse-design
workload), its intensities to 1e-5.
"""

import math

import numpy as np
import pytest

from oracle import adjoint as o_adj, asm as o_asm, carrier as o_car, element as o_el
from oracle import field as o_field, merit as o_merit, observe as o_obs, adam as o_adam

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from optics_studio_gb300 import inverse as inv, element as el  # noqa: E402
from optics_studio_gb300.propagation.asm import AsmConfig  # noqa: E402

N, D = 64, 4e-6
BANDS = [520e-9, 580e-9]
Z1, Z2 = 2e-3, 3e-3
R_AP = 100e-6


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def phases(seed=7):
    return np.random.default_rng(seed).uniform(0.0, 2 * math.pi, (N, N))


def o_source(x0, y0, lam):
    return o_field.gaussian(60e-6, 1.0, (x0, y0), 0.0, lam, N, N, D, D)


def o_design(v, lam):
    d = o_car.Design()
    d.push(o_el.PhaseMask.sampled(v, (N, N), (D, D)), Z1)
    d.push(o_el.EllipticalAperture.circle(R_AP), Z2)
    return d


def o_renderer(scenes=((0.0, 0.0),)):
    car = o_car.Carrier.analytic(N * N, 0.0, 2 * math.pi, o_design)
    return o_obs.Renderer(car, o_source, bands=list(BANDS), scenes=list(scenes),
                          asm_cfg=o_asm.AsmConfig())


def g_renderer(precision, lattice32=False, scenes=((0.0, 0.0),)):
    cdt = torch.complex128 if precision == "f64" else torch.complex64

    def source(x0, y0, lam):
        return torch.from_numpy(o_source(x0, y0, lam).samples).to("cuda", cdt)

    def carrier(values, lam):
        lat = values.float() if lattice32 else values
        d = inv.Design()
        d.push(inv.DevicePhaseMask(lat, (N, N), (D, D)), Z1)
        d.push(el.EllipticalAperture.circle(R_AP), Z2)
        return d

    return inv.Renderer(carrier, source, (D, D), bands=list(BANDS), scenes=list(scenes),
                        asm_cfg=AsmConfig(), precision=precision)


def windows():
    w = np.zeros((N, N), dtype=bool)
    for cy in (20, 32, 44):
        for cx in (20, 32, 44):
            w[cy - 1:cy + 2, cx - 1:cx + 2] = True
    return w


def p_in():
    return [float(np.sum(np.abs(o_source(0.0, 0.0, lam).samples) ** 2)) for lam in BANDS]


@pytest.mark.parametrize("precision,lattice32", [("f64", False), ("f32", False), ("f32", True)])
def test_grid_gradient_matches_oracle(precision, lattice32):
    phi = phases()
    o_m = o_merit.SpotArrayEfficiency(windows(), p_in())
    want = o_adj.grid_gradient(o_renderer(), phi.reshape(-1), o_m)
    want_val = o_m.evaluate(o_renderer().render(phi.reshape(-1)))

    rend = g_renderer(precision, lattice32)
    values = torch.from_numpy(phi).cuda()
    g_m = inv.SpotArrayEfficiency(torch.from_numpy(windows()).cuda(), p_in())
    got, val, obs = inv.grid_gradient(rend, values, g_m)
    torch.cuda.synchronize()
    tol = 1e-12 if precision == "f64" else 1e-4
    assert sorted(got) == sorted(want) == [0, 1]
    for ei in (0, 1):
        err = rel_l2(got[ei].cpu().numpy(), want[ei].reshape(N, N))
        assert err <= tol, (ei, err)
    assert abs(val - want_val) <= (1e-12 if precision == "f64" else 1e-5) * abs(want_val)
    ref_obs = o_renderer().render(phi.reshape(-1)).data
    assert rel_l2(obs.data.cpu().numpy(), ref_obs) <= (1e-12 if precision == "f64" else 1e-5)


def chain_design_o(v, lam):
    d = o_car.Design()
    d.push(o_el.ThinLens.fixed(5e-3), 0.0)  # two elements before the first propagation
    d.push(o_el.PhaseMask.sampled(v, (N, N), (D, D)), 1e-3)
    d.gap(1.5e-3)
    d.push(o_el.RectangularAperture((90e-6, 70e-6)), 0.0)  # trailing element at the detector
    return d


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_push_back_chain_gap_trailing_matches_oracle(precision):
    lam = 550e-9
    phi = phases(11)
    dmdi = np.random.default_rng(5).normal(size=(N, N))
    want = o_adj.push_back(chain_design_o(phi.reshape(-1), lam), o_source(0.0, 0.0, lam),
                           o_asm.AsmConfig(), dmdi)
    cdt = torch.complex128 if precision == "f64" else torch.complex64
    rdt = torch.float64 if precision == "f64" else torch.float32

    def carrier(values, lam_):
        d = inv.Design()
        d.push(el.ThinLens.fixed(5e-3), 0.0)
        d.push(inv.DevicePhaseMask(values, (N, N), (D, D)), 1e-3)
        d.gap(1.5e-3)
        d.push(el.RectangularAperture((90e-6, 70e-6)), 0.0)
        return d

    def source(x0, y0, lam_):
        return torch.from_numpy(o_source(x0, y0, lam_).samples).to("cuda", cdt)

    rend = inv.Renderer(carrier, source, (D, D), bands=[lam], precision=precision)
    got = inv.push_back(rend, torch.from_numpy(phi).cuda(), lam, 0.0, 0.0,
                        torch.from_numpy(dmdi).cuda().to(rdt))
    torch.cuda.synchronize()
    assert sorted(got) == sorted(want) == [0, 1, 2]
    tol = 1e-12 if precision == "f64" else 1e-4
    for ei in (0, 1):
        err = rel_l2(got[ei].cpu().numpy(), want[ei].reshape(N, N))
        assert err <= tol, (ei, err)
    # an element at the detector plane cannot change |u|^2 through its phase:
    # its gradient is zero up to rounding in both implementations
    scale = np.abs(want[1]).max()
    noise = 1e-12 if precision == "f64" else 1e-6
    assert np.abs(want[2]).max() <= 1e-12 * scale
    assert np.abs(got[2].cpu().numpy()).max() <= noise * scale


def test_tape_and_recompute_agree_and_budget_falls_back():
    phi = torch.from_numpy(phases(3)).cuda()
    rend = g_renderer("f64", scenes=((0.0, 0.0), (20e-6, -10e-6)))
    g_m = inv.SpotArrayEfficiency(torch.from_numpy(windows()).cuda(), p_in())
    with_tape, _, _ = inv.grid_gradient(rend, phi, g_m)
    small = inv.Tape(budget_bytes=1024)  # too small: nothing recorded, push_back recomputes
    recomputed, _, _ = inv.grid_gradient(rend, phi, g_m, tape=small)
    assert small.nbytes() == 0
    small.close()
    torch.cuda.synchronize()
    for ei in (0, 1):
        assert torch.equal(with_tape[ei], recomputed[ei])


def test_merits_match_oracle_with_selectors():
    rng = np.random.default_rng(9)
    B, S = 2, 3
    data = rng.uniform(0.0, 2.0, (1, B, S, N, N))
    obs_o = o_obs.Observation(["intensity"], [5e-7, 6e-7], [(0, 0)] * S, (N, N), (D, D), data)
    obs_g = inv.Observation(["intensity"], [5e-7, 6e-7], [(0, 0)] * S, (N, N), (D, D),
                            torch.from_numpy(data).cuda())
    target = rng.uniform(0.0, 1.0, (N, N))
    for band, scene in [(None, None), (1, None), (None, 2), (0, 1)]:
        om = o_merit.MseToTarget(target, band, scene)
        gm = inv.MseToTarget(torch.from_numpy(target).cuda(), band, scene)
        assert gm.evaluate(obs_g) == pytest.approx(om.evaluate(obs_o), rel=1e-12)
        np.testing.assert_allclose(gm.obs_gradient(obs_g).cpu().numpy(), om.obs_gradient(obs_o),
                                   rtol=1e-12, atol=0)
        oe = o_merit.EncircledEnergyMerit(50e-6, band, scene)
        ge = inv.EncircledEnergyMerit(50e-6, band, scene)
        assert ge.evaluate(obs_g) == pytest.approx(oe.evaluate(obs_o), rel=1e-12)
        np.testing.assert_allclose(ge.obs_gradient(obs_g).cpu().numpy(), oe.obs_gradient(obs_o),
                                   rtol=1e-12, atol=1e-300)
    zero = inv.Observation(["intensity"], [5e-7], [(0, 0)], (N, N), (D, D),
                           torch.zeros((1, 1, 1, N, N), dtype=torch.float64, device="cuda"))
    assert inv.EncircledEnergyMerit(50e-6).evaluate(zero) == 0.0
    assert inv.EncircledEnergyMerit(50e-6).obs_gradient(zero) is None


@pytest.mark.parametrize("clip", [1.0, None])
def test_adam_steps_match_oracle(clip):
    rng = np.random.default_rng(21)
    n = 4096
    x = rng.uniform(0.0, 2 * math.pi, n)
    cfg = inv.AdamConfig(lr_frac=0.05 / (2 * math.pi), clip_norm=clip)
    xd = torch.from_numpy(x).cuda()
    x32 = torch.empty(n, dtype=torch.float32, device="cuda")
    opt = inv.Adam(xd, 0.0, 2 * math.pi, cfg, x32=x32)
    xo, mo, vo = x.copy(), np.zeros(n), np.zeros(n)
    for t in range(1, 4):
        g = rng.normal(size=n) * (0.5 if t < 3 else 10.0)
        g[:3] = [1e3, -1e3, 0.0]  # drives samples into both bounds
        opt.step(torch.from_numpy(g).cuda())
        xo, mo, vo = o_adam.adam_step(xo, g, mo, vo, t, 0.0, 2 * math.pi, cfg.lr_frac, cfg.beta1,
                                      cfg.beta2, cfg.eps, clip)
    torch.cuda.synchronize()
    got = xd.cpu().numpy()
    if clip is None:
        assert np.array_equal(got, xo)
    else:
        np.testing.assert_allclose(got, xo, rtol=1e-14, atol=1e-14)
    assert np.array_equal(x32.cpu().numpy(), got.astype(np.float32))
    assert got.min() >= 0.0 and got.max() <= 2 * math.pi


def test_adjoint_gradient_matches_central_fd():
    """adjoint.rs:499-544 form on the GPU FP64 path: dM/dphi vs central
    differences (h = 1e-4 rad) on seeded pixels."""
    phi = phases(13)
    rend = g_renderer("f64")
    g_m = inv.SpotArrayEfficiency(torch.from_numpy(windows()).cuda(), p_in())
    values = torch.from_numpy(phi).cuda()
    got, _, _ = inv.grid_gradient(rend, values, g_m)
    g = got[0].cpu().numpy().reshape(-1)
    idx = np.random.default_rng(17).choice(np.flatnonzero(np.abs(g) > 1e-3 * np.abs(g).max()),
                                           8, replace=False)
    h = 1e-4
    for i in idx:
        vp = phi.reshape(-1).copy(); vp[i] += h
        vm = phi.reshape(-1).copy(); vm[i] -= h
        fp = g_m.evaluate(rend.render(torch.from_numpy(vp.reshape(N, N)).cuda()))
        fm = g_m.evaluate(rend.render(torch.from_numpy(vm.reshape(N, N)).cuda()))
        fd = (fp - fm) / (2 * h)
        assert abs(g[i] - fd) <= 1e-4 * abs(fd), (i, g[i], fd)


def test_field_power_compensated():
    rng = np.random.default_rng(2)
    u = rng.normal(size=(256, 256)) + 1j * rng.normal(size=(256, 256))
    p = inv.field_power(torch.from_numpy(u).cuda())
    assert p == pytest.approx(float(np.sum(np.abs(u) ** 2)), rel=1e-13)


def thickness_renderer(precision, index):
    cdt = torch.complex128 if precision == "f64" else torch.complex64

    def source(x0, y0, lam):
        return torch.from_numpy(o_source(x0, y0, lam).samples).to("cuda", cdt)

    carrier, slope = inv.grid_thickness(
        (N, N), (D, D), index, z_after=Z1,
        rest=lambda d, lam: d.push(el.EllipticalAperture.circle(R_AP), Z2))
    rend = inv.Renderer(carrier, source, (D, D), bands=list(BANDS), asm_cfg=AsmConfig(),
                        precision=precision, param_slope=slope)
    return rend, slope


def test_grid_thickness_gradient_chain_rule():
    """carrier.rs:247-354 GridThickness: phase 2 pi (n(lam) - 1) h / lam per band.
    grid_gradient with the carrier's per-band slope returns dM/dh: checked
    against central differences in h (FP64 engine), against the weighted sum
    over bands of single-band dM/dphi that adjoint.rs:255-262 prescribes, and
    the f32 engine against the FP64 one (1e-4)."""
    index = lambda lam: 1.46 + 3.0e-15 / lam ** 2  # dispersive (Cauchy form)
    h0 = np.random.default_rng(21).uniform(0.0, 1.2e-6, (N, N))
    g_m = inv.SpotArrayEfficiency(torch.from_numpy(windows()).cuda(), p_in())
    rend, slope = thickness_renderer("f64", index)
    got, _, _ = inv.grid_gradient(rend, torch.from_numpy(h0).cuda(), g_m)
    g = got[0].cpu().numpy()
    # weighted sum of per-band phase gradients, each from a one-band render
    want = np.zeros((N, N))
    for b, lam in enumerate(BANDS):
        one = inv.Renderer(rend.carrier, rend.source, (D, D), bands=[lam], asm_cfg=AsmConfig(),
                           precision="f64")
        mb = inv.SpotArrayEfficiency(torch.from_numpy(windows()).cuda(), [p_in()[b]])
        gb, _, _ = inv.grid_gradient(one, torch.from_numpy(h0).cuda(), mb)
        want += slope(lam) * gb[0].cpu().numpy()
    assert rel_l2(g, want) <= 1e-12
    # central differences in h
    flat = g.reshape(-1)
    idx = np.random.default_rng(5).choice(np.flatnonzero(np.abs(flat) > 1e-3 * np.abs(flat).max()),
                                          6, replace=False)
    dh = 1e-11  # m (about 1e-4 rad of phase)
    for i in idx:
        hp = h0.reshape(-1).copy(); hp[i] += dh
        hm = h0.reshape(-1).copy(); hm[i] -= dh
        fp = g_m.evaluate(rend.render(torch.from_numpy(hp.reshape(N, N)).cuda()))
        fm = g_m.evaluate(rend.render(torch.from_numpy(hm.reshape(N, N)).cuda()))
        fd = (fp - fm) / (2 * dh)
        assert abs(flat[i] - fd) <= 1e-4 * abs(fd), (i, flat[i], fd)
    r32, _ = thickness_renderer("f32", index)
    g32, _, _ = inv.grid_gradient(r32, torch.from_numpy(h0).cuda().float(), g_m)
    assert rel_l2(g32[0].cpu().numpy(), g) <= 1e-4


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_weighted_spot_efficiency_gradient_matches_oracle(precision):
    """The Gaussian spot-array efficiency merit (the inverse-design workload's
    merit): value, dM/dI and the grid gradient through it against the oracle
    (FP64 1e-12, f32 1e-4 on the gradient)."""
    phi = phases(29)
    w = inv.gaussian_spot_array((N, N), 3, 12, 1.5)
    o_m = o_merit.WeightedSpotEfficiency(w, p_in())
    o_obs_ = o_renderer().render(phi.reshape(-1))
    want = o_adj.grid_gradient(o_renderer(), phi.reshape(-1), o_m)
    g_m = inv.WeightedSpotEfficiency(torch.from_numpy(w).cuda(), p_in())
    got, val, obs = inv.grid_gradient(g_renderer(precision), torch.from_numpy(phi).cuda(), g_m)
    torch.cuda.synchronize()
    tol = 1e-12 if precision == "f64" else 1e-4
    assert sorted(got) == sorted(want) == [0, 1]
    assert rel_l2(got[0].cpu().numpy(), want[0].reshape(N, N)) <= tol
    assert val == pytest.approx(o_m.evaluate(o_obs_), rel=1e-12 if precision == "f64" else 1e-5)
    seed = g_m.obs_gradient(obs).double().cpu().numpy()
    np.testing.assert_allclose(seed, o_m.obs_gradient(o_obs_),
                               rtol=1e-15 if precision == "f64" else 1e-7, atol=0)
