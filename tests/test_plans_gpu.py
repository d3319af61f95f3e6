"""Kernel-spectrum plans (osgpu_plan_cache_*) against the oracle and the
padded f32 path.

A plan replaces an f32 ASM propagation padded above 2n by the circular
convolution of period 2n with the same kernel (built once: the kernel by the
f32 engine, its spectrum in FP64), so its results match the f64 oracle (oracle/asm.py, restating
src/propagation/asm.rs:438-538) to the f32 bounds of the padded path: 1e-5
relative L2 for fields, 1e-4 for gradients.
"""

import math

import numpy as np
import pytest

from oracle import adjoint as o_adj, asm as oasm, carrier as o_car, element as o_el
from oracle import field as ofield, merit as o_merit, observe as o_obs

from _util import rel_l2, rng_field, to_gpu_band

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from optics_studio_gb300 import inverse as inv, element as el, plans  # noqa: E402
from optics_studio_gb300.propagation import asm as gasm  # noqa: E402

# strict densification pads this geometry 256 -> 1024 at 532 nm, 10 mm
N, D, LAM, Z = 256, 3e-6, 532e-9, 10e-3


@pytest.fixture
def plans_on():
    plans.clear()
    plans.enable(1 << 30)
    yield
    plans.disable()
    plans.clear()


def band(seed=5, lam=LAM):
    return ofield.BandField(rng_field(N, N, seed=seed), D, D, lam)


def test_plan_propagation_matches_oracle_and_padded_path(plans_on):
    ob = band()
    assert oasm.resolve_report(ob, Z, oasm.AsmConfig()).padded_dims == (1024, 1024)
    ref = oasm.propagate(ob, Z)
    out1 = gasm.propagate(to_gpu_band(ob), Z, gasm.AsmConfig(), "f32")
    assert (out1.report.nx_pad, out1.report.ny_pad) == (1024, 1024)  # the reference's report
    st = plans.stats()
    assert (st["plans"], st["builds"], st["hits"]) == (1, 1, 0)
    assert st["bytes"] == (N + 1) * (N + 1) * 8
    assert rel_l2(out1.samples, ref.samples) <= 1e-5
    out2 = gasm.propagate(to_gpu_band(ob), Z, gasm.AsmConfig(), "f32")
    assert plans.stats()["hits"] == 1
    np.testing.assert_array_equal(out1.samples, out2.samples)
    # the adjoint distance uses the conjugate of the same table
    back = gasm.propagate(to_gpu_band(ob), -Z, gasm.AsmConfig(), "f32")
    assert rel_l2(back.samples, oasm.propagate(ob, -Z).samples) <= 1e-5
    assert plans.stats()["builds"] == 1
    plans.disable()
    padded = gasm.propagate(to_gpu_band(ob), Z, gasm.AsmConfig(), "f32")
    assert rel_l2(out1.samples, padded.samples) <= 1e-5


def test_plan_applies_only_to_f32_above_2n(plans_on):
    ob = band(seed=9)
    out64 = gasm.propagate(to_gpu_band(ob), Z, gasm.AsmConfig(), "f64")
    assert rel_l2(out64.samples, oasm.propagate(ob, Z).samples) <= 1e-12
    z2 = 5e-3  # pads 256 -> 512: already 2n
    assert oasm.resolve_report(ob, z2, oasm.AsmConfig()).padded_dims == (512, 512)
    gasm.propagate(to_gpu_band(ob), z2, gasm.AsmConfig(), "f32")
    assert plans.stats()["builds"] == 0


def test_plan_cache_evicts_least_recently_used():
    table = (N + 1) * (N + 1) * 8
    plans.clear()
    plans.enable(table * 3 // 2)
    try:
        a, b = band(seed=1, lam=532e-9), band(seed=2, lam=580e-9)
        za, zb = 10e-3, 8e-3  # both pad 256 -> 1024
        assert oasm.resolve_report(b, zb, oasm.AsmConfig()).padded_dims == (1024, 1024)
        ra = gasm.propagate(to_gpu_band(a), za, gasm.AsmConfig(), "f32")
        rb = gasm.propagate(to_gpu_band(b), zb, gasm.AsmConfig(), "f32")
        st = plans.stats()
        assert (st["plans"], st["builds"], st["bytes"]) == (1, 2, table)
        ra2 = gasm.propagate(to_gpu_band(a), za, gasm.AsmConfig(), "f32")
        assert plans.stats()["builds"] == 3
        np.testing.assert_array_equal(ra.samples, ra2.samples)
        assert rel_l2(rb.samples, oasm.propagate(b, zb).samples) <= 1e-5
    finally:
        plans.disable()
        plans.clear()


# inverse design: [DOE, 2 mm] [aperture r 250 um, 10 mm]; at 532 nm the second
# propagation pads to 4n (plan), at 580 nm to 2n (padded path)
BANDS = [532e-9, 580e-9]
Z1, Z2, R_AP = 2e-3, 10e-3, 250e-6


def o_source(x0, y0, lam):
    return ofield.gaussian(200e-6, 1.0, (x0, y0), 0.0, lam, N, N, D, D)


def o_design(v, lam):
    d = o_car.Design()
    d.push(o_el.PhaseMask.sampled(v, (N, N), (D, D)), Z1)
    d.push(o_el.EllipticalAperture.circle(R_AP), Z2)
    return d


def windows():
    w = np.zeros((N, N), dtype=bool)
    for cy in (96, 128, 160):
        for cx in (96, 128, 160):
            w[cy - 2:cy + 3, cx - 2:cx + 3] = True
    return w


def g_gradient(phi):
    def source(x0, y0, lam):
        return torch.from_numpy(o_source(x0, y0, lam).samples).to("cuda", torch.complex64)

    def carrier(values, lam):
        d = inv.Design()
        d.push(inv.DevicePhaseMask(values, (N, N), (D, D)), Z1)
        d.push(el.EllipticalAperture.circle(R_AP), Z2)
        return d

    rend = inv.Renderer(carrier, source, (D, D), bands=list(BANDS),
                        asm_cfg=gasm.AsmConfig(), precision="f32")
    p_in = [float(np.sum(np.abs(o_source(0.0, 0.0, lam).samples) ** 2)) for lam in BANDS]
    m = inv.SpotArrayEfficiency(torch.from_numpy(windows()).cuda(), p_in)
    g, val, obs = inv.grid_gradient(rend, torch.from_numpy(phi).cuda(), m)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in g.items()}, val, obs.data.cpu().numpy()


def test_plan_gradients_match_oracle_and_padded_path(plans_on):
    pads = [oasm.resolve_report(band(lam=lam), Z2, oasm.AsmConfig()).padded_dims[0]
            for lam in BANDS]
    assert pads == [1024, 512]
    phi = np.random.default_rng(11).uniform(0.0, 2 * math.pi, (N, N))
    got, val, obs = g_gradient(phi)
    st = plans.stats()
    assert st["builds"] == 1 and st["hits"] >= 1  # forward and adjoint share the table
    car = o_car.Carrier.analytic(N * N, 0.0, 2 * math.pi, o_design)
    p_in = [float(np.sum(np.abs(o_source(0.0, 0.0, lam).samples) ** 2)) for lam in BANDS]
    o_m = o_merit.SpotArrayEfficiency(windows(), p_in)
    rend = o_obs.Renderer(car, o_source, bands=list(BANDS), scenes=[(0.0, 0.0)],
                          asm_cfg=oasm.AsmConfig())
    want = o_adj.grid_gradient(rend, phi.reshape(-1), o_m)
    for ei in (0, 1):
        assert rel_l2(got[ei], want[ei].reshape(N, N)) <= 1e-4, ei
    ref_obs = rend.render(phi.reshape(-1)).data
    assert rel_l2(obs, ref_obs) <= 1e-5
    plans.disable()
    pad, pval, pobs = g_gradient(phi)
    for ei in (0, 1):
        assert rel_l2(got[ei], pad[ei]) <= 1e-4, ei
    assert abs(val - pval) <= 1e-5 * abs(pval)


@pytest.mark.parametrize("ny,nx,lam,z", [(256, 512, 532e-9, 10e-3), (512, 256, 580e-9, 8e-3)])
def test_plan_non_square_grid(plans_on, ny, nx, lam, z):
    ob = ofield.BandField(rng_field(ny, nx, seed=ny + nx), D, D, lam)
    py, px = oasm.resolve_report(ob, z, oasm.AsmConfig()).padded_dims[::-1]
    assert px > 2 * nx or py > 2 * ny
    out = gasm.propagate(to_gpu_band(ob), z, gasm.AsmConfig(), "f32")
    assert plans.stats()["builds"] == 1
    assert plans.stats()["bytes"] == (nx + 1) * (ny + 1) * 8
    assert rel_l2(out.samples, oasm.propagate(ob, z).samples) <= 1e-5


def test_plans_with_graph_capture_and_host_batch(plans_on):
    """A captured batch takes the padded path inside the graph (no plan is
    built or used under capture) and still matches the oracle; the host-buffer
    batch uses the plan."""
    import ctypes as C
    import optics_studio_gb300 as og
    from optics_studio_gb300 import _ffi as ffi
    L = og.lib()
    obs_ = [band(seed=s) for s in (3, 4)]
    refs = [oasm.propagate(b, Z).samples for b in obs_]
    arr = (ffi.TraceItemC * 2)()
    keep, outs = [], []
    for i, b in enumerate(obs_):
        tin = torch.from_numpy(b.samples).to("cuda", torch.complex64)
        tout = torch.zeros_like(tin)
        steps = (ffi.StepC * 1)(ffi.StepC(None, 0, Z, 1.0))
        keep += [tin, steps]
        outs.append(tout)
        arr[i] = ffi.TraceItemC(tin.data_ptr(), tout.data_ptr(), ffi.Grid(N, N, D, D, LAM), steps, 1)
    cfg = ffi.AsmConfigC(2, 1, 1, 8, 1)
    g = C.c_void_p()
    ffi.check(L.osgpu_beamline_trace_batch_graph(arr, 2, cfg, ffi.C64, C.byref(g)))
    built = plans.stats()["builds"]  # the warm-up run before capture may build the plan
    for o in outs:
        o.zero_()
    ffi.check(L.osgpu_graph_launch(g, None))
    torch.cuda.synchronize()
    ffi.check(L.osgpu_graph_destroy(g))
    assert plans.stats()["builds"] == built
    for o, r in zip(outs, refs):
        assert rel_l2(o.cpu().numpy().astype(np.complex128), r) <= 1e-5
    # host buffers (complex128), f32 engine: the plan is used
    hits0 = plans.stats()["hits"]
    hitems = (ffi.HostTraceItemC * 2)()
    hout = [np.zeros((N, N), dtype=np.complex128) for _ in obs_]
    hin = [np.ascontiguousarray(b.samples, dtype=np.complex128) for b in obs_]
    for i in range(2):
        hitems[i] = ffi.HostTraceItemC(hin[i].ctypes.data_as(ffi.c_double_p),
                                       hout[i].ctypes.data_as(ffi.c_double_p),
                                       ffi.Grid(N, N, D, D, LAM), arr[i].steps, 1)
    ffi.check(L.osgpu_beamline_trace_batch(hitems, 2, cfg, ffi.F32, None, 0))
    assert plans.stats()["hits"] >= hits0 + 2
    for o, r in zip(hout, refs):
        assert rel_l2(o, r) <= 1e-5


def test_shutdown_after_real_work_frees_caches_and_library_stays_usable():
    """osgpu_shutdown after plans, an encircled-energy merit and batched work:
    the plan cache is emptied, the pooled scratch is trimmed (free device
    memory does not drop), and later calls of every kind still work."""
    import optics_studio_gb300 as og
    from optics_studio_gb300 import _ffi
    plans.clear()
    plans.enable(1 << 30)
    ob = band(seed=9)
    first = gasm.propagate(to_gpu_band(ob), Z, gasm.AsmConfig(), "f32")
    assert plans.stats()["plans"] == 1
    obs = inv.Observation(["intensity"], [LAM], [(0.0, 0.0)], (N, N), (D, D),
                          torch.from_numpy(np.abs(ob.samples)[None, None, None] ** 2).cuda())
    ee = inv.EncircledEnergyMerit(100e-6)
    v0 = ee.evaluate(obs)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    _ffi.check(og.lib().osgpu_shutdown())
    free1 = torch.cuda.mem_get_info()[0]
    assert plans.stats()["plans"] == 0 and plans.stats()["bytes"] == 0
    assert free1 >= free0
    # usable again: a plan is rebuilt, the merit re-sorts its order
    again = gasm.propagate(to_gpu_band(ob), Z, gasm.AsmConfig(), "f32")
    np.testing.assert_array_equal(first.samples, again.samples)
    assert plans.stats()["builds"] >= 1
    assert ee.evaluate(obs) == v0
    plans.disable()
    plans.clear()
    plain = gasm.propagate(to_gpu_band(ob), Z, gasm.AsmConfig(), "f64")
    assert rel_l2(plain.samples, oasm.propagate(ob, Z).samples) <= 1e-12
