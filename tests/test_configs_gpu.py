"""Parity at the full sizes of the benchmarked workloads, through the C ABI,
against the f64 oracle (oracle/*.py):

* 2048^2 batched BandField beamline (32 bands 450-650 nm, dx 3 um, [16-level
  DOE, square aperture 5 mm, lens f 100 mm, ASM 100 mm], strict densification
  to 8192^2): the first and last band of the batch through
  osgpu_beamline_trace_batch_device, f32 <= 1e-5 and FP64 <= 1e-12 relative L2
  against oracle.beamline (restating src/beamline.rs:109-144 and
  src/propagation/asm.rs:438-538).
* 1024^2 single-plane engine sweep (dx 4 um, 532 nm, unit plane wave x
  8-level DOE x thin lens f 50 mm): Fresnel transfer function 50 mm and
  convolution 200 mm (src/propagation/fresnel.rs:430,531), Fraunhofer 50 mm
  with strict off (fraunhofer.rs:364) and Rayleigh-Sommerfeld 5 mm with
  strict off (rayleigh_sommerfeld.rs:384, whose strict guard rejects this
  case), FP64 <= 1e-12 and f32 <= 1e-5, reports identical to the oracle's.
* 2048^2 Gerchberg-Saxton (Fraunhofer far field, spot-array target): the
  FP64 loop iterate for iterate (merit history 1e-10) and the fused f32 loop
  (merit history 1e-4) against the oracle loop (crates/optics-inverse/src/
  gs.rs:482-578).
* 2048^2 adjoint inverse design ([DOE, 20 mm] [aperture 6 mm, 80 mm], 9 x 9
  Gaussian spot-array efficiency): central differences with h = 1e-4 rad on
  64 seeded pixels (FP64 renders) against the FP64 and f32 adjoint
  gradients, and the oracle's grid_gradient (adjoint.rs:268-340) on one band.

The workloads are the benchmark's own (bench.py), so these tests pin the
configurations the throughput is reported on.
"""

import ctypes as C
import math

import numpy as np
import pytest

import bench
from oracle import asm as oasm, fresnel as ofr, fraunhofer as ofh, rs as ors
from oracle import field as ofield, element as oel, beamline as obl
from oracle import adjoint as o_adj, carrier as o_car, merit as o_merit, observe as o_obs
from oracle import gs as o_gs

from _util import rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import optics_studio_gb300 as og  # noqa: E402
from optics_studio_gb300 import _ffi as ffi, element as gel  # noqa: E402
from optics_studio_gb300 import inverse as inv, gs as ggs  # noqa: E402
from optics_studio_gb300.field import BandField  # noqa: E402
from optics_studio_gb300.propagation import fresnel as gfr, fraunhofer as gfh  # noqa: E402
from optics_studio_gb300.propagation import rayleigh_sommerfeld as grs  # noqa: E402
from optics_studio_gb300.propagation.asm import AsmConfig  # noqa: E402
from optics_studio_gb300.propagation.fraunhofer import FraunhoferConfig  # noqa: E402

TOL64 = 1e-12
TOL32 = 1e-5

# ---------------------------------------------------------------- beamline batch

N = bench.N
C3_BANDS = (0, 31)  # 450 nm and 650 nm


def oracle_band(lam, lat):
    b = ofield.plane_wave(0.0, 0.0, 1.0, N, N, bench.DX, bench.DX, lam)
    bl = obl.Beamline()
    bl.push(oel.PhaseMask.sampled(lat, (N, N), (bench.DX, bench.DX)), 0.0)
    bl.push(oel.RectangularAperture((bench.HALF_AP, bench.HALF_AP)), 0.0)
    bl.push(oel.ThinLens.fixed(bench.F_LENS), bench.Z)
    return bl.trace(b, obl.asm_engine(oasm.AsmConfig())).samples


@pytest.fixture(scope="module")
def c3():
    lat = bench.doe_lattice()
    lams = np.linspace(450e-9, 650e-9, 32)
    ref = {b: oracle_band(float(lams[b]), lat) for b in C3_BANDS}
    return lat, lams, ref


def trace_batch(lat, lams, dtype):
    """The benchmark's items for the given wavelengths, device resident."""
    L = og.lib()
    cdt = torch.complex128 if dtype == ffi.C128 else torch.complex64
    handle = C.c_void_p()
    ffi.check(L.osgpu_lattice_create(lat.ctypes.data_as(ffi.c_double_p), N, N, C.byref(handle)))
    try:
        fin = torch.ones((len(lams), N, N), dtype=cdt, device="cuda")
        fout = torch.full_like(fin, complex(math.nan, math.nan))
        keep = []
        items = (ffi.TraceItemC * len(lams))()
        for b, lam in enumerate(lams):
            doe = ffi.ElementC(4, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                               C.cast(C.c_void_p(handle.value), ffi.c_double_p), N, N, bench.DX,
                               bench.DX, 1)
            ap = ffi.ElementC(2, 0, bench.HALF_AP, bench.HALF_AP, 0, 0, 0, 0, 0, 0, None, 0, 0,
                              0, 0, 0)
            lens = ffi.ElementC(3, 0, 0, 0, 0, 0, 0, bench.F_LENS, 0, 0, None, 0, 0, 0, 0, 0)
            e = [(ffi.ElementC * 1)(x) for x in (doe, ap, lens)]
            steps = (ffi.StepC * 3)(ffi.StepC(e[0], 1, 0.0, 1.0), ffi.StepC(e[1], 1, 0.0, 1.0),
                                    ffi.StepC(e[2], 1, bench.Z, 1.0))
            keep += e + [steps]
            items[b] = ffi.TraceItemC(fin[b].data_ptr(), fout[b].data_ptr(),
                                      ffi.Grid(N, N, bench.DX, bench.DX, float(lam)), steps, 3)
        cfg = ffi.AsmConfigC(2.0, 1, 1, 8.0, 1.0)
        reps = (ffi.AsmReportC * (3 * len(lams)))()
        ffi.check(L.osgpu_beamline_trace_batch_device(items, len(lams), cfg, dtype, None, reps,
                                                      3))
        torch.cuda.synchronize()
        ffi.check(L.osgpu_sync_status())
        return fout.cpu().numpy().astype(np.complex128), [reps[3 * b + 2] for b in range(len(lams))]
    finally:
        L.osgpu_lattice_destroy(handle)


def test_c3_batch_f32_matches_oracle(c3):
    lat, lams, ref = c3
    out, reps = trace_batch(lat, [lams[b] for b in C3_BANDS], ffi.C64)
    for i, b in enumerate(C3_BANDS):
        # the strict densification ladder picks the oracle's padded grid
        ob = ofield.BandField(np.ones((N, N), complex), bench.DX, bench.DX, float(lams[b]))
        want = oasm.resolve_report(ob, bench.Z, oasm.AsmConfig())
        assert (reps[i].nx_pad, reps[i].ny_pad) == want.padded_dims == (8192, 8192)
        assert reps[i].used_padding == want.used_padding == 4.0
        assert reps[i].max_phase_step_x == want.max_phase_step_x
        err = rel_l2(out[i], ref[b])
        assert err <= TOL32, (b, err)


def test_c3_batch_f64_matches_oracle(c3):
    lat, lams, ref = c3
    out, _ = trace_batch(lat, [lams[0]], ffi.C128)
    assert rel_l2(out[0], ref[0]) <= TOL64


# ---------------------------------------------------------------- engine sweep

C2_N, C2_DX, C2_LAM, C2_F, C2_SEED = 1024, 4e-6, 532e-9, 50e-3, 808


def c2_lattice():
    rng = np.random.default_rng(C2_SEED)
    return np.floor(rng.uniform(0, 8, (C2_N, C2_N))) * (2 * math.pi / 8)


@pytest.fixture(scope="module")
def c2():
    lat = c2_lattice()
    ob = ofield.plane_wave(0.0, 0.0, 1.0, C2_N, C2_N, C2_DX, C2_DX, C2_LAM)
    ob = oel.PhaseMask.sampled(lat, (C2_N, C2_N), (C2_DX, C2_DX)).apply(ob)
    ob = oel.ThinLens.fixed(C2_F).apply(ob)
    return lat, ob


def c2_gpu_input(lat, prec):
    """Plane wave x DOE x lens applied on the device (elements of the plane)."""
    b = BandField(np.ones((C2_N, C2_N), complex), C2_DX, C2_DX, C2_LAM)
    return gel.apply_elements(b, [gel.PhaseMask.sampled(lat, (C2_N, C2_N), (C2_DX, C2_DX)),
                                  gel.ThinLens.fixed(C2_F)], prec)


@pytest.mark.parametrize("prec,tol", [("f64", TOL64), ("f32", TOL32)])
def test_c2_engine_sweep_matches_oracle(c2, prec, tol):
    lat, ob = c2
    g = c2_gpu_input(lat, prec)
    assert rel_l2(g.samples, ob.samples) <= (1e-14 if prec == "f64" else 2e-7)
    # identical inputs from here on: each engine alone against the oracle
    gin = BandField(ob.samples, C2_DX, C2_DX, C2_LAM)
    errs = {}
    r = gfr.propagate(gin, 50e-3, gfr.FresnelConfig(), prec)
    want = ofr.propagate(ob, 50e-3, ofr.FresnelConfig())
    assert (r.report.nx_pad, r.report.ny_pad) == (2048, 2048)
    errs["fresnel_tf"] = rel_l2(r.samples, want.samples)
    r = gfr.propagate_convolution(gin, 200e-3, gfr.FresnelConfig(), prec)
    want = ofr.propagate_convolution(ob, 200e-3, ofr.FresnelConfig())
    errs["fresnel_conv"] = rel_l2(r.samples, want.samples)
    r = gfh.propagate(gin, 50e-3, gfh.FraunhoferConfig(strict=False), prec)
    want = ofh.propagate(ob, 50e-3, ofh.FraunhoferConfig(strict=False))
    assert (r.dx, r.dy) == (want.dx, want.dy)
    errs["fraunhofer"] = rel_l2(r.samples, want.samples)
    r = grs.propagate(gin, 5e-3, grs.RayleighSommerfeldConfig(strict=False), prec)
    want = ors.propagate(ob, 5e-3, ors.RayleighSommerfeldConfig(strict=False))
    errs["rayleigh_sommerfeld"] = rel_l2(r.samples, want.samples)
    for k, e in errs.items():
        assert e <= tol, (k, e)


def test_c2_guard_reports_match_oracle(c2):
    """The strict guards: RS at 5 mm raises AliasingRisk in both (the report
    carried by the error matches), Fraunhofer at 50 mm fails its regime check
    when strict; the Fresnel reports of the two forms pass."""
    lat, ob = c2
    gin = BandField(ob.samples, C2_DX, C2_DX, C2_LAM)
    with pytest.raises(ors.RayleighSommerfeldError) as eo:
        ors.propagate(ob, 5e-3, ors.RayleighSommerfeldConfig())
    with pytest.raises(og.OsgpuError) as eg:
        grs.propagate(gin, 5e-3, grs.RayleighSommerfeldConfig())
    assert eg.value.variant == eo.value.variant == "AliasingRisk"
    ro, rg = eo.value.report, eg.value.report
    assert (rg.nx_pad, rg.ny_pad) == ro.padded_dims
    assert rg.max_kernel_step_x == ro.max_kernel_step_x
    assert rg.max_kernel_step_y == ro.max_kernel_step_y
    with pytest.raises(ofh.FraunhoferError) as eo:
        ofh.propagate(ob, 50e-3, ofh.FraunhoferConfig())
    with pytest.raises(og.OsgpuError) as eg:
        gfh.propagate(gin, 50e-3, gfh.FraunhoferConfig())
    assert eg.value.variant == eo.value.variant == "RegimeViolation"
    for z in (50e-3, 200e-3):
        ro = ofr.sampling_report(ob, z, ofr.FresnelConfig())
        rg = gfr.sampling_report(gin, z, gfr.FresnelConfig())
        assert (rg.nx_pad, rg.ny_pad) == ro.padded_dims
        assert rg.max_phase_step_x == ro.max_phase_step_x
        assert rg.max_kernel_step_x == ro.max_kernel_step_x
        assert bool(rg.nyquist_ok) == ro.nyquist_ok
        assert bool(rg.kernel_nyquist_ok) == ro.kernel_nyquist_ok


# ---------------------------------------------------------------- GS

GS_ITERS = 5


@pytest.fixture(scope="module")
def gs_case():
    rng = np.random.default_rng(bench.GS_SEED)
    tamp, _ = bench.gs_targets(1, rng)[0]
    init = rng.uniform(-math.pi, math.pi, (N, N))
    c = bench.DX * bench.DX / (bench.GS_LAM * bench.GS_Z)
    tamp = tamp * (c * N * N)
    u = np.ones((N, N), dtype=np.complex128)
    cfg = ofh.FraunhoferConfig(strict=False)
    fwd = lambda s: ofh.propagate(ofield.BandField(s, bench.DX, bench.DX, bench.GS_LAM),
                                  bench.GS_Z, cfg).samples
    back = lambda s: o_gs.fraunhofer_adjoint(s, N, N, bench.DX, bench.DX, bench.GS_LAM,
                                             bench.GS_Z)
    tint = tamp * tamp
    merit = lambda inten: float(np.sum((inten - tint) ** 2) / inten.size)
    want = o_gs.run(u, np.ones((N, N), bool), tamp, -math.pi, math.pi, init, fwd, back, merit,
                    max_iterations=GS_ITERS, patience=GS_ITERS + 1, illum=np.abs(u))
    return u, tamp, init, want


def gs_problem(u, tamp, init, dtype):
    cdt, rdt = ((torch.complex64, torch.float32) if dtype == "f32"
                else (torch.complex128, torch.float64))
    cfg = ggs.GsConfig(max_iterations=GS_ITERS, patience=GS_ITERS + 1)
    return ggs.GsProblem(torch.from_numpy(u).to("cuda", cdt), (bench.DX, bench.DX), bench.GS_LAM,
                         bench.GS_Z, torch.from_numpy(tamp).to("cuda", rdt),
                         torch.from_numpy(init).to("cuda", rdt), config=cfg,
                         engine="fraunhofer", fraunhofer=FraunhoferConfig(strict=False))


@pytest.mark.parametrize("dtype,tol", [("f64", 1e-10), ("f32", 1e-4)])
def test_c4_gs_2048_follows_oracle(gs_case, dtype, tol):
    u, tamp, init, want = gs_case
    got = ggs.run(gs_problem(u, tamp, init, dtype))
    assert got.iterations == want.iterations == GS_ITERS
    assert got.best_iteration == want.best_iteration
    for hg, hw in zip(got.history, want.history):
        assert hg["merit"] == pytest.approx(hw.merit, rel=tol)
        assert hg["amplitude_mse"] == pytest.approx(hw.amplitude_mse, rel=tol)
    bi = got.target_intensity.double().cpu().numpy()
    assert rel_l2(bi, want.target_intensity) <= (1e-9 if dtype == "f64" else 1e-4)


# ---------------------------------------------------------------- adjoint

ADJ_BAND = float(bench.ADJ_LAMS[0])


def adj_renderer(precision, lam):
    cdt = torch.complex128 if precision == "f64" else torch.complex64
    src = torch.ones((N, N), dtype=cdt, device="cuda")

    def carrier(values, lam_):
        v = values.float() if precision == "f32" else values
        d = inv.Design()
        d.push(inv.DevicePhaseMask(v, (N, N), (bench.DX, bench.DX)), bench.ADJ_Z1)
        d.push(gel.EllipticalAperture.circle(bench.ADJ_R), bench.ADJ_Z2)
        return d

    return inv.Renderer(carrier, lambda x0, y0, l: src, (bench.DX, bench.DX), bands=[lam],
                        asm_cfg=AsmConfig(), precision=precision)


@pytest.fixture(scope="module")
def adj_case():
    phi = bench.adjoint_phases()
    w = bench.adjoint_spot_weights()
    merit = inv.WeightedSpotEfficiency(torch.from_numpy(w).cuda(), [float(N * N)])
    g64, val64, _ = inv.grid_gradient(adj_renderer("f64", ADJ_BAND),
                                      torch.from_numpy(phi).cuda(), merit)
    g32, val32, _ = inv.grid_gradient(adj_renderer("f32", ADJ_BAND),
                                      torch.from_numpy(phi).cuda(), merit)
    torch.cuda.synchronize()
    return phi, w, merit, g64[0].cpu().numpy(), val64, g32[0].cpu().numpy(), val32


def test_c5_adjoint_matches_central_differences(adj_case):
    phi, w, merit, g64, val64, g32, val32 = adj_case
    assert val32 == pytest.approx(val64, rel=1e-5)
    flat = g64.reshape(-1)
    cand = np.flatnonzero(np.abs(flat) >= 0.05 * np.abs(flat).max())
    idx = np.random.default_rng(64).choice(cand, 64, replace=False)
    rend = adj_renderer("f64", ADJ_BAND)
    h = 1e-4
    fd = np.empty(len(idx))
    base = phi.reshape(-1)
    for j, i in enumerate(idx):
        vp = base.copy(); vp[i] += h
        vm = base.copy(); vm[i] -= h
        fp = merit.evaluate(rend.render(torch.from_numpy(vp.reshape(N, N)).cuda()))
        fm = merit.evaluate(rend.render(torch.from_numpy(vm.reshape(N, N)).cuda()))
        fd[j] = (fp - fm) / (2 * h)
    a64 = flat[idx]
    a32 = g32.reshape(-1)[idx]
    assert np.all(np.abs(a64 - fd) <= 1e-4 * np.abs(fd)), np.max(np.abs(a64 - fd) / np.abs(fd))
    assert np.linalg.norm(a32 - fd) <= 1e-4 * np.linalg.norm(fd)
    # the f32 gradient over the whole grid against the FP64 engine
    assert rel_l2(g32, g64) <= 1e-4


def test_c5_adjoint_matches_oracle_grid_gradient(adj_case):
    phi, w, merit, g64, val64, g32, val32 = adj_case

    def design(v, lam):
        d = o_car.Design()
        d.push(oel.PhaseMask.sampled(v, (N, N), (bench.DX, bench.DX)), bench.ADJ_Z1)
        d.push(oel.EllipticalAperture.circle(bench.ADJ_R), bench.ADJ_Z2)
        return d

    car = o_car.Carrier.analytic(N * N, 0.0, 2 * math.pi, design)
    src = lambda x0, y0, lam: ofield.plane_wave(0.0, 0.0, 1.0, N, N, bench.DX, bench.DX, lam)
    rend = o_obs.Renderer(car, src, bands=[ADJ_BAND], asm_cfg=oasm.AsmConfig())
    om = o_merit.WeightedSpotEfficiency(w, [float(N * N)])
    want = o_adj.grid_gradient(rend, phi.reshape(-1), om)
    assert sorted(want) == [0, 1]
    ref = want[0].reshape(N, N)
    assert rel_l2(g64, ref) <= TOL64
    assert rel_l2(g32, ref) <= 1e-4
    assert val64 == pytest.approx(om.evaluate(rend.render(phi.reshape(-1))), rel=1e-12)
