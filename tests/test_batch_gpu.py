"""Batched, device-resident beamline traces (osgpu_beamline_trace_batch_device)
against the f64 oracle: ragged grid sizes, wavelengths and distances in one
call, complex64 (f32 engine, <= 1e-5) and complex128 (f64 engine, <= 1e-12)."""

import ctypes as C
import math

import numpy as np
import pytest

import optics_studio_gb300 as og
from optics_studio_gb300 import _ffi as ffi
from oracle import asm as oasm, field as ofield, element as oel, beamline as obl

from _util import rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

ITEMS = [  # n, dx, lam, z, lens f, aperture half-width
    (64, 4e-6, 450e-9, 1e-3, 0.05, 100e-6),
    (96, 3e-6, 550e-9, 4e-3, 0.08, 120e-6),
    (48, 5e-6, 650e-9, -2e-3, 0.03, 90e-6),
]


def oracle_item(n, dx, lam, z, f, half, lat, u):
    b = ofield.BandField(u, dx, dx, lam)
    bl = obl.Beamline()
    bl.push(oel.PhaseMask.sampled(lat, (n, n), (dx, dx)), 0.0)
    bl.push(oel.RectangularAperture((half, half)), 0.0)
    bl.push(oel.ThinLens.fixed(f), z)
    return bl.trace(b, obl.asm_engine(oasm.AsmConfig())).samples


@pytest.mark.parametrize("dtype,tol", [(ffi.C64, 1e-5), (ffi.C128, 1e-12)])
def test_batch_device_ragged_matches_oracle(dtype, tol):
    L = og.lib()
    tdt = torch.complex64 if dtype == ffi.C64 else torch.complex128
    rng = np.random.default_rng(7)
    keep, items, refs, outs, handles = [], [], [], [], []
    arr = (ffi.TraceItemC * len(ITEMS))()
    for i, (n, dx, lam, z, f, half) in enumerate(ITEMS):
        lat = np.floor(rng.uniform(0, 16, (n, n))) * (2 * math.pi / 16)
        u = np.exp(1j * rng.uniform(0, 0.3, (n, n)))
        refs.append(oracle_item(n, dx, lam, z, f, half, lat, u))
        h = C.c_void_p()
        ffi.check(L.osgpu_lattice_create(lat.ctypes.data_as(ffi.c_double_p), n, n, C.byref(h)))
        handles.append(h)
        tin = torch.from_numpy(u).to(device="cuda", dtype=tdt)
        tout = torch.empty_like(tin)
        outs.append(tout)
        doe = ffi.ElementC(4, 0, 0, 0, 0, 0, 0, 0, 0, 0, C.cast(h, ffi.c_double_p), n, n, dx, dx, 1)
        ap = ffi.ElementC(2, 0, half, half, 0, 0, 0, 0, 0, 0, None, 0, 0, 0, 0, 0)
        lens = ffi.ElementC(3, 0, 0, 0, 0, 0, 0, f, 0, 0, None, 0, 0, 0, 0, 0)
        e1, e2, e3 = (ffi.ElementC * 1)(doe), (ffi.ElementC * 1)(ap), (ffi.ElementC * 1)(lens)
        steps = (ffi.StepC * 3)(ffi.StepC(e1, 1, 0.0, 1.0), ffi.StepC(e2, 1, 0.0, 1.0),
                                ffi.StepC(e3, 1, z, 1.0))
        keep += [tin, e1, e2, e3, steps]
        arr[i] = ffi.TraceItemC(tin.data_ptr(), tout.data_ptr(), ffi.Grid(n, n, dx, dx, lam),
                                steps, 3)
    reps = (ffi.AsmReportC * (3 * len(ITEMS)))()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    ffi.check(L.osgpu_beamline_trace_batch_device(arr, len(ITEMS), ffi.AsmConfigC(2, 1, 1, 8, 1),
                                                  dtype, stream, reps, 3))
    torch.cuda.synchronize()
    ffi.check(L.osgpu_sync_status())
    for i, ref in enumerate(refs):
        got = outs[i].cpu().numpy().astype(np.complex128)
        assert rel_l2(got, ref) <= tol, (i, rel_l2(got, ref))
        assert reps[3 * i + 2].nx_pad >= ITEMS[i][0]
    for h in handles:
        ffi.check(L.osgpu_lattice_destroy(h))


def test_profile_reports_kernel_classes():
    L = og.lib()
    n = 64
    u = torch.ones((n, n), dtype=torch.complex64, device="cuda")
    out = torch.empty_like(u)
    ffi.check(L.osgpu_profile_begin())
    ffi.check(L.osgpu_asm_propagate_device(u.data_ptr(), out.data_ptr(), ffi.C64,
                                           ffi.Grid(n, n, 5e-6, 5e-6, 500e-9), 1e-3,
                                           ffi.AsmConfigC(2, 1, 1, 8, 1), None, None))
    stats = (ffi.KernelStatC * 16)()
    k = C.c_int32()
    ffi.check(L.osgpu_profile_end(stats, 16, C.byref(k)))
    names = {stats[i].name.decode() for i in range(k.value)}
    assert {"pass_a_rows", "pass_b_columns", "pass_c_rows"} <= names
    for i in range(k.value):
        assert stats[i].total_ms >= 0 and stats[i].launches >= 1


def ragged_items(rng, sides, n_items):
    """Gaussian-source ASM items of the ragged batch form: side from `sides`,
    z log-uniform 1-50 mm, waist 50-500 um (scaled to the grid), dx 3 um,
    lam 450-650 nm."""
    out = []
    for _ in range(n_items):
        n = int(rng.choice(sides))
        z = float(np.exp(rng.uniform(np.log(1e-3), np.log(50e-3))))
        lam = float(rng.uniform(450e-9, 650e-9))
        w0 = float(rng.uniform(50e-6, 500e-6)) * n / 2048
        out.append((n, 3e-6, lam, z, max(w0, 6e-6)))
    return out


@pytest.mark.parametrize("dtype,tol", [(ffi.C64, 1e-5), (ffi.C128, 1e-12)])
def test_ragged_batch_graph_replays_the_batch(dtype, tol):
    """osgpu_beamline_trace_batch_graph: a captured ragged batch replays
    bit-identically to the direct batched call and matches the oracle."""
    L = og.lib()
    tdt = torch.complex64 if dtype == ffi.C64 else torch.complex128
    rng = np.random.default_rng(11)
    spec = ragged_items(rng, [64, 96, 128, 256], 12)
    arr = (ffi.TraceItemC * len(spec))()
    keep, ins, outs, refs = [], [], [], []
    for i, (n, dx, lam, z, w0) in enumerate(spec):
        b = ofield.gaussian(w0, 1.0, (0.0, 0.0), 0.0, lam, n, n, dx, dx)
        if i < 4:
            refs.append(oasm.propagate(b, z, oasm.AsmConfig()).samples)
        tin = torch.from_numpy(b.samples).to("cuda", tdt)
        tout = torch.zeros_like(tin)
        steps = (ffi.StepC * 1)(ffi.StepC(None, 0, z, 1.0))
        keep += [tin, steps]
        ins.append(tin)
        outs.append(tout)
        arr[i] = ffi.TraceItemC(tin.data_ptr(), tout.data_ptr(), ffi.Grid(n, n, dx, dx, lam),
                                steps, 1)
    cfg = ffi.AsmConfigC(2, 1, 1, 8, 1)
    ffi.check(L.osgpu_beamline_trace_batch_device(arr, len(spec), cfg, dtype, None, None, 0))
    torch.cuda.synchronize()
    direct = [o.clone() for o in outs]
    for o in outs:
        o.zero_()
    g = C.c_void_p()
    ffi.check(L.osgpu_beamline_trace_batch_graph(arr, len(spec), cfg, dtype, C.byref(g)))
    for o in outs:
        o.zero_()
    torch.cuda.synchronize()
    launches0 = L.osgpu_launch_count()
    for _ in range(2):
        ffi.check(L.osgpu_graph_launch(g, None))
    torch.cuda.synchronize()
    assert L.osgpu_launch_count() == launches0  # replays launch no host-side kernels
    ffi.check(L.osgpu_sync_status())
    for d, o in zip(direct, outs):
        assert torch.equal(d, o)
    for i, ref in enumerate(refs):
        assert rel_l2(outs[i].cpu().numpy().astype(np.complex128), ref) <= tol
    ffi.check(L.osgpu_graph_destroy(g))


@pytest.mark.parametrize("pinned", [True, False])
def test_host_batch_pipeline_equals_single_calls(pinned):
    """osgpu_beamline_trace_batch (host complex128 buffers, copies pipelined
    against the traces) returns exactly what one osgpu_beamline_trace call
    per band returns."""
    L = og.lib()
    rng = np.random.default_rng(5)
    spec = [(64, 4e-6, 480e-9, 2e-3), (128, 3e-6, 520e-9, 5e-3), (96, 3e-6, 600e-9, -3e-3),
            (128, 3e-6, 640e-9, 8e-3), (64, 4e-6, 455e-9, 1e-3)]
    items = (ffi.HostTraceItemC * len(spec))()
    keep, outs, want = [], [], []
    for i, (n, dx, lam, z) in enumerate(spec):
        u = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))).astype(np.complex128)
        if pinned:
            hin = torch.from_numpy(u).pin_memory()
            hout = torch.zeros((n, n), dtype=torch.complex128).pin_memory()
            pin, pout = hin.data_ptr(), hout.data_ptr()
        else:
            hin, hout = u, np.zeros((n, n), dtype=np.complex128)
            pin, pout = hin.ctypes.data, hout.ctypes.data
        lens = (ffi.ElementC * 1)(ffi.ElementC(3, 1, 100e-6, 100e-6, 0, 0, 0, 0.04, 0, 0, None,
                                               0, 0, 0, 0, 0))
        steps = (ffi.StepC * 2)(ffi.StepC(lens, 1, z, 1.0), ffi.StepC(None, 0, z / 2, 1.0))
        keep += [hin, hout, lens, steps, u]
        outs.append(hout)
        items[i] = ffi.HostTraceItemC(C.cast(C.c_void_p(pin), ffi.c_double_p),
                                      C.cast(C.c_void_p(pout), ffi.c_double_p),
                                      ffi.Grid(n, n, dx, dx, lam), steps, 2)
        ref = np.empty_like(u)
        ffi.check(L.osgpu_beamline_trace(u.ctypes.data_as(ffi.c_double_p),
                                         ref.ctypes.data_as(ffi.c_double_p),
                                         C.byref(ffi.Grid(n, n, dx, dx, lam)), steps, 2,
                                         C.byref(ffi.AsmConfigC(2, 1, 1, 8, 1)), ffi.F32, None))
        want.append(ref)
    ffi.check(L.osgpu_beamline_trace_batch(items, len(spec), ffi.AsmConfigC(2, 1, 1, 8, 1),
                                           ffi.F32, None, 0))
    for o, w in zip(outs, want):
        got = o.numpy() if pinned else o
        assert np.array_equal(got, w)
    bad = np.full((64, 64), np.nan, dtype=np.complex128)
    items[0].in_ = bad.ctypes.data_as(ffi.c_double_p)
    code = L.osgpu_beamline_trace_batch(items, 1, ffi.AsmConfigC(2, 1, 1, 8, 1), ffi.F32, None, 0)
    assert ffi.STATUS_NAMES[code] == "NonFiniteSample"
    # reported once: the device-resident status check afterwards is clean
    ffi.check(L.osgpu_sync_status())
