"""Kernel variants of the f32 passes and the measured schedules
(osgpu_autotune_*, optics_studio_gb300/tuning.py).

Every variant of every pass, forced through OSGPU_SCHED_A / _B / _C, gives
the f32 engine's result: within 1e-5 relative L2 of the f64 oracle
(oracle/beamline.py and oracle/asm.py, restating src/beamline.rs:109-144
and src/propagation/asm.rs:438-538) and within 1e-6 of the default
schedule's output.  The tuner records one schedule per geometry and lane
count, a batch with tuning on matches the oracle, and a second call does not
tune again.
"""

import ctypes as C
import math

import numpy as np
import pytest

from oracle import asm as oasm, beamline as obl, element as oel, field as ofield

from _util import rel_l2, rng_field

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import optics_studio_gb300 as og  # noqa: E402
from optics_studio_gb300 import _ffi as ffi, tuning  # noqa: E402
from optics_studio_gb300.propagation.asm import AsmConfig  # noqa: E402

# 512^2 padded to 1024^2 (r = 2, m = 512): every row-tile and persistent
# variant is eligible at this size
N, D, LAM, Z = 512, 3e-6, 532e-9, 2e-3
HALF = 0.6e-3
VARIANTS = {
    "OSGPU_SCHED_A": ["bulk", "tstore", "tile4", "tile2", "g1", "g2", "g4"],
    "OSGPU_SCHED_B": ["pair", "g1", "g2", "g4"],
    "OSGPU_SCHED_C": ["tma", "pipe", "tile2", "tile4", "g1", "g2", "g4"],
}


def fields():
    return [rng_field(N, N, seed=40 + i) for i in range(2)]


@pytest.fixture(scope="module")
def oracle_out():
    out = []
    for u in fields():
        bl = obl.Beamline()
        bl.push(oel.RectangularAperture((HALF, HALF)), Z)
        out.append(bl.trace(ofield.BandField(u, D, D, LAM), obl.asm_engine(oasm.AsmConfig())).samples)
    return out


def run_batch():
    """Two items (two lanes) of [square aperture, ASM Z], complex64 on the device."""
    L = og.lib()
    fin = torch.stack([torch.from_numpy(u).to(torch.complex64) for u in fields()]).cuda()
    fout = torch.full_like(fin, complex(math.nan, math.nan))
    ap = (ffi.ElementC * 1)(ffi.ElementC(2, 0, HALF, HALF, 0, 0, 0, 0, 0, 0, None, 0, 0, 0, 0, 0))
    steps = (ffi.StepC * 1)(ffi.StepC(ap, 1, Z, 1.0))
    items = (ffi.TraceItemC * 2)(*[ffi.TraceItemC(fin[i].data_ptr(), fout[i].data_ptr(),
                                                  ffi.Grid(N, N, D, D, LAM), steps, 1)
                                   for i in range(2)])
    ffi.check(L.osgpu_beamline_trace_batch_device(items, 2, ffi.AsmConfigC(2.0, 1, 1, 8.0, 1.0),
                                                  ffi.C64, None, None, 0))
    torch.cuda.synchronize()
    ffi.check(L.osgpu_sync_status())
    return fout.cpu().numpy().astype(np.complex128)


def test_every_pass_variant_matches_oracle_and_default(monkeypatch, oracle_out):
    for var in VARIANTS:
        monkeypatch.delenv(var, raising=False)
    base = run_batch()
    for i in range(2):
        assert rel_l2(base[i], oracle_out[i]) <= 1e-5
    for var, names in VARIANTS.items():
        for name in names:
            monkeypatch.setenv(var, name)
            got = run_batch()
            for i in range(2):
                assert rel_l2(got[i], oracle_out[i]) <= 1e-5, (var, name)
                assert rel_l2(got[i], base[i]) <= 1e-6, (var, name)
        monkeypatch.delenv(var)


def test_autotune_records_schedules_and_batch_matches_oracle(oracle_out):
    tuning.clear()
    grid = ffi.Grid(N, N, D, D, LAM)
    info = tuning.tune(grid, Z, AsmConfig(), lanes=1)
    assert info["m"] == (512, 512) and info["r"] == (2, 2) and info["lanes"] == 1
    assert info["pass_a"] in ["default"] + VARIANTS["OSGPU_SCHED_A"]
    assert info["pass_b"] in ["default"] + VARIANTS["OSGPU_SCHED_B"]
    assert info["pass_c"] in ["default"] + VARIANTS["OSGPU_SCHED_C"]
    assert 0.0 < info["ms_best"] <= info["ms_default"]
    tuning.enable()
    try:
        got = run_batch()  # tunes the two-lane schedule of this geometry first
        scheds = tuning.schedules()
        assert sorted(s["lanes"] for s in scheds) == [1, 2]
        for i in range(2):
            assert rel_l2(got[i], oracle_out[i]) <= 1e-5
        again = run_batch()  # cached: no new schedule
        assert len(tuning.schedules()) == 2
        np.testing.assert_array_equal(got, again)
    finally:
        tuning.disable()
        tuning.clear()
    assert tuning.schedules() == []
