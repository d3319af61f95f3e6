"""Device-resident field handles (osgpu_field_*): zero fill, upload/download
round trips in both storage types, and a handle's buffer driven through
osgpu_asm_propagate_device against the oracle (oracle/asm.py, restating
src/propagation/asm.rs:438-538): f64 engine within 1e-12, f32 within 1e-5
relative L2."""

import ctypes as C

import numpy as np
import pytest

from oracle import asm as oasm, field as ofield

from _util import rel_l2, rng_field

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

import optics_studio_gb300 as og  # noqa: E402
from optics_studio_gb300 import _ffi  # noqa: E402
from optics_studio_gb300.propagation import asm as gasm  # noqa: E402

N, D, LAM, Z = 64, 4e-6, 532e-9, 2e-3


def create(dtype):
    h = C.c_void_p()
    _ffi.check(og.lib().osgpu_field_create(N, N, dtype, C.byref(h)))
    return h


@pytest.mark.parametrize("dtype", [_ffi.C128, _ffi.C64])
def test_field_handle_round_trip(dtype):
    L = og.lib()
    src = np.ascontiguousarray(rng_field(N, N, seed=3), dtype=np.complex128)
    h = create(dtype)
    try:
        out = np.full((N, N), 1.0 + 1.0j)
        _ffi.check(L.osgpu_field_download(h, out.ctypes.data, None))
        assert np.all(out == 0)
        _ffi.check(L.osgpu_field_upload(h, src.ctypes.data, None))
        _ffi.check(L.osgpu_field_download(h, out.ctypes.data, None))
        want = src if dtype == _ffi.C128 else src.astype(np.complex64).astype(np.complex128)
        np.testing.assert_array_equal(out, want)
        p, nx, ny, dt = C.c_void_p(), C.c_uint64(), C.c_uint64(), C.c_int32()
        _ffi.check(L.osgpu_field_info(h, C.byref(p), C.byref(nx), C.byref(ny), C.byref(dt)))
        assert p.value and (nx.value, ny.value, dt.value) == (N, N, dtype)
    finally:
        _ffi.check(L.osgpu_field_destroy(h))


@pytest.mark.parametrize("dtype,tol", [(_ffi.C128, 1e-12), (_ffi.C64, 1e-5)])
def test_field_handles_through_device_propagation(dtype, tol):
    L = og.lib()
    ob = ofield.BandField(rng_field(N, N, seed=8), D, D, LAM)
    want = oasm.propagate(ob, Z).samples
    hin, hout = create(dtype), create(dtype)
    try:
        src = np.ascontiguousarray(ob.samples, dtype=np.complex128)
        _ffi.check(L.osgpu_field_upload(hin, src.ctypes.data, None))
        pin, pout = C.c_void_p(), C.c_void_p()
        _ffi.check(L.osgpu_field_info(hin, C.byref(pin), None, None, None))
        _ffi.check(L.osgpu_field_info(hout, C.byref(pout), None, None, None))
        rep = _ffi.AsmReportC()
        _ffi.check(L.osgpu_asm_propagate_device(pin, pout, dtype, _ffi.Grid(N, N, D, D, LAM), Z,
                                                gasm.AsmConfig().c(), None, rep))
        _ffi.check(L.osgpu_sync_status())
        out = np.empty((N, N), dtype=np.complex128)
        _ffi.check(L.osgpu_field_download(hout, out.ctypes.data, None))
        assert rel_l2(out, want) <= tol
    finally:
        _ffi.check(L.osgpu_field_destroy(hin))
        _ffi.check(L.osgpu_field_destroy(hout))
