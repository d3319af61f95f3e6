"""osgpu_asm_propagate_noalloc: the ASM propagation for callers that cannot
let a library allocate device memory (code under CUDA graph capture, memory
owned by another allocator, latency-critical loops).  Its output must match
the allocating device entry point, osgpu_asm_propagate_device, within the
f32 tolerance of the other parity tests, on two calls in a row (the second
call reuses the static scratch array the first one left behind).

This file is named to be collected last, so a run that stops at the first
failure has run every other test before it; it also passes alone in a fresh
process (the first call performs the one-time address lookup)."""

import math

import numpy as np
import pytest

import optics_studio_gb300 as og
from optics_studio_gb300 import _ffi as ffi

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL32 = 1e-5


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    L = og.lib()
    n, d = 256, 4e-6
    rng = np.random.default_rng(2024)
    cfg = ffi.AsmConfigC(2.0, 1, 1, 8.0, 1.0)
    for lam, z in [(500e-9, 2e-3), (633e-9, -1.5e-3)]:
        u = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))).astype(np.complex64)
        tin = torch.from_numpy(u).cuda()
        ref = torch.empty_like(tin)
        out = torch.full_like(tin, complex(math.nan, math.nan))
        g = ffi.Grid(n, n, d, d, lam)
        ffi.check(L.osgpu_asm_propagate_device(tin.data_ptr(), ref.data_ptr(), ffi.C64, g, z, cfg,
                                               None, None))
        torch.cuda.synchronize()
        rep = ffi.AsmReportC()
        code = L.osgpu_asm_propagate_noalloc(tin.data_ptr(), out.data_ptr(), g, z, cfg, None, rep)
        assert code == 0
        torch.cuda.synchronize()
        assert (rep.nx_pad, rep.ny_pad) == (512, 512)
        got = out.cpu().numpy().astype(np.complex128)
        want = ref.cpu().numpy().astype(np.complex128)
        assert np.all(np.isfinite(got))
        assert rel_l2(got, want) <= TOL32


def test_noalloc_rejects_sizes_beyond_its_scratch():
    L = og.lib()
    n = 2048
    t = torch.zeros((4, 4), dtype=torch.complex64, device="cuda")
    g = ffi.Grid(n, n, 3e-6, 3e-6, 500e-9)
    cfg = ffi.AsmConfigC(2.0, 1, 1, 8.0, 1.0)  # 2048^2 padded to >= 4096^2: > 32 MiB
    code = L.osgpu_asm_propagate_noalloc(t.data_ptr(), t.data_ptr(), g, 0.1, cfg, None, None)
    assert ffi.STATUS_NAMES[code] == "Unsupported"
