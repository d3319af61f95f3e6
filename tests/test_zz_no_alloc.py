"""osgpu_asm_propagate_noalloc: the ASM propagation for callers that cannot
let a library allocate device memory (an application whose device memory is
owned by its own allocator, latency-critical loops that cannot absorb
cudaMalloc's synchronisation, host processes that forbid a library from
allocating).  Its output must match the allocating device entry point,
osgpu_asm_propagate_device, and the f64 oracle (oracle/asm.py, restating
src/propagation/asm.rs:438-538) within the f32 tolerance of the other parity
tests (1e-5 relative L2), on two calls in a row (the second call reuses the
static scratch array the first one left behind), at a register-FFT size and
at a mixed-radix size.  Free device memory must not change across a call
once the first call has looked up the scratch array (a coarse check: the
driver reports free memory in pages, and every buffer this propagation would
need spans at least one).

This file is named to be collected last, so a run that stops at the first
failure has run every other test before it; it also passes alone in a fresh
process (the first call performs the one-time address lookup)."""

import math

import numpy as np
import pytest

import optics_studio_gb300 as og
from optics_studio_gb300 import _ffi as ffi
from oracle import asm as oasm, field as ofield

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL32 = 1e-5


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


CASES = [
    # nx, ny, d, (padding, band_limited, strict, max_padding, medium), padded, calls (lam, z)
    (256, 256, 4e-6, (2.0, 1, 1, 8.0, 1.0), (512, 512), [(500e-9, 2e-3), (633e-9, -1.5e-3)]),
    (300, 200, 4e-6, (2.0, 0, 0, 8.0, 1.3), (600, 400), [(532e-9, 1e-3), (450e-9, -0.7e-3)]),
]


@pytest.mark.parametrize("case", CASES)
def test_noalloc_matches_oracle_and_allocating_entry_point_on_two_calls(case):
    nx, ny, d, cfg_t, padded, calls = case
    L = og.lib()
    rng = np.random.default_rng(2024 + nx)
    cfg = ffi.AsmConfigC(*cfg_t)
    ocfg = oasm.AsmConfig(cfg_t[0], bool(cfg_t[1]), bool(cfg_t[2]), cfg_t[3], cfg_t[4])
    for call, (lam, z) in enumerate(calls):
        u = (rng.normal(size=(ny, nx)) + 1j * rng.normal(size=(ny, nx))).astype(np.complex64)
        tin = torch.from_numpy(u).cuda()
        ref = torch.empty_like(tin)
        out = torch.full_like(tin, complex(math.nan, math.nan))
        g = ffi.Grid(nx, ny, d, d, lam)
        ffi.check(L.osgpu_asm_propagate_device(tin.data_ptr(), ref.data_ptr(), ffi.C64, g, z, cfg,
                                               None, None))
        torch.cuda.synchronize()
        rep = ffi.AsmReportC()
        free0 = torch.cuda.mem_get_info()[0]
        code = L.osgpu_asm_propagate_noalloc(tin.data_ptr(), out.data_ptr(), g, z, cfg, None, rep)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        assert code == 0, ffi.last_error()
        if call > 0:  # the first call may load the module holding the static array
            assert free1 == free0
        assert (rep.nx_pad, rep.ny_pad) == padded
        got = out.cpu().numpy().astype(np.complex128)
        want = ref.cpu().numpy().astype(np.complex128)
        oracle = oasm.propagate(ofield.BandField(u.astype(np.complex128), d, d, lam), z,
                                ocfg).samples
        assert np.all(np.isfinite(got))
        assert rel_l2(got, want) <= TOL32
        assert rel_l2(got, oracle) <= TOL32


def test_noalloc_rejects_sizes_beyond_its_scratch():
    L = og.lib()
    n = 2048
    t = torch.zeros((4, 4), dtype=torch.complex64, device="cuda")
    g = ffi.Grid(n, n, 3e-6, 3e-6, 500e-9)
    cfg = ffi.AsmConfigC(2.0, 1, 1, 8.0, 1.0)  # 2048^2 padded to >= 4096^2: > 32 MiB
    code = L.osgpu_asm_propagate_noalloc(t.data_ptr(), t.data_ptr(), g, 0.1, cfg, None, None)
    assert ffi.STATUS_NAMES[code] == "Unsupported"
    assert "exceeds" in ffi.last_error()
