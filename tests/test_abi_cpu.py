"""CPU tests of the C ABI: the library builds and exports every symbol of
include/osgpu.h, and its host-side analysis (which picks the padded grid and
fills the reports) matches the f64 oracle bit for bit.  No GPU needed."""

import ctypes
import math
import pathlib
import re

import numpy as np
import pytest

import optics_studio_gb300 as og
from optics_studio_gb300 import _ffi
from optics_studio_gb300.field import BandField
from optics_studio_gb300.propagation import asm as gasm, fresnel as gfr, fraunhofer as gfh
from optics_studio_gb300.propagation import rayleigh_sommerfeld as grs
from oracle import asm as oasm, fresnel as ofr, fraunhofer as ofh, rs as ors, field as ofield

HEADER = pathlib.Path(__file__).resolve().parents[1] / "include" / "osgpu.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(osgpu_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = og.lib()
    syms = declared_symbols()
    assert len(syms) >= 17
    for s in syms:
        assert hasattr(L, s), s
    bound = {n for n, _, _ in _ffi.SIGNATURES}
    assert set(syms) == bound


# ctypes mirror of each struct typedef of the header
STRUCTS = {
    "osgpu_grid": "Grid", "osgpu_asm_config": "AsmConfigC", "osgpu_asm_report": "AsmReportC",
    "osgpu_fresnel_config": "FresnelConfigC", "osgpu_fresnel_report": "FresnelReportC",
    "osgpu_fraunhofer_config": "FraunhoferConfigC",
    "osgpu_fraunhofer_report": "FraunhoferReportC", "osgpu_rs_config": "RsConfigC",
    "osgpu_rs_report": "RsReportC", "osgpu_element": "ElementC", "osgpu_step": "StepC",
    "osgpu_trace_item": "TraceItemC", "osgpu_kernel_stat": "KernelStatC",
    "osgpu_frame": "FrameC", "osgpu_adam_config": "AdamConfigC",
    "osgpu_gs_config": "GsConfigC", "osgpu_gs_record": "GsRecordC",
    "osgpu_gs_result": "GsResultC", "osgpu_gs_item": "GsItemC",
    "osgpu_host_trace_item": "HostTraceItemC", "osgpu_plan_stats": "PlanStatsC",
    "osgpu_schedule_info": "ScheduleInfoC",
}


def test_struct_layouts_match_header_sizes(tmp_path):
    """Every struct typedef of the header has a ctypes mirror of the same size,
    with sizes taken from the header compiled by the host C compiler."""
    import shutil
    import subprocess
    typedefs = set(re.findall(r"\}\s*(osgpu_[a-z0-9_]+)\s*;", HEADER.read_text()))
    assert typedefs == set(STRUCTS), typedefs ^ set(STRUCTS)
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    src = tmp_path / "sizes.c"
    body = "".join(f'  printf("{t} %zu\\n", sizeof({t}));\n' for t in sorted(STRUCTS))
    src.write_text(f'#include <stdio.h>\n#include "{HEADER}"\nint main(void) {{\n{body}  return 0;\n}}\n')
    exe = tmp_path / "sizes"
    subprocess.run([cc, "-std=c99", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    sizes = {k: int(v) for k, v in (ln.split() for ln in out.splitlines())}
    for t, name in STRUCTS.items():
        assert ctypes.sizeof(getattr(_ffi, name)) == sizes[t], (t, sizes[t])


GEOMS = [
    # (nx, ny, dx, dy, lam, z, padding, band_limited, strict, max_padding, medium)
    (512, 512, 2e-6, 2e-6, 633e-9, 10e-3, 2.0, True, True, 8.0, 1.0),
    (2048, 2048, 3e-6, 3e-6, 450e-9, 0.1, 2.0, True, True, 8.0, 1.0),
    (2048, 2048, 3e-6, 3e-6, 650e-9, 1e-3, 2.0, True, True, 8.0, 1.0),
    (64, 64, 1e-6, 1e-6, 500e-9, 7.68e-4, 1.0, False, True, 8.0, 1.0),
    (32, 32, 1e-6, 1e-6, 500e-9, 0.5, 2.0, False, False, 8.0, 1.5),
    (45, 37, 4e-6, 5e-6, 532e-9, -2e-3, 1.5, True, True, 8.0, 1.3),
    (1536, 1536, 20e-6, 20e-6, 500e-9, 40.0, 2.0, True, True, 8.0, 1.0),
]


@pytest.mark.parametrize("geom", GEOMS)
def test_asm_sampling_report_matches_oracle(geom):
    nx, ny, dx, dy, lam, z, pad, bl, strict, mp, med = geom
    cfg = gasm.AsmConfig(pad, bl, strict, mp, med)
    gb = BandField(np.zeros((1, 1), complex), dx, dy, lam)
    grid = _ffi.Grid(nx, ny, dx, dy, lam)
    rep = _ffi.AsmReportC()
    assert og.lib().osgpu_asm_sampling_report(grid, z, cfg.c(), rep) == 0
    ob = ofield.BandField(np.zeros((ny, nx), complex), dx, dy, lam)
    oref = oasm.sampling_report(ob, z, oasm.AsmConfig(pad, bl, strict, mp, med))
    assert (rep.nx_pad, rep.ny_pad) == oref.padded_dims
    for a, b in [(rep.band_limit_fx, oref.band_limit_fx), (rep.band_limit_fy, oref.band_limit_fy),
                 (rep.max_phase_step_x, oref.max_phase_step_x),
                 (rep.max_phase_step_y, oref.max_phase_step_y)]:
        assert a == b
    assert bool(rep.nyquist_ok) == oref.nyquist_ok


@pytest.mark.parametrize("geom", GEOMS)
def test_asm_densification_ladder_matches_oracle(geom):
    """The padded grid the propagation runs on (asm.rs:465-479) — resolved on
    the host before any device work, so it is observable without a GPU."""
    nx, ny, dx, dy, lam, z, pad, bl, strict, mp, med = geom
    cfg = gasm.AsmConfig(pad, bl, strict, mp, med)
    ob = ofield.BandField(np.zeros((ny, nx), complex), dx, dy, lam)
    try:
        oref = oasm.resolve_report(ob, z, oasm.AsmConfig(pad, bl, strict, mp, med))
        want = 0
    except oasm.PropagationError as e:
        oref = e.report
        want = 6
    rep = _ffi.AsmReportC()
    buf = np.zeros((ny, nx), complex)
    code = og.lib().osgpu_asm_propagate(buf.ctypes.data_as(_ffi.c_double_p),
                                        buf.ctypes.data_as(_ffi.c_double_p),
                                        _ffi.Grid(nx, ny, dx, dy, lam), z, cfg.c(), 0, rep)
    if want == 6:
        assert code == 6
    else:
        assert code in (0, 103)  # 103 = no device here
    assert (rep.nx_pad, rep.ny_pad) == oref.padded_dims
    assert rep.used_padding == oref.used_padding


@pytest.mark.parametrize("z", [50e-3, 200e-3, -5e-3, 1e-4])
def test_fresnel_report_matches_oracle(z):
    for pad in (1.0, 2.0, 3.5):
        cfg = gfr.FresnelConfig(pad, True, 8.0)
        ob = ofield.BandField(np.zeros((100, 120), complex), 4e-6, 3e-6, 532e-9)
        rep = _ffi.FresnelReportC()
        og.lib().osgpu_fresnel_sampling_report(_ffi.Grid(120, 100, 4e-6, 3e-6, 532e-9), z,
                                               cfg.c(), rep)
        o = ofr.sampling_report(ob, z, ofr.FresnelConfig(pad, True, 8.0))
        assert (rep.nx_pad, rep.ny_pad) == o.padded_dims
        assert rep.max_phase_step_x == o.max_phase_step_x
        assert rep.max_kernel_step_y == o.max_kernel_step_y
        assert rep.max_phase_error_vs_asm == o.max_phase_error_vs_asm
        assert bool(rep.kernel_nyquist_ok) == o.kernel_nyquist_ok


def test_fraunhofer_and_rs_reports_match_oracle():
    ob = ofield.BandField(np.zeros((31, 33), complex), 10e-6, 12e-6, 633e-9)
    for cfgp in [gfh.FraunhoferConfig(), gfh.FraunhoferConfig(True, 0.1, (1e-5, -2e-5), None),
                 gfh.FraunhoferConfig(False, 1.0, None, 2e-4)]:
        rep = _ffi.FraunhoferReportC()
        og.lib().osgpu_fraunhofer_regime_report(_ffi.Grid(33, 31, 10e-6, 12e-6, 633e-9), -0.3,
                                                cfgp.c(), rep)
        o = ofh.regime_report(ob, -0.3, ofh.FraunhoferConfig(cfgp.strict, cfgp.max_n_f,
                                                             cfgp.source_pos,
                                                             cfgp.aperture_extent))
        assert (rep.dx_out, rep.dy_out) == o.output_pitch
        assert (rep.n_f_x, rep.n_f_y) == (o.n_f_x, o.n_f_y)
        assert bool(rep.regime_ok) == o.regime_ok and rep.extent_used == o.extent_used
    rr = _ffi.RsReportC()
    og.lib().osgpu_rs_sampling_report(_ffi.Grid(33, 31, 10e-6, 12e-6, 633e-9), 5e-3,
                                      grs.RayleighSommerfeldConfig().c(), rr)
    o = ors.sampling_report(ob, 5e-3, ors.RayleighSommerfeldConfig())
    assert (rr.max_kernel_step_x, rr.max_phase_error_vs_fresnel) == (
        o.max_kernel_step_x, o.max_phase_error_vs_fresnel)


def test_host_validation_errors_without_device():
    L = og.lib()
    buf = np.zeros((8, 8), complex)
    p = buf.ctypes.data_as(_ffi.c_double_p)
    g = _ffi.Grid(8, 8, 20e-6, 20e-6, 500e-9)
    assert L.osgpu_asm_propagate(p, p, g, float("nan"), gasm.AsmConfig().c(), 0, None) == 1
    assert L.osgpu_asm_propagate(p, p, g, 1e-3, gasm.AsmConfig(medium=0.0).c(), 0, None) == 3
    assert L.osgpu_asm_propagate(p, p, _ffi.Grid(8, 8, 20e-6, 20e-6, -1.0), 1e-3,
                                 gasm.AsmConfig().c(), 0, None) == 2
    assert L.osgpu_fraunhofer_propagate(p, p, g, 0.0, gfh.FraunhoferConfig().c(), 0, None) == 1
    assert L.osgpu_rs_propagate(p, p, g, 0.0, grs.RayleighSommerfeldConfig().c(), 0, None) == 1
    # z == 0 is the identity (asm.rs:461-463) and needs no device; NaN is still rejected
    src = np.arange(64, dtype=float).reshape(8, 8) + 0j
    out = np.zeros_like(src)
    assert L.osgpu_asm_propagate(src.ctypes.data_as(_ffi.c_double_p),
                                 out.ctypes.data_as(_ffi.c_double_p), g, 0.0,
                                 gasm.AsmConfig().c(), 0, None) == 0
    assert np.array_equal(out, src)
    src[3, 3] = np.nan
    assert L.osgpu_asm_propagate(src.ctypes.data_as(_ffi.c_double_p),
                                 out.ctypes.data_as(_ffi.c_double_p), g, 0.0,
                                 gasm.AsmConfig().c(), 0, None) == 5


def test_observation_dlpack_export_is_zero_copy():
    """observe.rs:10-16 layout [C][B][S][Ny][Nx] exported through DLPack in place."""
    torch = pytest.importorskip("torch")
    from optics_studio_gb300.inverse import Observation
    data = torch.arange(2 * 3 * 1 * 4 * 5, dtype=torch.float64).reshape(2, 3, 1, 4, 5)
    obs = Observation(["intensity", "d_dx"], [5e-7, 6e-7, 7e-7], [(0.0, 0.0)], (5, 4),
                      (1e-6, 1e-6), data)
    view = np.from_dlpack(obs)
    assert view.shape == (2, 3, 1, 4, 5)
    data[1, 2, 0, 3, 4] = -1.0
    assert view[1, 2, 0, 3, 4] == -1.0  # same memory


# the reference unit tests' guard geometries (fresnel.rs, fraunhofer.rs,
# rayleigh_sommerfeld.rs): the product's host decision (status before any
# device work) equals the oracle's outcome
ERR = {"AliasingRisk": 6, "RegimeViolation": 7, "InvalidDistance": 1}
GUARD_CASES = [
    ("fresnel", 32, 1e-6, 3e-4, (1.0, True, 1.0)),
    ("fresnel", 32, 1e-6, 3e-4, (1.0, False, 1.0)),
    ("fresnel", 32, 1e-6, 3e-4, (1.0, True, 8.0)),
    ("fresnel", 64, 1e-6, 5e-4, (1.0, True, 1.0)),
    ("fresnel_conv", 64, 1e-6, 5e-4, (1.0, True, 1.0)),
    ("fresnel", 8, 20e-6, math.inf, (2.0, True, 8.0)),
    ("fresnel_conv", 8, 20e-6, math.nan, (2.0, True, 8.0)),
    ("rs", 64, 10e-6, 1e-3, (1.0, True)),
    ("rs", 64, 10e-6, 1e-3, (1.0, False)),
    ("rs", 8, 20e-6, 0.0, (2.0, True)),
    ("fraunhofer", 64, 1e-5, 0.01, (True, 1.0, None, None)),
    ("fraunhofer", 64, 1e-5, 0.01, (False, 1.0, None, None)),
    ("fraunhofer", 64, 1e-5, 0.05, (True, 1.0, None, 1e-4)),
    ("fraunhofer", 64, 1e-5, 0.05, (True, 1.0, None, 0.0)),
    ("fraunhofer", 8, 20e-6, 0.0, (False, 1.0, None, None)),
]


@pytest.mark.parametrize("case", GUARD_CASES)
def test_guard_decisions_match_oracle(case):
    from optics_studio_gb300.propagation import rayleigh_sommerfeld as grs
    from oracle import rs as ors
    engine, n, d, z, cargs = case
    lam = 500e-9
    ob = ofield.BandField(np.ones((n, n), complex), d, d, lam)
    o_fn, o_cfg, g_fn, g_cfg = {
        "fresnel": (ofr.propagate, ofr.FresnelConfig, og.lib().osgpu_fresnel_propagate,
                    gfr.FresnelConfig),
        "fresnel_conv": (ofr.propagate_convolution, ofr.FresnelConfig,
                         og.lib().osgpu_fresnel_propagate_convolution, gfr.FresnelConfig),
        "rs": (ors.propagate, ors.RayleighSommerfeldConfig, og.lib().osgpu_rs_propagate,
               grs.RayleighSommerfeldConfig),
        "fraunhofer": (ofh.propagate, ofh.FraunhoferConfig, og.lib().osgpu_fraunhofer_propagate,
                       gfh.FraunhoferConfig),
    }[engine]
    try:
        o_fn(ob, z, o_cfg(*cargs))
        want = None
    except Exception as e:  # the oracle's typed error
        want = ERR[e.variant]
    rep = {"fresnel": _ffi.FresnelReportC, "fresnel_conv": _ffi.FresnelReportC,
           "rs": _ffi.RsReportC, "fraunhofer": _ffi.FraunhoferReportC}[engine]()
    buf = np.ones((n, n), complex)
    code = g_fn(buf.ctypes.data_as(_ffi.c_double_p), buf.ctypes.data_as(_ffi.c_double_p),
                _ffi.Grid(n, n, d, d, lam), z, g_cfg(*cargs).c(), 0, rep)
    if want is None:
        assert code in (0, 103)  # 103 = no device here
    else:
        assert code == want


def test_renderer_rejects_empty_axes_and_bad_steps_before_device_work():
    """observe.rs:214-230: no band or scene, or a non-positive / non-finite
    finite-difference step of a requested channel, is a Render error raised
    before the source or any device call."""
    pytest.importorskip("torch")
    from optics_studio_gb300 import inverse as inv

    def never(*_):
        raise AssertionError("the renderer must validate before building frames")

    for kw in ({"bands": []}, {"scenes": []}, {"deriv_x": True, "scene_step": 0.0},
               {"deriv_y": True, "scene_step": math.inf},
               {"deriv_lambda": True, "lambda_step": -1e-9},
               {"deriv_lambda": True, "lambda_step": math.nan}):
        r = inv.Renderer(never, never, (1e-6, 1e-6), **kw)
        with pytest.raises(og.OsgpuError) as e:
            r.render(None)
        assert e.value.variant == "Render"


def test_field_handles_validate_without_device():
    """osgpu_field_*: argument checks come before any device call; without a
    GPU a well-formed create reports NoDevice."""
    L = og.lib()
    h = ctypes.c_void_p()
    assert L.osgpu_field_create(0, 4, 0, ctypes.byref(h)) == 102
    assert L.osgpu_field_create(4, 4, 7, ctypes.byref(h)) == 102
    assert L.osgpu_field_create(4, 4, 0, None) == 102
    assert h.value is None
    assert L.osgpu_field_upload(None, None, None) == 102
    assert L.osgpu_field_download(None, None, None) == 102
    assert L.osgpu_field_info(None, None, None, None, None) == 102
    assert L.osgpu_field_destroy(None) == 0
    assert L.osgpu_shutdown() == 0  # nothing initialised: a no-op
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = False
    if not has_gpu:
        assert L.osgpu_field_create(4, 4, 0, ctypes.byref(h)) == 103
        assert h.value is None


def test_fd_gradient_matches_reference_unit_tests():
    """fd.rs fd_gradient_matches_closed_form (1e-6), fd_gradient_uses_params_steps_and_clamps_probes
    (1.75 exactly), zero_width_slot_is_ignored, gradient_rejects_bad_inputs."""
    pytest.importorskip("torch")
    from optics_studio_gb300 import inverse as inv
    unit = [inv.Param(f"x{i}", -1.0, 1.0) for i in range(3)]
    t = [0.3, -0.2, 0.5]
    bowl = lambda v: sum((a - b) ** 2 for a, b in zip(v, t)) + v[0] * v[1]
    x = [0.1, 0.05, -0.4]
    g, ev = inv.fd_gradient(unit, bowl, x)
    want = [2 * (a - b) for a, b in zip(x, t)]
    want[0] += x[1]
    want[1] += x[0]
    assert ev == 6
    assert all(abs(a - b) < 1e-6 * (1 + abs(b)) for a, b in zip(g, want))
    g, ev = inv.fd_gradient([inv.Param("x", 0.0, 1.0, 1.0, 0.25)], lambda v: v[0] * v[0], [1.0])
    assert ev == 2 and abs(g[0] - 1.75) < 1e-12
    g, ev = inv.fd_gradient([inv.Param("k", 2.0, 2.0, 2.0), inv.Param("x", 0.0, 1.0, 0.5)],
                            lambda v: v[0] + v[1] * v[1], [2.0, 0.5])
    assert ev == 2 and g[0] == 0.0 and abs(g[1] - 1.0) < 1e-9
    two = unit[:2]
    for bad, code in (([0.0], 40), ([math.nan, 0.0], 41), ([0.0, 2.0], 42)):
        with pytest.raises(og.OsgpuError) as e:
            inv.fd_gradient(two, lambda v: 1.0, bad)
        assert e.value.code == code


def test_gs_setup_validation_before_device_work():
    """gs.rs run_rejects_invalid_setup (GsVariant::validate, gs.rs:165-178):
    DVR beta outside (0, 2), FPR beta outside (0, 1] and zero iterations are
    Render errors, an unknown variant or engine a bad argument - all decided
    before any device call."""
    L = og.lib()
    items = (_ffi.GsItemC * 1)()
    asm_c = gasm.AsmConfig().c()
    fr_c = gfh.FraunhoferConfig().c()

    def run(variant, beta, iters=10, engine=0):
        cfg = _ffi.GsConfigC(iters, 10, 1e-4, variant, beta, -math.pi, math.pi, engine)
        return L.osgpu_gs_run_batch_device(items, 1, cfg, asm_c, fr_c, 0, None)

    assert run(1, 3.0) == 43 and run(1, 0.0) == 43 and run(1, math.nan) == 43
    assert run(2, 0.0) == 43 and run(2, 1.5) == 43
    assert run(0, 1.0, iters=0) == 43
    assert run(7, 1.0) == 102 and run(0, 1.0, engine=5) == 102


def test_adam_config_validation_before_device_work():
    """fd.rs adam_config_validation_errors (AdamConfig::validate, fd.rs:95-121):
    lr_frac 0 or NaN, beta1 = 1, beta2 < 0, infinite eps and a zero clip norm
    are Render errors, decided before any device access (the device pointers
    below are never dereferenced)."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("host-only check: its placeholder device pointers stay off a real device")
    L = og.lib()
    fake = ctypes.c_void_p(16)

    def step(lr=0.02, b1=0.9, b2=0.999, eps=1e-8, clip_norm=1.0, clip=1):
        cfg = _ffi.AdamConfigC(lr, b1, b2, eps, clip_norm, clip)
        return L.osgpu_adam_step_device(fake, None, fake, 0, fake, fake, 4, ctypes.byref(cfg), 1,
                                        -1.0, 1.0, None)

    for kw in ({"lr": 0.0}, {"lr": math.nan}, {"b1": 1.0}, {"b2": -0.1}, {"eps": math.inf},
               {"clip_norm": 0.0}):
        assert step(**kw) == 43, kw


def test_gaussian_spot_array_target():
    """Host-side target of the spot-array merit: peak 1 at every centre of the
    centred count x count array, mirror-symmetric about the grid centre for
    an odd count on an odd grid."""
    from optics_studio_gb300.inverse import gaussian_spot_array
    w = gaussian_spot_array((129, 129), 3, 20, 2.0)
    for i in (-1, 0, 1):
        for j in (-1, 0, 1):
            assert abs(w[64 + 20 * i, 64 + 20 * j] - 1.0) < 1e-9
    assert np.allclose(w, w[::-1, ::-1])
    assert w.min() >= 0.0 and w.max() <= 1.0 + 1e-9
