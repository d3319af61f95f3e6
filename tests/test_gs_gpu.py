"""Gerchberg-Saxton on the GPU against the oracle loop (oracle/gs.py, a
restatement of crates/optics-inverse/src/gs.rs:347-597).

The FP64 engine follows the oracle iterate for iterate: merit and
amplitude-MSE histories to 1e-10 relative and the best phase to 1e-9
relative L2 over the first iterations (the loop is a projection iteration:
rounding-level differences of the propagations, <= 1e-12, are not
amplified over a few iterations).  The f32 engine follows the merit history
to 1e-4 relative.
"""

import math

import numpy as np
import pytest

from oracle import gs as o_gs, asm as o_asm, fraunhofer as o_fr, field as o_field

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from optics_studio_gb300 import gs as ggs, _ffi  # noqa: E402
from optics_studio_gb300.element import ClearAperture  # noqa: E402
from optics_studio_gb300.propagation.asm import AsmConfig  # noqa: E402
from optics_studio_gb300.propagation.fraunhofer import FraunhoferConfig  # noqa: E402

N, D, LAM = 64, 8e-6, 532e-9


def spot_target(n, seed=1):
    rng = np.random.default_rng(seed)
    k = 4
    t = np.zeros((n, n))
    yy, xx = np.mgrid[0:n, 0:n]
    for i in range(k):
        for j in range(k):
            cy, cx = (i + 1) * n // (k + 1), (j + 1) * n // (k + 1)
            t += rng.uniform(0.5, 1.0) * np.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / (2 * 2.0 ** 2))
    return np.sqrt(t) * 40.0


def oracle_run(engine, u_in, open_mask, tamp, init, z, iters, patience=1000, beta_f=1.0,
               beta_p=1.0):
    if engine == "asm":
        cfg = o_asm.AsmConfig(band_limited=False, strict=False)
        half = z / 2.0
        fwd = lambda s: o_asm.propagate(o_field.BandField(s, D, D, LAM), half, cfg).samples
        back = lambda s: o_asm.propagate(o_field.BandField(s, D, D, LAM), -half, cfg).samples
        illum = None
    else:
        cfg = o_fr.FraunhoferConfig(strict=False)
        fwd = lambda s: o_fr.propagate(o_field.BandField(s, D, D, LAM), z, cfg).samples
        back = lambda s: o_gs.fraunhofer_adjoint(s, N, N, D, D, LAM, z)
        illum = np.abs(u_in)
    tint = tamp * tamp
    merit = lambda inten: float(np.sum((inten - tint) ** 2) / inten.size)
    return o_gs.run(u_in, open_mask, tamp, -math.pi, math.pi, init, fwd, back, merit,
                    max_iterations=iters, patience=patience, beta_f=beta_f, beta_p=beta_p,
                    illum=illum)


def gpu_problem(engine, u_in, tamp, init, z, iters, dtype, patience=1000, variant="classic",
                beta=1.0, aperture=None):
    cdt = torch.complex128 if dtype == "f64" else torch.complex64
    rdt = torch.float64 if dtype == "f64" else torch.float32
    cfg = ggs.GsConfig(max_iterations=iters, patience=patience, variant=variant, beta=beta)
    return ggs.GsProblem(torch.from_numpy(u_in).to("cuda", cdt), (D, D), LAM, z,
                         torch.from_numpy(tamp).to("cuda", rdt),
                         torch.from_numpy(init).to("cuda", rdt),
                         aperture=aperture or ClearAperture.field(), config=cfg, engine=engine,
                         asm=AsmConfig(band_limited=False, strict=False),
                         fraunhofer=FraunhoferConfig(strict=False))


def inputs(engine):
    rng = np.random.default_rng(3)
    if engine == "asm":
        u = o_field.gaussian(150e-6, 1.0, (0.0, 0.0), 0.0, LAM, N, N, D, D).samples
        z = 4e-3
    else:
        u = np.ones((N, N), dtype=np.complex128)
        z = 50e-3
    init = rng.uniform(-math.pi, math.pi, (N, N))
    tamp = spot_target(N)
    if engine == "asm":
        tamp = tamp * math.sqrt(np.sum(np.abs(u) ** 2) / np.sum(tamp ** 2))
    else:
        scale = (D * D / (LAM * z)) * math.sqrt(np.sum(np.abs(u) ** 2))
        tamp = tamp / math.sqrt(np.sum(tamp ** 2)) * scale
    return u, tamp, init, z


@pytest.mark.parametrize("engine", ["asm", "fraunhofer"])
def test_gs_f64_follows_oracle(engine):
    u, tamp, init, z = inputs(engine)
    iters = 6
    want = oracle_run(engine, u, np.ones((N, N), bool), tamp, init, z, iters)
    got = ggs.run(gpu_problem(engine, u, tamp, init, z, iters, "f64"))
    assert got.iterations == want.iterations == iters
    assert got.best_iteration == want.best_iteration
    for hg, hw in zip(got.history, want.history):
        assert hg["merit"] == pytest.approx(hw.merit, rel=1e-10)
        assert hg["amplitude_mse"] == pytest.approx(hw.amplitude_mse, rel=1e-10)
        assert hg["phase_update_rms"] == pytest.approx(hw.phase_update_rms, rel=1e-8)
    ph = got.phase.cpu().numpy()
    assert np.linalg.norm(ph - want.phase) / np.linalg.norm(want.phase) <= 1e-9
    np.testing.assert_allclose(got.illumination_amplitude.cpu().numpy(),
                               want.illumination_amplitude, rtol=1e-12, atol=1e-12)
    bi = got.target_intensity.cpu().numpy()
    assert np.linalg.norm(bi - want.target_intensity) / np.linalg.norm(want.target_intensity) <= 1e-9
    te = got.target_amplitude_error.cpu().numpy()
    assert (np.linalg.norm(te - want.target_amplitude_error)
            <= 1e-9 * np.linalg.norm(want.target_amplitude_error))
    pe = got.phase_error.cpu().numpy()
    assert np.linalg.norm(pe - want.phase_error) <= 1e-9 * np.linalg.norm(want.phase_error)


def test_gs_f32_fraunhofer_follows_oracle_merit():
    u, tamp, init, z = inputs("fraunhofer")
    iters = 12
    want = oracle_run("fraunhofer", u, np.ones((N, N), bool), tamp, init, z, iters)
    got = ggs.run(gpu_problem("fraunhofer", u, tamp, init, z, iters, "f32"))
    for hg, hw in zip(got.history, want.history):
        assert hg["merit"] == pytest.approx(hw.merit, rel=1e-4)
    assert got.merit == pytest.approx(want.merit, rel=1e-4)


def test_gs_patience_stop_and_variants():
    u, tamp, init, z = inputs("fraunhofer")
    want = oracle_run("fraunhofer", u, np.ones((N, N), bool), tamp, init, z, 60, patience=3,
                      beta_p=1.5)
    got = ggs.run(gpu_problem("fraunhofer", u, tamp, init, z, 60, "f64", patience=3,
                              variant="dvr", beta=1.5))
    assert got.converged == want.converged
    assert got.iterations == want.iterations
    assert got.best_iteration == want.best_iteration
    with pytest.raises(_ffi.OsgpuError) as e:
        ggs.run(gpu_problem("fraunhofer", u, tamp, init, z, 5, "f64", variant="fpr", beta=1.5))
    assert e.value.variant == "Render"


def test_gs_aperture_and_batch():
    """Two problems in one call, one with a circular carrier aperture."""
    u, tamp, init, z = inputs("fraunhofer")
    open_mask = (o_field.axis_coords(N, D)[None, :] ** 2
                 + o_field.axis_coords(N, D)[:, None] ** 2) <= (200e-6) ** 2
    want0 = oracle_run("fraunhofer", u, np.ones((N, N), bool), tamp, init, z, 4)
    want1 = oracle_run("fraunhofer", u, open_mask, tamp, init, z, 4)
    p0 = gpu_problem("fraunhofer", u, tamp, init, z, 4, "f64")
    p1 = gpu_problem("fraunhofer", u, tamp, init, z, 4, "f64",
                     aperture=ClearAperture.circle(200e-6))
    g0, g1 = ggs.run_batch([p0, p1])
    for g, w in ((g0, want0), (g1, want1)):
        assert g.merit == pytest.approx(w.merit, rel=1e-10)
        ph = g.phase.cpu().numpy()
        assert np.linalg.norm(ph - w.phase) / np.linalg.norm(w.phase) <= 1e-9


def inputs_fraunhofer(n, seed=3):
    rng = np.random.default_rng(seed)
    u = np.ones((n, n), dtype=np.complex128)
    z = 50e-3
    init = rng.uniform(-math.pi, math.pi, (n, n))
    tamp = spot_target(n, seed)
    scale = (D * D / (LAM * z)) * math.sqrt(np.sum(np.abs(u) ** 2))
    return u, tamp / math.sqrt(np.sum(tamp ** 2)) * scale, init, z


def oracle_fraunhofer(n, u, tamp, init, z, iters, patience=1000):
    cfg = o_fr.FraunhoferConfig(strict=False)
    fwd = lambda s: o_fr.propagate(o_field.BandField(s, D, D, LAM), z, cfg).samples
    back = lambda s: o_gs.fraunhofer_adjoint(s, n, n, D, D, LAM, z)
    tint = tamp * tamp
    merit = lambda inten: float(np.sum((inten - tint) ** 2) / inten.size)
    return o_gs.run(u, np.ones((n, n), bool), tamp, -math.pi, math.pi, init, fwd, back, merit,
                    max_iterations=iters, patience=patience, illum=np.abs(u))


def fraunhofer_problem(n, u, tamp, init, z, iters, patience=1000):
    cfg = ggs.GsConfig(max_iterations=iters, patience=patience)
    return ggs.GsProblem(torch.from_numpy(u).to("cuda", torch.complex64), (D, D), LAM, z,
                         torch.from_numpy(tamp).to("cuda", torch.float32),
                         torch.from_numpy(init).to("cuda", torch.float32), config=cfg,
                         engine="fraunhofer", fraunhofer=FraunhoferConfig(strict=False))


def test_gs_fused_f32_follows_oracle_at_256():
    """The fused f32 Fraunhofer kernels (square power-of-two grids) against the
    oracle loop: merit history to 1e-4, same best iteration, best intensity
    to 1e-4 relative L2."""
    n = 256
    u, tamp, init, z = inputs_fraunhofer(n)
    want = oracle_fraunhofer(n, u, tamp, init, z, 10)
    got = ggs.run(fraunhofer_problem(n, u, tamp, init, z, 10))
    assert got.iterations == 10
    for hg, hw in zip(got.history, want.history):
        assert hg["merit"] == pytest.approx(hw.merit, rel=1e-4)
        assert hg["amplitude_mse"] == pytest.approx(hw.amplitude_mse, rel=1e-4)
    assert got.best_iteration == want.best_iteration
    bi = got.target_intensity.cpu().numpy()
    assert np.linalg.norm(bi - want.target_intensity) / np.linalg.norm(want.target_intensity) <= 1e-4
    # |U| - T of the last iteration (written column-major in the loop, transposed at the end)
    te = got.target_amplitude_error.cpu().numpy()
    assert (np.linalg.norm(te - want.target_amplitude_error)
            <= 1e-4 * np.linalg.norm(want.target_amplitude_error))


def test_gs_fused_matches_generic_path_and_patience(monkeypatch):
    n = 256
    u, tamp, init, z = inputs_fraunhofer(n, seed=8)
    probs = lambda: [fraunhofer_problem(n, u, tamp, init, z, 40, patience=4),
                     fraunhofer_problem(n, u, tamp * 0.9, init, z, 40, patience=4)]
    fused = ggs.run_batch(probs())
    monkeypatch.setenv("OSGPU_GS_GENERIC", "1")
    generic = ggs.run_batch(probs())
    for f, g in zip(fused, generic):
        assert f.iterations == g.iterations
        assert f.converged == g.converged
        for hf, hg in zip(f.history, g.history):
            assert hf["merit"] == pytest.approx(hg["merit"], rel=1e-4)


def test_gs_row_pass_tma_staging_matches_direct_gather(monkeypatch):
    """The fused row pass with its inputs staged by TMA (spectrum tiles, phase
    and amplitude rows of the next unit prefetched) computes exactly what the
    direct-gather row pass computes: identical merit histories and phases."""
    n = 512
    u, tamp, init, z = inputs_fraunhofer(n, seed=12)
    probs = lambda: [fraunhofer_problem(n, u, tamp, init, z, 6),
                     fraunhofer_problem(n, u, tamp * 0.8, init, z, 6)]
    monkeypatch.delenv("OSGPU_GS_TMA", raising=False)
    staged = ggs.run_batch(probs())
    monkeypatch.setenv("OSGPU_GS_TMA", "0")
    direct = ggs.run_batch(probs())
    for s, d in zip(staged, direct):
        assert [h["merit"] for h in s.history] == [h["merit"] for h in d.history]
        assert torch.equal(s.phase, d.phase)
    want = oracle_fraunhofer(n, u, tamp, init, z, 6)
    for hg, hw in zip(staged[0].history, want.history):
        assert hg["merit"] == pytest.approx(hw.merit, rel=1e-4)
