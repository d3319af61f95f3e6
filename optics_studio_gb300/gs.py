"""Gerchberg-Saxton on the GPU (mirror of crates/optics-inverse/src/gs.rs).

``run(problem)`` / ``run_batch(problems)`` drive ``osgpu_gs_run_batch_device``:
one call runs every problem's loop on the device (mask, half-transform,
target-plane projection with the MseToTarget merit and the Eq. 5.18
amplitude MSE, back-propagation, DOE-plane update, best-so-far and
patience stop), and returns ``GsSolution`` objects whose arrays are device
tensors.  Two engines: the reference's ASM relay (``engine="asm"``, DOE at
z_total / 2) and the Fraunhofer far field with its exact adjoint
(``engine="fraunhofer"``, DOE at the input plane).
"""

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional

from . import _ffi
from .element import ClearAperture
from .propagation.asm import AsmConfig
from .propagation.fraunhofer import FraunhoferConfig

CLASSIC, DVR, FPR = "classic", "dvr", "fpr"
_VARIANT = {CLASSIC: 0, DVR: 1, FPR: 2}
_ENGINE = {"asm": 0, "fraunhofer": 1}


@dataclass
class GsConfig:
    """gs.rs:197-221 (GsInit::Given: the initial phase is GsProblem.init_phase)."""
    max_iterations: int = 100
    patience: int = 10
    merit_tolerance: float = 1e-4
    variant: str = CLASSIC
    beta: float = 1.0  # Dvr / Fpr beta


@dataclass
class GsProblem:
    """gs.rs:223-250 with the carrier reduced to its aperture and bounds."""
    input: object             # device complex tensor (ny, nx)
    pitch: tuple
    lam: float
    z: float                  # asm: z_total; fraunhofer: DOE -> target distance
    target_amplitude: object  # device real tensor (ny, nx)
    init_phase: object        # device real tensor (ny, nx)
    lo: float = -3.141592653589793
    hi: float = 3.141592653589793
    aperture: ClearAperture = field(default_factory=ClearAperture.field)
    center: tuple = (0.0, 0.0)
    target_intensity: Optional[object] = None  # MseToTarget target (default T^2)
    config: GsConfig = field(default_factory=GsConfig)
    engine: str = "fraunhofer"
    asm: AsmConfig = field(default_factory=AsmConfig)
    fraunhofer: FraunhoferConfig = field(default_factory=lambda: FraunhoferConfig(strict=False))


@dataclass
class GsSolution:
    """gs.rs:268-306."""
    phase: object
    merit: float
    best_iteration: int
    amplitude_mse: float
    converged: bool
    iterations: int
    history: list
    target_intensity: object
    target_amplitude_error: object
    phase_error: object
    illumination_amplitude: object
    last_phase: object


def run(problem, stream=None):
    return run_batch([problem], stream)[0]


def run_batch(problems, stream=None):
    """Runs every problem (same config, engine and precision) in one call."""
    import torch
    from .inverse import _stream_handle
    if not problems:
        return []
    p0 = problems[0]
    c128 = p0.input.dtype == torch.complex128
    rdt = torch.float64 if c128 else torch.float32
    cfg = p0.config
    gcfg = _ffi.GsConfigC(cfg.max_iterations, cfg.patience, cfg.merit_tolerance,
                          _VARIANT[cfg.variant], cfg.beta, p0.lo, p0.hi, _ENGINE[p0.engine])
    items = (_ffi.GsItemC * len(problems))()
    keep, outs = [], []
    for i, p in enumerate(problems):
        ny, nx = p.input.shape
        phase = p.init_phase.to(rdt).contiguous().clone()
        o = {k: torch.empty((ny, nx), dtype=rdt, device=p.input.device)
             for k in ("last", "best_int", "terr", "perr", "illum")}
        hist = (_ffi.GsRecordC * cfg.max_iterations)()
        tamp = p.target_amplitude.to(rdt).contiguous()
        tint = p.target_intensity.to(rdt).contiguous() if p.target_intensity is not None else None
        inp = p.input.contiguous()
        keep.extend([tamp, tint, inp, hist])
        ap = p.aperture
        items[i] = _ffi.GsItemC(
            _ffi.Grid(nx, ny, p.pitch[0], p.pitch[1], p.lam), p.z, ap.kind, ap.a, ap.b,
            p.center[0], p.center[1], inp.data_ptr(), tamp.data_ptr(),
            tint.data_ptr() if tint is not None else None, phase.data_ptr(),
            o["last"].data_ptr(), o["best_int"].data_ptr(), o["terr"].data_ptr(),
            o["perr"].data_ptr(), o["illum"].data_ptr(), hist, _ffi.GsResultC())
        outs.append((phase, o, hist))
    _ffi.check(_ffi.lib().osgpu_gs_run_batch_device(
        items, len(problems), gcfg, p0.asm.c(), p0.fraunhofer.c(),
        _ffi.C128 if c128 else _ffi.C64, _stream_handle(stream)))
    sols = []
    for i, (phase, o, hist) in enumerate(outs):
        r = items[i].result
        h = [dict(iteration=int(hist[k].iteration), merit=hist[k].merit,
                  best_merit=hist[k].best_merit, amplitude_mse=hist[k].amplitude_mse,
                  target_error_rms=hist[k].target_error_rms,
                  phase_update_rms=hist[k].phase_update_rms) for k in range(int(r.iterations))]
        sols.append(GsSolution(phase, r.merit, int(r.best_iteration), r.amplitude_mse,
                               bool(r.converged), int(r.iterations), h, o["best_int"], o["terr"],
                               o["perr"], o["illum"], o["last"]))
    return sols
