"""optics-inverse hot loops on the GPU (mirror of crates/optics-inverse/src).

* ``Design`` — carrier.rs:49-123: elements plus (element | gap, z_after,
  medium) steps.
* ``Renderer.render`` — observe.rs:195-314 (intensity channel and the
  source-position / band central differences): every (band, scene) frame is
  one frame of ``osgpu_render_batch_device``; the observation stays on the
  device.
* ``push_back`` / ``grid_gradient`` — adjoint.rs:140-340 through
  ``osgpu_push_back_batch_device``: the forward planes recorded by the render
  (a tape) are reused, the detector seed is fused into the first FFT pass of
  the first adjoint propagation and each element plane into the last pass of
  the propagation before it.
* ``MseToTarget``, ``EncircledEnergyMerit`` (merit.rs:112-245) and the
  spot-window efficiency merit of the inverse-design workload, evaluated on
  the device with FP64-compensated sums.
* ``Adam`` — the update of fd.rs:186-257 on device parameters.

Fields and observations are torch tensors on ``cuda``; torch only provides
device memory and streams.  Arrays are real float64 for ``precision="f64"``
(complex128 fields) and float32 for ``precision="f32"`` (complex64 fields).
"""

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Callable, List

from . import _ffi
from .element import Element, ClearAperture, EL_PHASE, _desc
from .propagation.asm import AsmConfig

INTENSITY, DX, DY, DLAMBDA = "intensity", "dx", "dy", "dlambda"


def _torch():
    import torch
    return torch


def _dtypes(precision):
    torch = _torch()
    if precision == "f64":
        return _ffi.C128, torch.complex128, torch.float64, _ffi.F64
    if precision == "f32":
        return _ffi.C64, torch.complex64, torch.float32, _ffi.F32
    raise ValueError(f"precision must be 'f64' or 'f32', got {precision!r}")


class DevicePhaseMask(Element):
    """``PhaseMask::sampled`` (element.rs:1321-1368) whose lattice is a device
    tensor (float64, or float32 for the f32 engine) used in place: the
    carrier's parameter vector becomes the DOE without a host round trip.
    The caller owns the finiteness of the lattice."""

    def __init__(self, lattice, dims, pitch, aperture=ClearAperture.field(), center=(0.0, 0.0)):
        torch = _torch()
        nx, ny = dims
        if lattice.numel() != nx * ny or not lattice.is_cuda:
            raise _ffi.OsgpuError(26)
        if lattice.dtype not in (torch.float64, torch.float32):
            raise ValueError("lattice must be float64 or float32")
        self.lattice = lattice.contiguous()
        self.dims = dims
        self.pitch = pitch
        self.aperture = aperture
        self.center = center

    def descriptor(self, band):
        torch = _torch()
        ap = self.aperture
        nx, ny = self.dims
        d = _desc(EL_PHASE, ap.kind, ap.a, ap.b, 0.0, self.center, lnx=nx, lny=ny,
                  ldx=self.pitch[0], ldy=self.pitch[1])
        d.lattice = C.cast(C.c_void_p(self.lattice.data_ptr()), _ffi.c_double_p)
        d.lattice_on_device = 1 if self.lattice.dtype == torch.float64 else 2
        return d, self.lattice


class Design:
    """carrier.rs:49-123."""

    def __init__(self):
        self.elements = []
        self.steps = []  # (element index | None, z_after, medium)

    def push(self, element, z_after, medium=1.0):
        self.elements.append(element)
        self.steps.append((len(self.elements) - 1, z_after, medium))
        return self

    def gap(self, z_after, medium=1.0):
        self.steps.append((None, z_after, medium))
        return self

    def __len__(self):
        return len(self.steps)


class _Lam:
    def __init__(self, lam):
        self.lam = lam


def _c_steps(design, lam, keep):
    """osgpu_step array of a design at wavelength lam; element order = step order."""
    steps, order = [], []
    for ei, z, medium in design.steps:
        if ei is None:
            steps.append(_ffi.StepC(None, 0, z, medium))
            continue
        d, k = design.elements[ei].descriptor(_Lam(lam))
        arr = (_ffi.ElementC * 1)(d)
        keep.extend([k, arr])
        steps.append(_ffi.StepC(arr, 1, z, medium))
        order.append(ei)
    sarr = (_ffi.StepC * max(len(steps), 1))(*steps)
    keep.append(sarr)
    return sarr, len(steps), order


@dataclass
class Observation:
    """observe.rs:64-147: data[channel, band, scene, row, col] on the device."""
    channels: list
    bands: list
    scenes: list
    dims: tuple
    pitch: tuple
    data: object
    fd_steps: tuple = (0.0, 0.0)

    def frame_len(self):
        return self.dims[0] * self.dims[1]

    # Zero-copy export of the [channel][band][scene][row][col] array (the
    # numpy layout of observe.rs:10-16) through DLPack: any DLPack consumer
    # (numpy for host data, or a GPU array library) views `data` in place.
    def __dlpack__(self, stream=None):
        return self.data.__dlpack__() if stream is None else self.data.__dlpack__(stream=stream)

    def __dlpack_device__(self):
        return self.data.__dlpack_device__()

    def channel_index(self, ch):
        return self.channels.index(ch) if ch in self.channels else None


class Tape:
    """Forward planes kept from a render for the adjoint sweep
    (``osgpu_tape``); ``budget_bytes`` > 0 caps the device memory it holds,
    beyond which push_back recomputes the forward planes."""

    def __init__(self, budget_bytes=0):
        h = C.c_void_p()
        _ffi.check(_ffi.lib().osgpu_tape_create(budget_bytes, C.byref(h)))
        self.handle = h

    def nbytes(self):
        return int(_ffi.lib().osgpu_tape_bytes(self.handle))

    def close(self):
        if self.handle:
            _ffi.lib().osgpu_tape_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Renderer:
    """observe.rs:150-314.  ``carrier(values, lam) -> Design``;
    ``source(x0, y0, lam) -> device complex tensor (ny, nx)`` with pitch
    ``pitch``."""
    carrier: Callable
    source: Callable
    pitch: tuple
    bands: List[float] = field(default_factory=lambda: [500e-9])
    scenes: List[tuple] = field(default_factory=lambda: [(0.0, 0.0)])
    asm_cfg: AsmConfig = AsmConfig()
    precision: str = "f32"
    deriv_x: bool = False
    deriv_y: bool = False
    deriv_lambda: bool = False
    scene_step: float = 1e-6
    lambda_step: float = 1e-9
    stream: object = None
    # d(phase)/d(parameter) per band for band-dependent phase laws (a
    # GridThickness carrier: 2 pi (n(lam) - 1) / lam); push_back then weights
    # each frame's contribution by it, so grid_gradient returns dM/dparameter
    # (adjoint.rs:255-262).  None: the phase is the parameter (weight 1).
    param_slope: Callable = None

    def _stream_ptr(self):
        return _stream_handle(self.stream)

    def _frames(self, values, jobs, outs, keep, seeds=None, grads=None):
        """osgpu_frame array for (lam, x0, y0) jobs."""
        frames = []
        self._designs = []
        for i, (lam, x0, y0) in enumerate(jobs):
            design = self.carrier(values, lam)
            src = self.source(x0, y0, lam)
            keep.append(src)
            ny, nx = src.shape
            sarr, ns, order = _c_steps(design, lam, keep)
            self._designs.append((design, order))
            g = _ffi.Grid(nx, ny, self.pitch[0], self.pitch[1], lam)
            slope = float(self.param_slope(lam)) if (seeds is not None and self.param_slope) else 1.0
            fr = _ffi.FrameC(g, src.data_ptr(), sarr, ns,
                             outs[i].data_ptr() if outs is not None else None,
                             seeds[i].data_ptr() if seeds is not None else None, slope, None)
            if grads is not None:
                ga = (C.c_void_p * max(len(order), 1))(
                    *[grads[ei].data_ptr() if ei in grads else None for ei in order])
                keep.append(ga)
                fr.d_grad = ga
            frames.append(fr)
        arr = (_ffi.FrameC * max(len(frames), 1))(*frames)
        keep.append(arr)
        return arr

    def render_frames(self, values, jobs, tape=None, out=None):
        """Intensity of each (lam, x0, y0) job: tensor (len(jobs), ny, nx)
        (written into `out` when given)."""
        torch = _torch()
        dtype, _, rdt, _ = _dtypes(self.precision)
        if out is None:
            b0 = self.source(jobs[0][1], jobs[0][2], jobs[0][0])
            ny, nx = b0.shape
            out = torch.empty((len(jobs), ny, nx), dtype=rdt, device=b0.device)
        keep = []
        arr = self._frames(values, jobs, out, keep)
        _ffi.check(_ffi.lib().osgpu_render_batch_device(
            arr, len(jobs), self.asm_cfg.c(), dtype, self._stream_ptr(),
            tape.handle if tape is not None else None, None, 0))
        return out

    def render(self, values, tape=None):
        """observe.rs:213-314 (frames band-major, scenes inner)."""
        if not self.bands or not self.scenes:
            raise _ffi.OsgpuError(43)
        # observe.rs:219-230: the finite-difference steps of the requested channels
        if (self.deriv_x or self.deriv_y) and not (math.isfinite(self.scene_step)
                                                   and self.scene_step > 0.0):
            raise _ffi.OsgpuError(43)
        if self.deriv_lambda and not (math.isfinite(self.lambda_step) and self.lambda_step > 0.0):
            raise _ffi.OsgpuError(43)
        chans = [INTENSITY]
        if self.deriv_x:
            chans.append(DX)
        if self.deriv_y:
            chans.append(DY)
        if self.deriv_lambda:
            chans.append(DLAMBDA)
        jobs = [(lam, x0, y0) for lam in self.bands for (x0, y0) in self.scenes]
        B, S = len(self.bands), len(self.scenes)
        torch = _torch()
        _, _, rdt, _ = _dtypes(self.precision)
        b0 = self.source(jobs[0][1], jobs[0][2], jobs[0][0])
        ny, nx = b0.shape
        data = torch.empty((len(chans), B, S, ny, nx), dtype=rdt, device=b0.device)
        self.render_frames(values, jobs, tape, out=data[0].view(B * S, ny, nx))
        h, hl = self.scene_step, self.lambda_step

        def fd(ci, hi_jobs, lo_jobs, step):
            hi = self.render_frames(values, hi_jobs)
            lo = self.render_frames(values, lo_jobs)
            data[ci] = ((hi - lo) / (2.0 * step)).reshape(B, S, ny, nx)

        if self.deriv_x:
            fd(chans.index(DX), [(l, x + h, y) for (l, x, y) in jobs],
               [(l, x - h, y) for (l, x, y) in jobs], h)
        if self.deriv_y:
            fd(chans.index(DY), [(l, x, y + h) for (l, x, y) in jobs],
               [(l, x, y - h) for (l, x, y) in jobs], h)
        if self.deriv_lambda:
            fd(chans.index(DLAMBDA), [(l + hl, x, y) for (l, x, y) in jobs],
               [(l - hl, x, y) for (l, x, y) in jobs], hl)
        return Observation(chans, list(self.bands), list(self.scenes), (nx, ny), self.pitch, data,
                           (h, hl))

    def prepare_push_back(self, values, jobs, seeds, grads):
        """Frame array of a push_back batch (host work only; the seeds and
        gradient buffers may still be in flight)."""
        keep = []
        arr = self._frames(values, jobs, None, keep, seeds=seeds, grads=grads)
        return arr, len(jobs), keep

    def launch_push_back(self, prepared, tape=None):
        dtype, _, _, _ = _dtypes(self.precision)
        arr, n, _keep = prepared
        _ffi.check(_ffi.lib().osgpu_push_back_batch_device(
            arr, n, self.asm_cfg.c(), dtype, self._stream_ptr(),
            tape.handle if tape is not None else None))

    def push_back_frames(self, values, jobs, seeds, grads, tape=None):
        """adjoint.rs:140-246 per job, accumulated into grads {element index: tensor}."""
        self.launch_push_back(self.prepare_push_back(values, jobs, seeds, grads), tape)


def grid_thickness(dims, pitch, index, aperture=ClearAperture.field(), center=(0.0, 0.0),
                   z_after=0.0, rest=None):
    """carrier.rs:247-275 + 338-354: a sampled relief-thickness carrier (m).
    The phase at band lam is 2 pi (n(lam) - 1) h / lam with n = index(lam)
    (a callable, or a constant index).  Returns (carrier, slope): the
    Renderer's ``carrier(values, lam)`` (a PhaseMask design built on the
    device from the thickness tensor, followed by z_after and by whatever
    ``rest(design, lam)`` appends) and its ``param_slope``, the per-band
    factor by which push_back weights each frame so that grid_gradient gives
    dM/dh."""
    n_at = index if callable(index) else (lambda lam, n0=float(index): n0)

    def slope(lam):
        if not (math.isfinite(lam) and lam > 0.0):
            raise _ffi.OsgpuError(102)
        n = float(n_at(lam))
        if not math.isfinite(n):
            raise _ffi.OsgpuError(102)
        return 2.0 * math.pi * (n - 1.0) / lam

    def carrier(values, lam):
        d = Design()
        d.push(DevicePhaseMask((values * slope(lam)).contiguous(), dims, pitch, aperture, center),
               z_after)
        if rest is not None:
            rest(d, lam)
        return d

    return carrier, slope


def push_back(renderer, values, lam, x0, y0, dmdi):
    """adjoint.rs:140-246 for one frame: {element index: dM/dphi tensor}."""
    torch = _torch()
    src = renderer.source(x0, y0, lam)
    design = renderer.carrier(values, lam)
    _, _, rdt, _ = _dtypes(renderer.precision)
    grads = {}
    for ei, _z, _m in design.steps:
        if ei is not None and ei not in grads:
            grads[ei] = torch.zeros(src.shape, dtype=rdt, device=src.device)
    renderer.push_back_frames(values, [(lam, x0, y0)], [dmdi.to(rdt).contiguous()], grads)
    return dict(sorted(grads.items()))


def grid_gradient(renderer, values, merit, tape=None):
    """adjoint.rs:268-340: one render (recording the tape), the merit's
    obs_gradient seed, then one push_back per frame, summed per element.
    Returns ({element index: dM/dphi}, merit value, observation)."""
    torch = _torch()
    own = tape is None
    if own:
        tape = Tape()
    try:
        obs = renderer.render(values, tape)
        # everything the adjoint sweep needs is prepared while the render runs;
        # the merit is the one host synchronisation of the step
        seed = torch.zeros_like(obs.data)
        jobs = [(lam, x0, y0) for lam in renderer.bands for (x0, y0) in renderer.scenes]
        B, S = len(renderer.bands), len(renderer.scenes)
        seeds = [seed[0, b, s] for b in range(B) for s in range(S)]
        design = renderer.carrier(values, renderer.bands[0])
        grads = {}
        for ei, _z, _m in design.steps:
            if ei is not None and ei not in grads:
                grads[ei] = torch.zeros(obs.data.shape[-2:], dtype=obs.data.dtype,
                                        device=obs.data.device)
        prepared = renderer.prepare_push_back(values, jobs, seeds, grads)
        value, ok = merit_value_and_seed(merit, obs, seed)
        if not ok:
            raise _ffi.OsgpuError(44)
        if len(obs.channels) > 1 and bool(torch.any(seed[1:] != 0)):
            raise _ffi.OsgpuError(44)
        if not bool(torch.any(seed[0] != 0)):
            return {}, value, obs
        # the tape holds the intensity frames' planes (the finite-difference
        # renders of the other channels record nothing)
        renderer.launch_push_back(prepared, tape)
        return dict(sorted(grads.items())), value, obs
    finally:
        if own:
            tape.close()


def merit_value_and_seed(merit, obs, seed):
    """(M, ok): the merit value, with dM/dI written into `seed` (shape of
    obs.data); ok is False when the merit has no obs_gradient.  The device
    merits produce both in one call."""
    if hasattr(merit, "value_and_seed"):
        return merit.value_and_seed(obs, seed)
    value = merit.evaluate(obs)
    g = merit.obs_gradient(obs)
    if g is None:
        return value, False
    seed.copy_(g)
    return value, True


def _real_code(t):
    torch = _torch()
    return _ffi.F64 if t.dtype == torch.float64 else _ffi.F32


def _stream_handle(stream=None):
    """cudaStream_t of a torch stream (default: the current one).  Torch's
    default stream is the legacy default stream, whose handle reads as 0;
    it is passed as cudaStreamLegacy (1) so that the library's kernels are
    ordered with torch's work instead of running on the library stream."""
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream or 1


def _sptr():
    return _stream_handle()


class MseToTarget:
    """merit.rs:112-164 (Selector: band/scene None sums over all)."""

    def __init__(self, target, band=None, scene=None):
        self.target = target  # device float64 (ny, nx)
        self.band, self.scene = band, scene

    def _call(self, obs, seed):
        v = C.c_double()
        B, S = len(obs.bands), len(obs.scenes)
        _ffi.check(_ffi.lib().osgpu_merit_mse_device(
            obs.data[0].data_ptr(), _real_code(obs.data), B, S, obs.frame_len(),
            self.target.data_ptr(), -1 if self.band is None else self.band,
            -1 if self.scene is None else self.scene,
            seed.data_ptr() if seed is not None else None, _sptr(), C.byref(v)))
        return v.value

    def evaluate(self, obs):
        return self._call(obs, None)

    def obs_gradient(self, obs):
        g = _torch().zeros_like(obs.data)
        self._call(obs, g[0])
        return g

    def value_and_seed(self, obs, seed):
        return self._call(obs, seed[0]), True


class EncircledEnergyMerit:
    """merit.rs:167-245."""

    def __init__(self, radius, band=None, scene=None):
        self.radius = radius
        self.band, self.scene = band, scene

    def _call(self, obs, seed):
        v = C.c_double()
        B, S = len(obs.bands), len(obs.scenes)
        nx, ny = obs.dims
        code = _ffi.lib().osgpu_merit_encircled_energy_device(
            obs.data[0].data_ptr(), _real_code(obs.data), B, S, nx, ny, obs.pitch[0],
            obs.pitch[1], self.radius, -1 if self.band is None else self.band,
            -1 if self.scene is None else self.scene,
            seed.data_ptr() if seed is not None else None, _sptr(), C.byref(v))
        return code, v.value

    def evaluate(self, obs):
        code, v = self._call(obs, None)
        _ffi.check(code)
        return v

    def obs_gradient(self, obs):
        g = _torch().zeros_like(obs.data)
        code, _ = self._call(obs, g[0])
        if code == 44:
            return None
        _ffi.check(code)
        return g

    def value_and_seed(self, obs, seed):
        code, v = self._call(obs, seed[0])
        if code == 44:
            return v, False
        _ffi.check(code)
        return v, True


def _sel(v):
    return -1 if v is None else v


class SpotRmsMerit:
    """merit.rs:248-321: the spot RMS radius sqrt(sum I rho^2 / sum I) of the
    selected frame, with its analytic obs gradient."""

    def __init__(self, band=None, scene=None):
        self.band, self.scene = band, scene

    def _call(self, obs, seed):
        v = C.c_double()
        B, S = len(obs.bands), len(obs.scenes)
        nx, ny = obs.dims
        code = _ffi.lib().osgpu_merit_spot_rms_device(
            obs.data[0].data_ptr(), _real_code(obs.data), B, S, nx, ny, obs.pitch[0],
            obs.pitch[1], _sel(self.band), _sel(self.scene),
            seed.data_ptr() if seed is not None else None, _sptr(), C.byref(v))
        return code, v.value

    def evaluate(self, obs):
        code, v = self._call(obs, None)
        _ffi.check(code)
        return v

    def obs_gradient(self, obs):
        g = _torch().zeros_like(obs.data)
        code, _ = self._call(obs, g[0])
        if code == 44:
            return None
        _ffi.check(code)
        return g

    def value_and_seed(self, obs, seed):
        code, v = self._call(obs, seed[0])
        if code == 44:
            return v, False
        _ffi.check(code)
        return v, True


class StrehlMerit:
    """merit.rs:323-352: the negative power-equalised peak ratio of the
    selected frame against a reference frame (device, the frame's grid).  No
    obs gradient: grid_gradient rejects it, as the reference does."""

    def __init__(self, reference, band=None, scene=None):
        torch = _torch()
        self.reference = torch.as_tensor(reference, dtype=torch.float64).contiguous()
        self.band, self.scene = band, scene

    def evaluate(self, obs):
        if self.reference.numel() != obs.frame_len():
            raise _ffi.OsgpuError(43)  # the frame and the reference differ in length
        ref = self.reference.to(obs.data.device)
        v = C.c_double()
        nx, ny = obs.dims
        _ffi.check(_ffi.lib().osgpu_merit_strehl_device(
            obs.data[0].data_ptr(), _real_code(obs.data), len(obs.bands), len(obs.scenes), nx,
            ny, ref.data_ptr(), _sel(self.band), _sel(self.scene), _sptr(), C.byref(v)))
        return v.value

    def obs_gradient(self, obs):
        return None


class MtfMerit:
    """merit.rs:354-400: the negative MTF of the selected frame at one DFT bin
    along x (freq in cycles/m, freq nx dx an integer below Nyquist).  No obs
    gradient."""

    def __init__(self, freq, band=None, scene=None):
        self.freq = freq
        self.band, self.scene = band, scene

    def evaluate(self, obs):
        v = C.c_double()
        nx, ny = obs.dims
        _ffi.check(_ffi.lib().osgpu_merit_mtf_device(
            obs.data[0].data_ptr(), _real_code(obs.data), len(obs.bands), len(obs.scenes), nx,
            ny, obs.pitch[0], self.freq, _sel(self.band), _sel(self.scene), _sptr(),
            C.byref(v)))
        return v.value

    def obs_gradient(self, obs):
        return None


class SpotArrayEfficiency:
    """Negative summed efficiency into a set of spot windows (the merit of the
    spot-array inverse design; no reference counterpart):
    M = -sum_frames sum_{k in windows} I[k] / p_in[frame]."""

    def __init__(self, windows, p_in):
        torch = _torch()
        self.windows = windows.to(torch.uint8).contiguous()  # device (ny, nx)
        self.p_in = [float(p) for p in p_in]  # per band

    def _call(self, obs, seed):
        B, S = len(obs.bands), len(obs.scenes)
        pin = (C.c_double * (B * S))(*[self.p_in[b] for b in range(B) for _ in range(S)])
        v = C.c_double()
        _ffi.check(_ffi.lib().osgpu_merit_spot_efficiency_device(
            obs.data[0].data_ptr(), _real_code(obs.data), B * S, obs.frame_len(),
            self.windows.data_ptr(), pin, seed.data_ptr() if seed is not None else None, _sptr(),
            C.byref(v)))
        return v.value

    def evaluate(self, obs):
        return self._call(obs, None)

    def obs_gradient(self, obs):
        g = _torch().zeros_like(obs.data)
        self._call(obs, g[0])
        return g

    def value_and_seed(self, obs, seed):
        return self._call(obs, seed[0]), True


def shard_bands(n_bands, rank, world):
    """Band indices of one rank when the bands of a gradient are split over
    `world` ranks: rank r takes bands r, r + world, ... (independent units;
    every band lands on exactly one rank)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    return list(range(rank, n_bands, world))


def grid_gradient_sharded(partial, n_bands, group=None):
    """grid_gradient (adjoint.rs:268-340) with its bands split over the ranks
    of a torch.distributed process group: the merit and every frame's
    contribution are sums over bands, so each rank computes the partial
    gradient of its own bands (``partial(band_indices) -> ({element: tensor},
    merit value)``, e.g. ``grid_gradient`` of a renderer and merit built for
    those bands) and one sum all-reduce per element grid (and one for the
    merit) gives every rank the gradient of all bands.  The exchange is the
    only collective of the inverse-design step; it runs on the backend of the
    group (NCCL on GPUs, gloo on CPUs)."""
    import torch
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    grads, value = partial(shard_bands(n_bands, rank, world))
    for key in sorted(grads):
        dist.all_reduce(grads[key], op=dist.ReduceOp.SUM, group=group)
    dev = next(iter(grads.values())).device if grads else "cpu"
    v = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(v, op=dist.ReduceOp.SUM, group=group)
    return grads, float(v.item())


def gaussian_spot_array(shape, count, pitch, sigma):
    """Target weights of a centred count x count array of Gaussian spots (peak 1,
    standard deviation ``sigma`` samples, ``pitch`` samples apart) on a
    (ny, nx) detector grid, as a float64 numpy array (host-side target
    preparation)."""
    import numpy as np
    ny, nx = shape
    w = np.zeros((ny, nx))
    half = int(math.ceil(5.0 * sigma))
    for i in range(count):
        for j in range(count):
            cy = ny // 2 + pitch * (i - (count - 1) / 2.0)
            cx = nx // 2 + pitch * (j - (count - 1) / 2.0)
            y0, y1 = max(0, math.floor(cy) - half), min(ny, math.ceil(cy) + half + 1)
            x0, x1 = max(0, math.floor(cx) - half), min(nx, math.ceil(cx) + half + 1)
            yy = np.arange(y0, y1, dtype=np.float64)[:, None] - cy
            xx = np.arange(x0, x1, dtype=np.float64)[None, :] - cx
            w[y0:y1, x0:x1] += np.exp(-(yy * yy + xx * xx) / (2.0 * sigma * sigma))
    return w


class WeightedSpotEfficiency:
    """Negative summed efficiency into a weighted spot-array target (the merit
    of the spot-array inverse design with Gaussian spots; no reference
    counterpart): M = -sum_frames sum_k w[k] I[k] / p_in[frame], with ``weights``
    a device (ny, nx) real array (e.g. ``gaussian_spot_array``), converted to
    the observation's real dtype, and ``p_in`` the input power of each band."""

    def __init__(self, weights, p_in):
        self.weights = weights.contiguous()
        self.p_in = [float(p) for p in p_in]  # per band
        self._w = {}

    def _weights(self, obs):
        dt = obs.data.dtype
        if dt not in self._w:
            self._w[dt] = self.weights.to(dt).contiguous()
        return self._w[dt]

    def _call(self, obs, seed):
        B, S = len(obs.bands), len(obs.scenes)
        pin = (C.c_double * (B * S))(*[self.p_in[b] for b in range(B) for _ in range(S)])
        v = C.c_double()
        _ffi.check(_ffi.lib().osgpu_merit_weighted_efficiency_device(
            obs.data[0].data_ptr(), _real_code(obs.data), B * S, obs.frame_len(),
            self._weights(obs).data_ptr(), pin, seed.data_ptr() if seed is not None else None,
            _sptr(), C.byref(v)))
        return v.value

    def evaluate(self, obs):
        return self._call(obs, None)

    def obs_gradient(self, obs):
        g = _torch().zeros_like(obs.data)
        self._call(obs, g[0])
        return g

    def value_and_seed(self, obs, seed):
        return self._call(obs, seed[0]), True


def field_power(u):
    """sum |u|^2 of a device field in FP64."""
    torch = _torch()
    v = C.c_double()
    dt = _ffi.C128 if u.dtype == torch.complex128 else _ffi.C64
    _ffi.check(_ffi.lib().osgpu_field_power_device(u.data_ptr(), dt, u.numel(), _sptr(),
                                                   C.byref(v)))
    return v.value


@dataclass
class Param:
    """params.rs:30-105: one bounded design slot with an optional
    finite-difference step."""
    name: str
    lo: float
    hi: float
    value: float = 0.0
    fd_step: float = None

    def step(self):
        """params.rs:62-71: the explicit step, else 1e-4 of the span (1e-9 for a
        point bound)."""
        if self.fd_step is not None:
            return self.fd_step
        rel = (self.hi - self.lo) * 1.0e-4
        return rel if rel > 0.0 else 1.0e-9

    def check(self, v):
        """params.rs:79-104 on the value v."""
        if not (math.isfinite(self.lo) and math.isfinite(self.hi)) or not math.isfinite(v):
            raise _ffi.OsgpuError(41)  # NotFinite
        if v < self.lo or v > self.hi:
            raise _ffi.OsgpuError(42)  # OutOfBounds


def fd_gradient(params, objective, x):
    """fd.rs:139-179: central-difference gradient of ``objective(values) ->
    float`` (typically a render plus a merit) at ``x``.  Probes are clamped
    into the bounds, so a slot at a bound gets the one-sided slope over the
    effective separation; zero-width slots are skipped (gradient 0).  Returns
    (gradient list, objective evaluations)."""
    if len(x) != len(params):
        raise _ffi.OsgpuError(40)  # WrongDimension
    for p, v in zip(params, x):
        p.check(v)
    g = [0.0] * len(params)
    evaluations = 0
    for i, p in enumerate(params):
        if p.lo == p.hi:
            continue
        s = p.step()
        up, dn = list(x), list(x)
        up[i] = min(max(x[i] + s, p.lo), p.hi)
        dn[i] = min(max(x[i] - s, p.lo), p.hi)
        fu = objective(up)
        fd = objective(dn)
        evaluations += 2
        d = up[i] - dn[i]
        if not d > 0.0:
            raise _ffi.OsgpuError(43)  # the step collapses to zero separation
        gi = (fu - fd) / d
        if not math.isfinite(gi):
            raise _ffi.OsgpuError(43)
        g[i] = gi
    return g, evaluations


@dataclass
class AdamConfig:
    """fd.rs:63-91 (defaults as the reference)."""
    lr_frac: float = 0.02
    beta1: float = 0.9
    beta2: float = 0.999
    eps: float = 1.0e-8
    clip_norm: object = 1.0  # None: no clipping

    def c(self):
        clip = self.clip_norm is not None
        return _ffi.AdamConfigC(self.lr_frac, self.beta1, self.beta2, self.eps,
                                float(self.clip_norm) if clip else 0.0, 1 if clip else 0)


class Adam:
    """Adam state over a device parameter vector with bounds [lo, hi]
    (fd.rs:186-257 update; x32 optionally mirrors x as float32)."""

    def __init__(self, x, lo, hi, cfg=AdamConfig(), x32=None):
        torch = _torch()
        self.x, self.x32, self.lo, self.hi, self.cfg = x, x32, lo, hi, cfg
        self.m = torch.zeros_like(x, dtype=torch.float64)
        self.v = torch.zeros_like(x, dtype=torch.float64)
        self.t = 0

    def step(self, g):
        self.t += 1
        _ffi.check(_ffi.lib().osgpu_adam_step_device(
            self.x.data_ptr(), self.x32.data_ptr() if self.x32 is not None else None,
            g.data_ptr(), _real_code(g), self.m.data_ptr(), self.v.data_ptr(), self.x.numel(),
            self.cfg.c(), self.t, self.lo, self.hi, _sptr()))
