"""Benchmark of the propagation hot path on one GB300 (or N replicas).

Workload (the 2048^2 batched BandField beamline): 32 wavelengths uniform
450-650 nm, each a 2048 x 2048 complex64 field (dx = 3 um, unit plane wave)
through [16-level random DOE phase (seeded), square aperture 5 mm, thin lens
f = 100 mm, ASM z = 100 mm] with the default AsmConfig (strict densification
gives a 8192 x 8192 padded grid for every band).  One step = the whole
32-band batch, device resident, through osgpu_beamline_trace_batch_device.
Metric: propagations (band-planes) per second.

Also reported: the ragged 64-item ASM batch replayed from one captured CUDA
graph (sides 256-2048, z 1 mm - 1 m), Gerchberg-Saxton target-iterations/s of the 16 x 2048^2
spot-array batch (GS_WORKLOAD below, with the spot efficiency / uniformity
of target 0 on the f32 and FP64 engines), adjoint gradients/s of the 2048^2
inverse-design workload
(ADJ_WORKLOAD below; f32 batched, with an FP64-plain sample and the f32
gradient's relative L2 error against the FP64 engine), the same batch on
the plain FP64 path, the same batch with kernel-spectrum plans (opt-in:
first call with the table builds, then the steady rate), end-to-end throughput
through the reference-facing host-buffer C ABI (osgpu_beamline_trace with
pinned complex128 buffers, copies inside the timed region), the roofline of
the dominant kernel (CUDA events recorded by the library on the launching
stream), SM clocks sampled during the timed region, and a bounded CPU
baseline (the f64 oracle restatement, one band, one thread).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun each rank runs its own 32-band batch (weak scaling, no
collective on the data path); rank 0 prints one JSON line.
"""

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 2048
DX = 3e-6
NBANDS = 32
LAMS = np.linspace(450e-9, 650e-9, NBANDS)
Z = 0.1
F_LENS = 0.1
HALF_AP = 2.5e-3
LEVELS = 16
SEED = 1234
METRIC = "2048^2 ASM propagations/s (batched BandField beamline, FP32)"
WORKLOAD = ("32 bands 450-650 nm x 2048^2, dx 3 um, [16-level DOE, square aperture 5 mm, "
            "thin lens f 100 mm, ASM z 100 mm], padded 8192^2")


def workload_config(world):
    """The `config` object of both arms' lines (the same workload)."""
    return {"workload": WORKLOAD, "bands_per_gpu": NBANDS, "grid": N, "padded": 8192,
            "l2": "inputs larger than L2 (1 GiB field batch + 134 MB spectrum per band)",
            "parallelism": f"replicas x{world}"}


def set_bands(n):
    global NBANDS, LAMS
    NBANDS = n
    LAMS = np.linspace(450e-9, 650e-9, 32)[:n] if n <= 32 else np.linspace(450e-9, 650e-9, n)


def doe_lattice():
    rng = np.random.default_rng(SEED)
    return np.floor(rng.uniform(0, LEVELS, (N, N))) * (2 * math.pi / LEVELS)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.first = threading.Event()

    def start(self):
        """Starts sampling and returns once nvidia-smi delivers its first
        sample (at most 5 s), so its start-up does not fall into the timed
        region that follows."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self.first.wait(timeout=5.0)
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())
            self.first.set()

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[3:7]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(ms, world):
    """Slowest rank's time (the job finishes with it); the all-reduce runs on
    the device of the process group's backend (NCCL: cuda, gloo: cpu)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(ms)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, ms_per_step):
    """Whole-job throughput: the units all ranks processed per second."""
    return units_per_rank * world / (ms_per_step / 1e3)


def make_items(og, ffi, d_in, d_out, lattice_handle, keep):
    """One osgpu_trace_item per band: DOE -> aperture -> lens -> ASM z."""
    items = (ffi.TraceItemC * NBANDS)()
    for b in range(NBANDS):
        doe = ffi.ElementC(4, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                           C.cast(C.c_void_p(lattice_handle), ffi.c_double_p), N, N, DX, DX, 1)
        ap = ffi.ElementC(2, 0, HALF_AP, HALF_AP, 0, 0, 0, 0, 0, 0, None, 0, 0, 0, 0, 0)
        lens = ffi.ElementC(3, 0, 0, 0, 0, 0, 0, F_LENS, 0, 0, None, 0, 0, 0, 0, 0)
        e1 = (ffi.ElementC * 1)(doe)
        e2 = (ffi.ElementC * 1)(ap)
        e3 = (ffi.ElementC * 1)(lens)
        steps = (ffi.StepC * 3)(ffi.StepC(e1, 1, 0.0, 1.0), ffi.StepC(e2, 1, 0.0, 1.0),
                                ffi.StepC(e3, 1, Z, 1.0))
        keep.extend([e1, e2, e3, steps])
        items[b] = ffi.TraceItemC(d_in[b], d_out[b], ffi.Grid(N, N, DX, DX, float(LAMS[b])),
                                  steps, 3)
    return items


def run_batch(og, ffi, items, dtype, stream):
    cfg = ffi.AsmConfigC(2.0, 1, 1, 8.0, 1.0)
    code = og.lib().osgpu_beamline_trace_batch_device(items, NBANDS, cfg, dtype, stream, None, 0)
    ffi.check(code)


def cpu_baseline_band(band=0):
    """Bounded CPU sample: one band of the batch through the f64 oracle, one
    thread."""
    from oracle import field as ofield, element as oel, beamline as obl, asm as oasm
    lat = doe_lattice()
    t0 = time.perf_counter()
    lam = float(np.linspace(450e-9, 650e-9, 32)[band % 32])
    b = ofield.plane_wave(0.0, 0.0, 1.0, N, N, DX, DX, lam)
    bl = obl.Beamline()
    bl.push(oel.PhaseMask.sampled(lat, (N, N), (DX, DX)), 0.0)
    bl.push(oel.RectangularAperture((HALF_AP, HALF_AP)), 0.0)
    bl.push(oel.ThinLens.fixed(F_LENS), Z)
    out = bl.trace(b, obl.asm_engine(oasm.AsmConfig()))
    dt = time.perf_counter() - t0
    return out.samples, dt


# Adjoint inverse-design workload: 2048^2 phase parameters (uniform [0, 2pi),
# seeded), design [DOE, ASM 20 mm] [circular aperture 6 mm, ASM 80 mm], 8
# wavelengths 500-600 nm, unit plane wave, merit = -summed efficiency into a
# 9 x 9 Gaussian spot-array target (spots of peak 1, sigma 2 samples, pitch 96
# samples, centred).  One gradient = render of the 8 bands (tape recorded),
# merit + seed, adjoint sweep of the 8 bands, Adam step (lr 0.05 rad).
ADJ_LAMS = np.linspace(500e-9, 600e-9, 8)
ADJ_Z1, ADJ_Z2, ADJ_R = 20e-3, 80e-3, 3e-3
ADJ_SEED = 2025
ADJ_SPOTS, ADJ_PITCH, ADJ_SIGMA = 9, 96, 2.0
ADJ_WORKLOAD = ("2048^2 phase DOE -> ASM 20 mm -> aperture 6 mm -> ASM 80 mm, 8 bands 500-600 nm, "
                "9x9 Gaussian spot-array efficiency merit (sigma 2 samples, pitch 96), "
                "Adam lr 0.05 rad")


def adjoint_phases():
    """The seeded initial phases, uniform [0, 2 pi)."""
    return np.random.default_rng(ADJ_SEED).uniform(0.0, 2 * math.pi, (N, N))


def adjoint_spot_weights():
    """The 9 x 9 Gaussian spot-array target weights (host float64)."""
    from optics_studio_gb300 import inverse as inv
    return inv.gaussian_spot_array((N, N), ADJ_SPOTS, ADJ_PITCH, ADJ_SIGMA)


def adjoint_setup(precision, bands):
    import torch
    from optics_studio_gb300 import inverse as inv, element as el
    from optics_studio_gb300.propagation.asm import AsmConfig
    cdt = torch.complex128 if precision == "f64" else torch.complex64
    phi = torch.from_numpy(adjoint_phases()).cuda()
    phi32 = phi.float() if precision == "f32" else None
    src = torch.ones((N, N), dtype=cdt, device="cuda")

    def carrier(values, lam):
        d = inv.Design()
        d.push(inv.DevicePhaseMask(phi32 if phi32 is not None else values, (N, N), (DX, DX)),
               ADJ_Z1)
        d.push(el.EllipticalAperture.circle(ADJ_R), ADJ_Z2)
        return d

    rend = inv.Renderer(carrier, lambda x0, y0, lam: src, (DX, DX), bands=list(bands),
                        asm_cfg=AsmConfig(), precision=precision)
    w = torch.from_numpy(adjoint_spot_weights()).cuda()
    merit = inv.WeightedSpotEfficiency(w, [float(N * N)] * len(bands))
    opt = inv.Adam(phi, 0.0, 2 * math.pi, inv.AdamConfig(lr_frac=0.05 / (2 * math.pi)), x32=phi32)
    tape = inv.Tape()
    return rend, merit, opt, tape, phi


ADJ_STEPS = 500  # Adam steps of the inverse-design run (plan builds amortised over them)


class nvtx_range:
    """NVTX push/pop range around a timed region (a no-op unless a profiler
    listens), so that `ncu --nvtx --nvtx-include "<name>/"` selects exactly the
    launches of that region."""

    def __init__(self, name):
        self.name = name

    def __enter__(self):
        import torch
        try:
            torch.cuda.nvtx.range_push(self.name)
            self.on = True
        except Exception:
            self.on = False
        return self

    def __exit__(self, *exc):
        if self.on:
            import torch
            torch.cuda.nvtx.range_pop()
        return False


def hbm_peak():
    """Measured HBM copy bandwidth (GB/s) of this GPU pool, else the fallback."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f).get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


KERNEL_SOURCES = ("optics_studio_gb300/csrc/prop_fast.cu", "optics_studio_gb300/csrc/fft_reg.cuh")


def kernel_sources_sha():
    """SHA-256 (first 16 hex digits) of the sources of the f32 passes."""
    import hashlib
    h = hashlib.sha256()
    for rel in KERNEL_SOURCES:
        with open(os.path.join(ROOT, rel), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def traffic_of(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu capture
    (profiles/traffic.json: dram__bytes_read.sum + dram__bytes_write.sum of one
    full-size launch), with where it came from and whether the kernel sources
    changed since that capture (then the figure is stale and not reported)."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None, None
    with open(path) as f:
        t = json.load(f)
    src = {"profile": t.get("profile"), "captured_sources_sha": t.get("sources_sha"),
           "current_sources_sha": kernel_sources_sha()}
    src["stale"] = src["captured_sources_sha"] != src["current_sources_sha"]
    val = t.get("kernels", {}).get(kernel)
    return (None if src["stale"] else val), src


def prop_bytes(n, p, s=8):
    """Algorithmic bytes of one pruned padded propagation of an n x n field on a
    p x p grid (element fused in, crop out): s (2 n^2 + 4 n p)."""
    return s * (2.0 * n * n + 4.0 * n * p)


def adjoint_roofline(ms, plans_on):
    """Algorithmic bytes of one gradient of the inverse-design workload, per
    band: the render's two propagations (20 mm on 4096^2, 80 mm on 8192^2),
    the adjoint's two, and n^2 (2 s + 12) bytes of detector field write/read,
    phase read and gradient read-modify-write; summed over the 8 bands.  With
    kernel-spectrum plans the 80 mm propagations run on 4096^2; the padded
    count is the workload's own (what the reference computes)."""
    peak, src = hbm_peak()
    per_band_padded = 2 * prop_bytes(N, 4096) + 2 * prop_bytes(N, 8192) + N * N * (2 * 8 + 12)
    per_band_run = (4 * prop_bytes(N, 4096) + N * N * (2 * 8 + 12)) if plans_on else per_band_padded
    nb = len(ADJ_LAMS)
    out = {"bound": "hbm", "peak": peak, "unit": "GB/s", "peak_source": src,
           "bytes_per_gradient_padded": per_band_padded * nb,
           "achieved_padded": per_band_padded * nb / (ms / 1e3) / 1e9}
    out["frac_padded"] = out["achieved_padded"] / peak
    if plans_on:
        out["bytes_per_gradient_run"] = per_band_run * nb
        out["achieved_run"] = per_band_run * nb / (ms / 1e3) / 1e9
        out["frac_run"] = out["achieved_run"] / peak
    return out


def adjoint_leg(args, stream):
    """Adjoint gradients/s (f32 batched, kernel-spectrum plans for the 80 mm
    leg), the padded path without plans, and the FP64 plain path on a sample."""
    import torch
    from optics_studio_gb300 import inverse as inv, plans
    rend, merit, opt, tape, phi = adjoint_setup("f32", ADJ_LAMS)

    def step():
        g, val, _ = inv.grid_gradient(rend, phi, merit, tape)
        opt.step(g[0])
        return g, val

    def timed(n):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    use_plans = not args.no_plans
    with torch.cuda.stream(stream):
        plans.clear()
        no_plan = None
        if use_plans:
            # the padded path first (the same steps without plans), then plans on:
            # the first gradient builds the tables
            step()
            no_plan_ms = timed(3)
            no_plan = {"value": 1e3 / no_plan_ms, "unit": "gradients/s",
                       "ms_per_gradient": no_plan_ms, "gradients": 3,
                       "roofline": adjoint_roofline(no_plan_ms, plans_on=False)}
            plans.enable(4 << 30)
            first_ms = timed(1)
        for _ in range(max(1, args.warmup)):
            step()
        torch.cuda.synchronize()
        nsteps = max(3, args.steps // 3)
        import ctypes as C
        import optics_studio_gb300 as og
        from optics_studio_gb300 import _ffi as ffi
        L = og.lib()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        with nvtx_range("adjoint_timed"):
            for _ in range(nsteps):
                g, val = step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / nsteps
        # per-kernel-class device times from a separate profiled pass of 2
        # gradients: every launch bracketed by events and the per-band table
        # builds serialised on the compute stream, so each class times its own
        # kernels (the timed run above overlaps the tables with the passes)
        ffi.check(L.osgpu_profile_begin())
        for _ in range(2):
            step()
        torch.cuda.synchronize()
        stats = (ffi.KernelStatC * 16)()
        nst = C.c_int32()
        ffi.check(L.osgpu_profile_end(stats, 16, C.byref(nst)))
        kst = {stats[i].name.decode(): round(stats[i].total_ms / 2, 4)
               for i in range(nst.value)}
        out = {"value": 1e3 / ms, "unit": "gradients/s", "ms_per_gradient": ms,
               "gradients": nsteps, "merit_last": val, "tape_bytes": tape.nbytes(),
               "workload": ADJ_WORKLOAD, "dtype": "f32",
               "kernel_ms_per_gradient_serialized": kst,
               "kernel_ms_sum_serialized": round(sum(kst.values()), 4),
               "roofline": adjoint_roofline(ms, plans_on=use_plans)}
        if use_plans:
            st = plans.stats()
            build_ms = max(0.0, first_ms - ms)
            out["plans"] = {
                "tables": st["plans"], "bytes": st["bytes"], "builds": st["builds"],
                "build_ms": build_ms,
                "note": "kernel-spectrum plans: the 80 mm propagations (padded 8192^2) run "
                        "as 4096^2 circular convolutions with a kernel spectrum built once "
                        "per band (kernel by the f32 engine, spectrum folded in FP64); the "
                        "20 mm ones (4096^2) are unchanged",
                f"rate_over_{ADJ_STEPS}_steps": ADJ_STEPS / ((ADJ_STEPS * ms + build_ms) / 1e3)}
            out["no_plan"] = no_plan
        tape.close()
        if not args.no_f64:
            # same gradient (first 2 bands) on both engines from the same phases
            rend32, merit32, _, tape32, phi0 = adjoint_setup("f32", ADJ_LAMS[:2])
            g32, _, _ = inv.grid_gradient(rend32, phi0, merit32, tape32)
            rend64, merit64, _, tape64, _ = adjoint_setup("f64", ADJ_LAMS[:2])
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            g64, _, _ = inv.grid_gradient(rend64, phi0, merit64, tape64)
            torch.cuda.synchronize()
            dt64 = (time.perf_counter() - t0) * 4  # 2 of the 8 bands
            a, b = g32[0].double(), g64[0]
            out["f64_plain"] = {"value": 1.0 / dt64, "unit": "gradients/s",
                                "sample": "bands 1-2 of 8 (complex128), scaled to 8 bands"}
            out["rel_l2_f32_vs_f64"] = float(torch.linalg.norm(a - b) / torch.linalg.norm(b))
            out["speedup_vs_f64"] = out["value"] / out["f64_plain"]["value"]
            tape32.close()
            tape64.close()
        plans.disable()
        plans.clear()
    return out


# Ragged batch: 64 independent ASM propagations, side uniform in {256, 512,
# 1024, 2048}, z log-uniform 1 mm - 1 m, Gaussian waist uniform 50-500 um,
# dx 3 um, lam uniform 450-650 nm, default AsmConfig (strict densification),
# complex64, replayed from one captured CUDA graph.
RAGGED_ITEMS, RAGGED_SEED = 64, 4242


def ragged_leg(args, stream):
    import ctypes as C
    import torch
    import optics_studio_gb300 as og
    from optics_studio_gb300 import _ffi as ffi
    L = og.lib()
    rng = np.random.default_rng(RAGGED_SEED)
    arr = (ffi.TraceItemC * RAGGED_ITEMS)()
    keep, samples = [], 0
    cfg = ffi.AsmConfigC(2.0, 1, 1, 8.0, 1.0)
    for i in range(RAGGED_ITEMS):
        n = int(rng.choice([256, 512, 1024, 2048]))
        z = float(np.exp(rng.uniform(np.log(1e-3), np.log(1.0))))
        w0 = float(rng.uniform(50e-6, 500e-6))
        lam = float(rng.uniform(450e-9, 650e-9))
        x = (np.arange(n) - (n - 1) / 2.0) * DX
        u = np.exp(-(x[None, :] ** 2 + x[:, None] ** 2) / (w0 * w0)).astype(np.complex64)
        tin = torch.from_numpy(u).cuda()
        tout = torch.empty_like(tin)
        steps = (ffi.StepC * 1)(ffi.StepC(None, 0, z, 1.0))
        keep += [tin, tout, steps]
        arr[i] = ffi.TraceItemC(tin.data_ptr(), tout.data_ptr(), ffi.Grid(n, n, DX, DX, lam),
                                steps, 1)
        samples += n * n
    sptr = C.c_void_p(stream.cuda_stream)
    g = C.c_void_p()
    ffi.check(L.osgpu_beamline_trace_batch_graph(arr, RAGGED_ITEMS, cfg, ffi.C64, C.byref(g)))
    reps = max(3, args.steps // 3)

    def timed(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    ms_graph = timed(lambda: ffi.check(L.osgpu_graph_launch(g, sptr)))
    ms_direct = timed(lambda: ffi.check(L.osgpu_beamline_trace_batch_device(
        arr, RAGGED_ITEMS, cfg, ffi.C64, sptr, None, 0)))
    ffi.check(L.osgpu_graph_destroy(g))
    ffi.check(L.osgpu_sync_status())
    sides = {}
    for i in range(RAGGED_ITEMS):
        sides[int(arr[i].grid.nx)] = sides.get(int(arr[i].grid.nx), 0) + 1
    # padded size of every item after the strict densification ladder (the
    # reports of one batch call), for the algorithmic bytes
    reps = (ffi.AsmReportC * RAGGED_ITEMS)()
    ffi.check(L.osgpu_beamline_trace_batch_device(arr, RAGGED_ITEMS, cfg, ffi.C64, sptr, reps, 1))
    torch.cuda.synchronize()
    padded = [int(reps[i].nx_pad) for i in range(RAGGED_ITEMS)]
    nbytes = sum(prop_bytes(int(arr[i].grid.nx), padded[i]) for i in range(RAGGED_ITEMS))
    peak, src = hbm_peak()
    achieved = nbytes / (ms_graph / 1e3) / 1e9
    return {"value": RAGGED_ITEMS / (ms_graph / 1e3), "unit": "propagations/s",
            "ms_per_batch_graph": ms_graph, "ms_per_batch_direct": ms_direct,
            "roofline": {"bound": "hbm", "bytes_per_batch": nbytes, "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": src,
                         "note": "s (2 n^2 + 4 n P) per item at its strict padded size P"},
            "items": RAGGED_ITEMS, "sides": sides, "padded_sides": sorted(set(padded)),
            "workload": "64 ASM items, side {256..2048}, z log-uniform 1 mm-1 m, Gaussian waist "
                        "50-500 um, dx 3 um, 450-650 nm, complex64, one captured CUDA graph"}


# Single-plane engine sweep at 1024^2 (dx 4 um, 532 nm): unit plane wave x
# 8-level quantised random DOE phase (levels k 2 pi / 8, seeded) x thin lens
# f 50 mm, then Fresnel transfer function 50 mm and Fresnel convolution
# 200 mm (strict; both pass at padding 2, P = 2048), Fraunhofer 50 mm and
# Rayleigh-Sommerfeld 5 mm (strict off: the reference's strict guards reject
# both; the reports are recorded).  Each engine through its reference-facing
# host-buffer entry point (complex128 in and out) on the plain FP64 and the
# f32 engines.
C2_N, C2_DX, C2_LAM, C2_F, C2_SEED = 1024, 4e-6, 532e-9, 50e-3, 808


def c2_input():
    """Host complex128 input of the sweep: the elements applied on the device
    (FP64 engine), so both precisions propagate the same samples."""
    from optics_studio_gb300 import element as gel
    from optics_studio_gb300.field import BandField
    lat = np.floor(np.random.default_rng(C2_SEED).uniform(0, 8, (C2_N, C2_N))) * (2 * math.pi / 8)
    b = BandField(np.ones((C2_N, C2_N), complex), C2_DX, C2_DX, C2_LAM)
    return gel.apply_elements(b, [gel.PhaseMask.sampled(lat, (C2_N, C2_N), (C2_DX, C2_DX)),
                                  gel.ThinLens.fixed(C2_F)], "f64"), lat


def c2_engines():
    from optics_studio_gb300.propagation import fresnel, fraunhofer, rayleigh_sommerfeld as rs
    n, P = C2_N, 2 * C2_N
    # algorithmic bytes per call (s = bytes per complex): pruned padded
    # propagation s (2 n^2 + 4 n P), plus the kernel spectrum P^2 for the
    # convolution engines; Fraunhofer is unpadded, s 4 n^2 (two passes)
    return {
        "fresnel_tf": (lambda b, p: fresnel.propagate(b, 50e-3, fresnel.FresnelConfig(), p),
                       lambda s: s * (2 * n * n + 4 * n * P)),
        "fresnel_conv": (lambda b, p: fresnel.propagate_convolution(
            b, 200e-3, fresnel.FresnelConfig(), p), lambda s: s * (2 * n * n + 4 * n * P + P * P)),
        "fraunhofer": (lambda b, p: fraunhofer.propagate(
            b, 50e-3, fraunhofer.FraunhoferConfig(strict=False), p), lambda s: s * 4 * n * n),
        "rayleigh_sommerfeld": (lambda b, p: rs.propagate(
            b, 5e-3, rs.RayleighSommerfeldConfig(strict=False), p),
            lambda s: s * (2 * n * n + 4 * n * P + P * P)),
    }


def c2_oracle(samples):
    from oracle import field as ofield, fresnel as ofr, fraunhofer as ofh, rs as ors
    ob = ofield.BandField(samples, C2_DX, C2_DX, C2_LAM)
    return {"fresnel_tf": ofr.propagate(ob, 50e-3, ofr.FresnelConfig()).samples,
            "fresnel_conv": ofr.propagate_convolution(ob, 200e-3, ofr.FresnelConfig()).samples,
            "fraunhofer": ofh.propagate(ob, 50e-3, ofh.FraunhoferConfig(strict=False)).samples,
            "rayleigh_sommerfeld": ors.propagate(
                ob, 5e-3, ors.RayleighSommerfeldConfig(strict=False)).samples}


def c2_leg(args):
    import ctypes as C
    import optics_studio_gb300 as og
    from optics_studio_gb300 import _ffi as ffi
    from optics_studio_gb300.propagation import fraunhofer, rayleigh_sommerfeld as rs
    L = og.lib()
    band, _ = c2_input()
    peak, src = hbm_peak()
    reps = max(5, args.steps)
    out = {"workload": "1024^2, dx 4 um, 532 nm, plane wave x 8-level DOE x lens f 50 mm; "
                       "Fresnel TF 50 mm, Fresnel conv 200 mm, Fraunhofer 50 mm (strict off), "
                       "RS 5 mm (strict off)",
           "api": "host-buffer entry points (complex128 in/out, copies in the timed call)",
           "engines": {}}
    results = {}
    for name, (fn, nbytes) in c2_engines().items():
        row = {}
        for prec in ("f64", "f32"):
            fn(band, prec)  # warm-up: twiddle tables, kernel attributes
            t0 = time.perf_counter()
            with nvtx_range(f"c2_{prec}"):
                for _ in range(reps):
                    r = fn(band, prec)
            dt = (time.perf_counter() - t0) / reps
            results[(name, prec)] = r.samples
            # device time of the kernels of one call (events on the launching stream)
            ffi.check(L.osgpu_profile_begin())
            fn(band, prec)
            stats = (ffi.KernelStatC * 16)()
            nst = C.c_int32()
            ffi.check(L.osgpu_profile_end(stats, 16, C.byref(nst)))
            kms = sum(stats[i].total_ms for i in range(nst.value))
            b = nbytes(16 if prec == "f64" else 8)
            row[prec] = {"value": 1.0 / dt, "unit": "propagations/s", "ms_per_call": dt * 1e3,
                         "kernel_ms": kms,
                         "roofline": {"bound": "hbm", "bytes": b,
                                      "achieved": b / (kms / 1e3) / 1e9 if kms > 0 else None,
                                      "peak": peak, "unit": "GB/s", "peak_source": src,
                                      "frac": b / (kms / 1e3) / 1e9 / peak if kms > 0 else None}}
        row["f32_speedup_vs_f64"] = row["f32"]["value"] / row["f64"]["value"]
        out["engines"][name] = row
    # the strict guards the reference would apply (reports of the rejected runs)
    try:
        rs.propagate(band, 5e-3, rs.RayleighSommerfeldConfig(strict=True))
        out["rs_strict"] = "passed"
    except og.OsgpuError as e:
        out["rs_strict"] = {"error": e.variant,
                            "max_kernel_step_x": e.report.max_kernel_step_x if e.report else None}
    fr = fraunhofer.regime_report(band, 50e-3, fraunhofer.FraunhoferConfig())
    out["fraunhofer_regime"] = {"n_f_x": fr.n_f_x, "max_n_f": fr.max_n_f,
                                "regime_ok": bool(fr.regime_ok)}
    if not args.no_cpu_baseline:
        ref = c2_oracle(band.samples)
        for name in out["engines"]:
            for prec in ("f64", "f32"):
                got = results[(name, prec)]
                out["engines"][name][prec]["rel_l2_vs_oracle"] = float(
                    np.linalg.norm(got - ref[name]) / np.linalg.norm(ref[name]))
    return out


# Gerchberg-Saxton batch: 16 targets at 2048^2, each an N x N array (N uniform
# in 4-16) of Gaussian spots (sigma 2 samples, amplitudes uniform 0.5-1) on a
# centred pitch of 3/4 of the frame / N; uniform input amplitude, seeded
# random initial phase, Fraunhofer far field (z = 0.2 m, dx = 3 um, 532 nm,
# strict off), 200 iterations with no early stop.  Work unit: one GS
# iteration of one target.
GS_TARGETS, GS_ITERS, GS_SEED = 16, 200, 77
GS_LAM, GS_Z = 532e-9, 0.2
GS_WORKLOAD = ("16 spot-array targets x 2048^2, Fraunhofer GS (z 0.2 m, 532 nm), 200 iterations, "
               "uniform input amplitude, seeded random initial phase")


def gs_targets(n_targets, rng):
    """Target amplitudes (unit total power) and spot centres of each target."""
    yy, xx = np.mgrid[0:N, 0:N]
    out = []
    for _ in range(n_targets):
        k = int(rng.integers(4, 17))
        pitch = 0.75 * N / k
        c0 = N / 2 - pitch * (k - 1) / 2
        cs = [(c0 + pitch * i, c0 + pitch * j) for i in range(k) for j in range(k)]
        t = np.zeros((N, N))
        for (cy, cx) in cs:
            a = rng.uniform(0.5, 1.0)
            y0, y1 = int(cy) - 8, int(cy) + 9
            x0, x1 = int(cx) - 8, int(cx) + 9
            t[y0:y1, x0:x1] += a * np.exp(-((yy[y0:y1, x0:x1] - cy) ** 2
                                            + (xx[y0:y1, x0:x1] - cx) ** 2) / (2 * 2.0 ** 2))
        amp = np.sqrt(t)
        out.append((amp / math.sqrt(np.sum(t)), cs))
    return out


def spot_metrics(inten, centres):
    """Efficiency = power in 5 x 5 windows at the spot centres / total power;
    uniformity = 1 - (max - min) / (max + min) of the window powers."""
    p = []
    for (cy, cx) in centres:
        iy, ix = int(round(cy)), int(round(cx))
        p.append(float(inten[iy - 2:iy + 3, ix - 2:ix + 3].sum()))
    p = np.array(p)
    return float(p.sum() / inten.sum()), float(1.0 - (p.max() - p.min()) / (p.max() + p.min()))


def gs_leg(args, stream):
    import torch
    from optics_studio_gb300 import gs as ggs
    from optics_studio_gb300.propagation.fraunhofer import FraunhoferConfig
    n_t, n_it = args.gs_targets, args.gs_iters
    rng = np.random.default_rng(GS_SEED)
    targets = gs_targets(n_t, rng)
    init = rng.uniform(-math.pi, math.pi, (n_t, N, N))
    c = DX * DX / (GS_LAM * GS_Z)
    scale = c * N * N  # sum |U|^2 = c^2 N^2 sum |u|^2 for a unit input
    u = torch.ones((N, N), dtype=torch.complex64, device="cuda")

    def problems(dtype, idx, iters):
        cdt, rdt = (torch.complex64, torch.float32) if dtype == "f32" else (torch.complex128,
                                                                             torch.float64)
        cfg = ggs.GsConfig(max_iterations=iters, patience=iters + 1)
        return [ggs.GsProblem(u.to(cdt), (DX, DX), GS_LAM, GS_Z,
                              torch.from_numpy(targets[i][0] * scale).to("cuda", rdt),
                              torch.from_numpy(init[i]).to("cuda", rdt), config=cfg,
                              engine="fraunhofer", fraunhofer=FraunhoferConfig(strict=False))
                for i in idx]

    with torch.cuda.stream(stream):
        ggs.run_batch(problems("f32", range(n_t), 3), stream)  # warm-up
        probs = problems("f32", range(n_t), n_it)
        torch.cuda.synchronize()
        import ctypes as C
        import optics_studio_gb300 as og
        from optics_studio_gb300 import _ffi as ffi
        L = og.lib()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        with nvtx_range("gs_timed"):
            sols = ggs.run_batch(probs, stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        its = sum(s.iterations for s in sols)
        # per-kernel device times from a separate profiled call of the same
        # batch cut to 20 iterations (events around every launch)
        ffi.check(L.osgpu_profile_begin())
        ggs.run_batch(problems("f32", range(n_t), 20), stream)
        torch.cuda.synchronize()
        stats = (ffi.KernelStatC * 16)()
        nst = C.c_int32()
        ffi.check(L.osgpu_profile_end(stats, 16, C.byref(nst)))
        kst = {stats[i].name.decode(): {"launches": int(stats[i].launches),
                                        "total_ms": stats[i].total_ms, "bytes": stats[i].bytes,
                                        "ms_per_launch": stats[i].total_ms / max(1, stats[i].launches)}
               for i in range(nst.value)}
        eff32, uni32 = spot_metrics(sols[0].target_intensity.double().cpu().numpy(),
                                    targets[0][1])
        peak, src = hbm_peak()
        gs_bytes = N * N * (8 * 8 + 16)  # per target-iteration: n^2 (8 s + 16), s = 8
        out = {"value": its / (ms / 1e3), "unit": "target-iterations/s", "ms_total": ms,
               "targets": n_t, "iterations_per_target": n_it,
               "workload": GS_WORKLOAD, "dtype": "f32",
               "kernels_profiled_20_iterations": kst,
               "roofline": {"bound": "hbm", "bytes_per_target_iteration": gs_bytes,
                            "achieved": its * gs_bytes / (ms / 1e3) / 1e9, "peak": peak,
                            "unit": "GB/s", "peak_source": src,
                            "frac": its * gs_bytes / (ms / 1e3) / 1e9 / peak,
                            "note": "whole call (set-up, 200 iterations, read-back) timed"},
               "target0": {"efficiency": eff32, "uniformity": uni32}}
        if not args.no_f64:
            t0 = time.perf_counter()
            s64 = ggs.run_batch(problems("f64", [0], n_it), stream)[0]
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            eff64, uni64 = spot_metrics(s64.target_intensity.cpu().numpy(), targets[0][1])
            out["f64_plain"] = {"value": s64.iterations / dt, "unit": "target-iterations/s",
                                "sample": "target 0, complex128, generic GS path",
                                "efficiency": eff64, "uniformity": uni64}
            out["speedup_vs_f64"] = out["value"] / out["f64_plain"]["value"]
    return out


def reference_arm(args):
    """--impl reference: the f64 oracle port on all usable host cores, one
    band per worker process per step (spawned processes, no GPU)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    try:
        with open("/proc/meminfo") as f:
            kb = int([ln for ln in f if ln.startswith("MemAvailable")][0].split()[1])
        mem_workers = max(1, int(kb / 1024 / 1024 // 8))  # ~8 GB per band at P = 8192
    except (OSError, IndexError, ValueError):
        mem_workers = 4
    workers = max(1, min(cores, mem_workers, NBANDS))
    # each step is ~6-7 s of CPU work on 16 cores: bounded so that the whole
    # run stays within a couple of minutes whatever --steps asks for
    steps, warmup = max(1, min(args.steps, 8)), max(1, min(args.warmup, 1))
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        for _ in range(warmup):
            pool.map(_ref_worker, range(workers))
        t0 = time.perf_counter()
        for _ in range(steps):
            pool.map(_ref_worker, range(workers))
        dt = time.perf_counter() - t0
    props = workers * steps
    val = props / dt
    line = {"metric": METRIC, "value": val, "unit": "propagations/s", "n_gpus": world,
            "steps": steps, "warmup": warmup, "ms_per_step": dt / steps * 1e3,
            "steps_requested": args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": workload_config(world),
            "step": f"{workers} bands, one per worker process",
            "cpu_baseline": {"value": val, "unit": "propagations/s", "cores": workers,
                             "kind": "port",
                             "sample": f"bands 0-{workers - 1} of the 32 per step (one band per "
                                       f"worker process), f64 oracle (numpy/pocketfft) "
                                       f"restatement"},
            "e2e": {"value": val, "unit": "propagations/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _ref_worker(i):
    sys.path.insert(0, ROOT)
    _, dt = cpu_baseline_band(i)
    return dt


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-f64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-gs", action="store_true")
    ap.add_argument("--no-ragged", action="store_true")
    ap.add_argument("--no-c2", action="store_true", help="no 1024^2 engine-sweep leg")
    ap.add_argument("--no-autotune", action="store_true",
                    help="built-in pass schedules instead of measured ones")
    ap.add_argument("--no-plans", action="store_true",
                    help="no kernel-spectrum plan legs (the batch with plans, the adjoint "
                         "leg's plans)")
    ap.add_argument("--gs-targets", type=int, default=GS_TARGETS,
                    help="GS leg targets (profiling runs use a smaller batch)")
    ap.add_argument("--gs-iters", type=int, default=GS_ITERS)
    ap.add_argument("--bands", type=int, default=NBANDS,
                    help="bands per step (profiling runs use a smaller batch)")
    args = ap.parse_args()
    set_bands(args.bands)
    if args.impl == "reference":
        reference_arm(args)
        return

    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    import optics_studio_gb300 as og
    from optics_studio_gb300 import _ffi as ffi
    L = og.lib()
    ffi.check(L.osgpu_init(local))
    # An explicit stream: the legacy default stream has handle 0, which the C
    # ABI reads as "the library's own stream", so torch events on it would
    # not bracket the library's kernels.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = C.c_void_p(stream.cuda_stream)
    assert sptr.value, "need a non-default CUDA stream"

    if not args.no_autotune:
        # measured pass schedules: the first (warm-up) batch of each geometry tunes it
        from optics_studio_gb300 import tuning
        tuning.enable()

    lat = doe_lattice()
    handle = C.c_void_p()
    ffi.check(L.osgpu_lattice_create(lat.ctypes.data_as(ffi.c_double_p), N, N, C.byref(handle)))

    # device-resident batch: inputs (unit plane wave) and outputs, complex64
    fin = torch.ones((NBANDS, N, N), dtype=torch.complex64, device="cuda")
    fout = torch.empty_like(fin)
    d_in = [fin[b].data_ptr() for b in range(NBANDS)]
    d_out = [fout[b].data_ptr() for b in range(NBANDS)]
    keep = []
    items = make_items(og, ffi, d_in, d_out, handle.value, keep)

    for _ in range(args.warmup):
        run_batch(og, ffi, items, ffi.C64, sptr)
    torch.cuda.synchronize()
    ffi.check(L.osgpu_sync_status())

    clocks = ClockSampler(local)
    clocks.start()
    launches0 = L.osgpu_launch_count()
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    with nvtx_range("prop_timed"):
        for _ in range(args.steps):
            run_batch(og, ffi, items, ffi.C64, sptr)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms_total = e0.elapsed_time(e1)
    launches = L.osgpu_launch_count() - launches0
    clk = clocks.stop()
    ffi.check(L.osgpu_sync_status())
    # per-kernel device times from a separate profiled pass (the library's
    # events between the passes would stand between its dependent launches)
    ffi.check(L.osgpu_profile_begin())
    prof_steps = min(args.steps, 3)
    for _ in range(prof_steps):
        run_batch(og, ffi, items, ffi.C64, sptr)
    torch.cuda.synchronize()
    stats = (ffi.KernelStatC * 16)()
    nst = C.c_int32()
    ffi.check(L.osgpu_profile_end(stats, 16, C.byref(nst)))

    # band 0 of the headline path, for the oracle check after the other legs
    # (the plans leg rewrites the same output buffers)
    headline_band0 = fout[0].cpu().numpy().astype(np.complex128)
    ms_total = max_over_ranks(ms_total, world)
    ms_step = ms_total / args.steps
    value = job_rate(NBANDS, world, ms_step)

    kstats = {}
    for i in range(nst.value):
        s = stats[i]
        kstats[s.name.decode()] = {"launches": int(s.launches), "total_ms": s.total_ms,
                                   "bytes": s.bytes}
    dom = max(kstats.items(), key=lambda kv: kv[1]["total_ms"])
    peak, peak_src = hbm_peak()
    dname, d = dom
    per_launch_bytes = d["bytes"] / d["launches"]
    per_launch_ms = d["total_ms"] / d["launches"]
    achieved = per_launch_bytes / (per_launch_ms / 1e3) / 1e9
    all_bytes = sum(v["bytes"] for v in kstats.values())
    traffic, traffic_src = traffic_of(dname)

    # Pass B is bound by FP32 instruction issue, not by HBM: its FFT arithmetic
    # against the nominal FP32 rate of this GPU (SMs x 128 lanes x 2 flops x
    # max SM clock), counting 5 m log2 m flops per m-point transform (2 r
    # transforms per spectral column: Px columns of a band).
    props = torch.cuda.get_device_properties(local)
    sm_clock_mhz = clk.get("sm_max_mhz") or 2070.0
    fp32_peak = props.multi_processor_count * 128 * 2 * sm_clock_mhz * 1e6 / 1e12
    m_fft, r_fft = N, 8192 // N
    fft_flops = 8192 * 2 * r_fft * 5.0 * m_fft * math.log2(m_fft)
    b_ms = kstats.get("pass_b_columns", {"total_ms": 0.0, "launches": 1})
    b_ms = b_ms["total_ms"] / max(1, b_ms["launches"])
    compute = None
    if b_ms > 0:
        compute = {"kernel": "pass_b_columns", "bound": "fp32 issue",
                   "fft_tflops": fft_flops / (b_ms / 1e3) / 1e12,
                   "fp32_peak_tflops": fp32_peak, "peak_source": "nominal (SMs x 128 x 2 x max clock)",
                   "frac": fft_flops / (b_ms / 1e3) / 1e12 / fp32_peak,
                   "note": "5 m log2 m flops per transform, 2 r transforms of m = 2048 per column; "
                           "twiddles, H and recombination not counted"}

    line = {"metric": METRIC, "value": value, "unit": "propagations/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": workload_config(world),
            "roofline": {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "traffic_source": traffic_src, "peak_source": peak_src,
                         "bytes_per_launch": per_launch_bytes,
                         "ms_per_launch": per_launch_ms, "compute": compute},
            "kernels": kstats,
            "whole_step_hbm_gbs": all_bytes / prof_steps / (ms_step / 1e3) / 1e9,
            "kernel_stats_steps": prof_steps,
            "clocks": clk, "gpu_launches": int(launches)}
    if not args.no_autotune:
        from optics_studio_gb300 import tuning
        line["schedules"] = tuning.schedules()

    # plain FP64 path on the same batch (device resident complex128)
    if not args.no_f64 and rank == 0:
        nb64 = min(8, NBANDS)
        fin64 = torch.ones((nb64, N, N), dtype=torch.complex128, device="cuda")
        fout64 = torch.empty_like(fin64)
        k2 = []
        it64 = make_items(og, ffi, [fin64[i % nb64].data_ptr() for i in range(NBANDS)],
                          [fout64[i % nb64].data_ptr() for i in range(NBANDS)], handle.value, k2)
        sub = (ffi.TraceItemC * nb64)(*[it64[i * (NBANDS // nb64)] for i in range(nb64)])
        cfg = ffi.AsmConfigC(2.0, 1, 1, 8.0, 1.0)
        ffi.check(L.osgpu_beamline_trace_batch_device(sub, nb64, cfg, ffi.C128, sptr, None, 0))
        torch.cuda.synchronize()
        e0.record(stream)
        ffi.check(L.osgpu_beamline_trace_batch_device(sub, nb64, cfg, ffi.C128, sptr, None, 0))
        e1.record(stream)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1)
        v64 = nb64 / (ms64 / 1e3)
        line["f64_plain"] = {"value": v64, "unit": "propagations/s",
                             "sample": f"{nb64} of the 32 bands, complex128 resident"}
        line["speedup_vs_f64"] = value / world / v64
        del fin64, fout64

    # end to end through the reference-facing host-buffer ABI
    if not args.no_e2e:
        host_in = torch.ones((NBANDS, N, N), dtype=torch.complex128).pin_memory()
        host_out = torch.empty((NBANDS, N, N), dtype=torch.complex128).pin_memory()
        cfg = ffi.AsmConfigC(2.0, 1, 1, 8.0, 1.0)

        hitems = (ffi.HostTraceItemC * NBANDS)()
        for b in range(NBANDS):
            hitems[b] = ffi.HostTraceItemC(
                C.cast(C.c_void_p(host_in[b].data_ptr()), ffi.c_double_p),
                C.cast(C.c_void_p(host_out[b].data_ptr()), ffi.c_double_p), items[b].grid,
                items[b].steps, 3)

        def e2e_step():
            ffi.check(L.osgpu_beamline_trace_batch(hitems, NBANDS, cfg, ffi.F32, None, 0))

        for _ in range(3):
            e2e_step()
        barrier()
        nrep = max(1, min(args.steps, 30))  # the main leg's step count (default 30)
        calls = []
        eclk = ClockSampler(local)
        eclk.start()
        time.sleep(0.3)  # nvidia-smi past its start-up before the host-timed calls
        t0 = time.perf_counter()
        for _ in range(nrep):
            tc = time.perf_counter()
            e2e_step()
            calls.append(NBANDS / (time.perf_counter() - tc))
        dt = max_over_ranks((time.perf_counter() - t0) / nrep * 1e3, world) / 1e3
        e2e_clocks = eclk.stop()
        barrier()
        # the host link's own pinned copy rates on this machine (2 GiB each way; best of 3
        # after one untimed pair)
        dev = torch.empty((NBANDS, N, N), dtype=torch.complex128, device="cuda")
        nb = float(NBANDS * N * N * 16)
        best_in = best_out = 0.0
        for rep in range(4):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            dev.copy_(host_in, non_blocking=True)
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            host_out.copy_(dev, non_blocking=True)
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            if rep:
                best_in = max(best_in, nb / (t2 - t1) / 1e9)
                best_out = max(best_out, nb / (t3 - t2) / 1e9)
        link = {"h2d_gbs": best_in, "d2h_gbs": best_out}
        del dev
        line["e2e"] = {"value": NBANDS * world / dt, "unit": "propagations/s",
                       "h2d_bytes_per_step": NBANDS * N * N * 16,
                       "d2h_bytes_per_step": NBANDS * N * N * 16,
                       "api": "osgpu_beamline_trace_batch (host complex128, pinned; copies "
                              "pipelined against the traces), f32 engine",
                       "host_link": link, "calls": nrep, "clocks": e2e_clocks,
                       "per_call_rates": [round(r, 1) for r in calls],
                       "median_call_rate": round(statistics.median(calls) * world, 1)}

    # the same batch with kernel-spectrum plans (opt-in, not the headline): the
    # first call builds one kernel table per band, later calls run every
    # band as a circular convolution of period 2n (4096^2 instead of 8192^2)
    if not args.no_plans:
        from optics_studio_gb300 import plans
        padded0 = fout[0].clone()
        plans.clear()
        plans.enable(4 << 30)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run_batch(og, ffi, items, ffi.C64, sptr)
        torch.cuda.synchronize()
        first_ms = (time.perf_counter() - t0) * 1e3
        built = plans.stats()
        for _ in range(args.warmup):
            run_batch(og, ffi, items, ffi.C64, sptr)
        barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            run_batch(og, ffi, items, ffi.C64, sptr)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        pms = max_over_ranks(e0.elapsed_time(e1), world) / args.steps
        st = plans.stats()
        rel = float(torch.linalg.norm(fout[0] - padded0) / torch.linalg.norm(padded0))
        gain = ms_step - pms
        line["plans"] = {
            "value": job_rate(NBANDS, world, pms), "unit": "propagations/s",
            "ms_per_step": pms, "steps": args.steps,
            "first_call_ms": first_ms, "tables": built["plans"], "table_bytes": built["bytes"],
            "builds": st["builds"], "hits": st["hits"],
            "break_even_steps": (first_ms - pms) / gain if gain > 0 else None,
            "rel_l2_vs_padded_band0": rel,
            "note": "osgpu_plan_cache_config on: the first call builds the 32 kernel tables "
                    "(one per band) and is timed apart (first_call_ms); value is the "
                    "steady rate of the later calls; the headline value runs without plans"}
        plans.disable()
        plans.clear()

    # adjoint gradients of the inverse-design workload
    if not args.no_adjoint:
        line["adjoint"] = adjoint_leg(args, stream)

    # ragged batch from a captured graph
    if not args.no_ragged:
        line["ragged"] = ragged_leg(args, stream)

    # Gerchberg-Saxton batch
    if not args.no_gs:
        line["gs"] = gs_leg(args, stream)

    # single-plane engine sweep at 1024^2
    if not args.no_c2:
        line["c2"] = c2_leg(args)

    if not args.no_autotune:  # every geometry the legs tuned (headline and ragged sizes)
        from optics_studio_gb300 import tuning
        line["schedules"] = tuning.schedules()

    # accuracy of band 0 against the f64 oracle + bounded CPU baseline
    if rank == 0 and not args.no_cpu_baseline:
        ref, dt_cpu = cpu_baseline_band(0)
        got = headline_band0
        line["rel_l2_vs_oracle_band0"] = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        line["cpu_baseline"] = {"value": 1.0 / dt_cpu, "unit": "propagations/s", "cores": 1,
                                "kind": "port",
                                "sample": "band 0 (450 nm) of the batch: 2048^2 DOE + aperture + "
                                          "lens + ASM at 8192^2, f64 oracle (numpy), 1 thread"}
    L.osgpu_lattice_destroy(handle)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
