"""ctypes binding of the C ABI declared in include/osgpu.h.

This is the same binding a Rust ``extern "C"`` block would declare; the
structs mirror the header field for field.
"""

import ctypes as C
import os

from . import _build

c_double_p = C.POINTER(C.c_double)

OK = 0
STATUS_NAMES = {
    1: "InvalidDistance", 2: "InvalidWavelength", 3: "InvalidMedium", 4: "EmptyGrid",
    5: "NonFiniteSample", 6: "AliasingRisk", 7: "RegimeViolation",
    20: "InvalidAperture", 21: "OutsideField", 22: "InvalidAxis", 23: "InvalidFocal",
    24: "InvalidOrientation", 25: "InvalidPhase", 26: "InvalidGrid", 27: "InvalidGridPitch",
    28: "InvalidGrating", 29: "InvalidSag", 30: "InvalidThickness", 31: "InvalidSurface",
    40: "WrongDimension", 41: "NotFinite", 42: "OutOfBounds", 43: "Render", 44: "Adjoint",
    100: "Unsupported", 101: "Cuda", 102: "BadArgument", 103: "NoDevice", 104: "OutOfMemory",
}
F64, F32 = 0, 1
C128, C64 = 0, 1


class Grid(C.Structure):
    _fields_ = [("nx", C.c_uint64), ("ny", C.c_uint64), ("dx", C.c_double), ("dy", C.c_double),
                ("lam", C.c_double)]


class AsmConfigC(C.Structure):
    _fields_ = [("padding", C.c_double), ("band_limited", C.c_int32), ("strict", C.c_int32),
                ("max_padding", C.c_double), ("medium", C.c_double)]


class AsmReportC(C.Structure):
    _fields_ = [("lam", C.c_double), ("medium", C.c_double), ("z", C.c_double),
                ("nx", C.c_uint64), ("ny", C.c_uint64), ("dx", C.c_double), ("dy", C.c_double),
                ("requested_padding", C.c_double), ("used_padding", C.c_double),
                ("nx_pad", C.c_uint64), ("ny_pad", C.c_uint64),
                ("band_limit_fx", C.c_double), ("band_limit_fy", C.c_double),
                ("max_phase_step_x", C.c_double), ("max_phase_step_y", C.c_double),
                ("nyquist_ok", C.c_int32)]


class FresnelConfigC(C.Structure):
    _fields_ = [("padding", C.c_double), ("strict", C.c_int32), ("max_padding", C.c_double)]


class FresnelReportC(C.Structure):
    _fields_ = [("lam", C.c_double), ("z", C.c_double), ("nx", C.c_uint64), ("ny", C.c_uint64),
                ("dx", C.c_double), ("dy", C.c_double), ("requested_padding", C.c_double),
                ("used_padding", C.c_double), ("nx_pad", C.c_uint64), ("ny_pad", C.c_uint64),
                ("max_phase_step_x", C.c_double), ("max_phase_step_y", C.c_double),
                ("nyquist_ok", C.c_int32), ("max_kernel_step_x", C.c_double),
                ("max_kernel_step_y", C.c_double), ("kernel_nyquist_ok", C.c_int32),
                ("max_phase_error_vs_asm", C.c_double), ("paraxial_ok", C.c_int32)]


class FraunhoferConfigC(C.Structure):
    _fields_ = [("strict", C.c_int32), ("max_n_f", C.c_double), ("has_source_pos", C.c_int32),
                ("source_x", C.c_double), ("source_y", C.c_double),
                ("has_aperture_extent", C.c_int32), ("aperture_extent", C.c_double)]


class FraunhoferReportC(C.Structure):
    _fields_ = [("lam", C.c_double), ("z", C.c_double), ("nx", C.c_uint64), ("ny", C.c_uint64),
                ("dx", C.c_double), ("dy", C.c_double), ("dx_out", C.c_double),
                ("dy_out", C.c_double), ("n_f_x", C.c_double), ("n_f_y", C.c_double),
                ("source_x", C.c_double), ("source_y", C.c_double), ("extent_used", C.c_double),
                ("extent_is_aperture", C.c_int32), ("quad_phase_error_rad", C.c_double),
                ("max_n_f", C.c_double), ("regime_ok", C.c_int32)]


class RsConfigC(C.Structure):
    _fields_ = [("padding", C.c_double), ("strict", C.c_int32)]


class RsReportC(C.Structure):
    _fields_ = [("lam", C.c_double), ("z", C.c_double), ("nx", C.c_uint64), ("ny", C.c_uint64),
                ("dx", C.c_double), ("dy", C.c_double), ("padding", C.c_double),
                ("nx_pad", C.c_uint64), ("ny_pad", C.c_uint64),
                ("max_kernel_step_x", C.c_double), ("max_kernel_step_y", C.c_double),
                ("kernel_nyquist_ok", C.c_int32), ("max_phase_error_vs_fresnel", C.c_double),
                ("paraxial_ok", C.c_int32)]


class ElementC(C.Structure):
    _fields_ = [("kind", C.c_int32), ("stop", C.c_int32), ("a", C.c_double), ("b", C.c_double),
                ("orientation", C.c_double), ("center_x", C.c_double), ("center_y", C.c_double),
                ("focal", C.c_double), ("period", C.c_double), ("depth", C.c_double),
                ("lattice", c_double_p), ("lnx", C.c_uint64), ("lny", C.c_uint64),
                ("ldx", C.c_double), ("ldy", C.c_double), ("lattice_on_device", C.c_int32)]


class StepC(C.Structure):
    _fields_ = [("elements", C.POINTER(ElementC)), ("n_elements", C.c_int32),
                ("z_after", C.c_double), ("medium", C.c_double)]


class TraceItemC(C.Structure):
    _fields_ = [("d_in", C.c_void_p), ("d_out", C.c_void_p), ("grid", Grid),
                ("steps", C.POINTER(StepC)), ("n_steps", C.c_int32)]


class FrameC(C.Structure):
    _fields_ = [("grid", Grid), ("d_source", C.c_void_p), ("steps", C.POINTER(StepC)),
                ("n_steps", C.c_int32), ("d_intensity", C.c_void_p), ("d_dmdi", C.c_void_p),
                ("dmdi_scale", C.c_double), ("d_grad", C.POINTER(C.c_void_p))]


class AdamConfigC(C.Structure):
    _fields_ = [("lr_frac", C.c_double), ("beta1", C.c_double), ("beta2", C.c_double),
                ("eps", C.c_double), ("clip_norm", C.c_double), ("clip", C.c_int32)]


class GsConfigC(C.Structure):
    _fields_ = [("max_iterations", C.c_int32), ("patience", C.c_int32),
                ("merit_tolerance", C.c_double), ("variant", C.c_int32), ("beta", C.c_double),
                ("lo", C.c_double), ("hi", C.c_double), ("engine", C.c_int32)]


class GsRecordC(C.Structure):
    _fields_ = [("iteration", C.c_uint64), ("merit", C.c_double), ("best_merit", C.c_double),
                ("amplitude_mse", C.c_double), ("target_error_rms", C.c_double),
                ("phase_update_rms", C.c_double)]


class GsResultC(C.Structure):
    _fields_ = [("merit", C.c_double), ("best_iteration", C.c_uint64),
                ("amplitude_mse", C.c_double), ("converged", C.c_int32),
                ("iterations", C.c_uint64)]


class GsItemC(C.Structure):
    _fields_ = [("grid", Grid), ("z", C.c_double), ("aperture", C.c_int32),
                ("aperture_a", C.c_double), ("aperture_b", C.c_double),
                ("center_x", C.c_double), ("center_y", C.c_double),
                ("d_input", C.c_void_p), ("d_target_amplitude", C.c_void_p),
                ("d_target_intensity", C.c_void_p), ("d_phase", C.c_void_p),
                ("d_last_phase", C.c_void_p), ("d_best_intensity", C.c_void_p),
                ("d_target_error", C.c_void_p), ("d_phase_error", C.c_void_p),
                ("d_illumination", C.c_void_p), ("history", C.POINTER(GsRecordC)),
                ("result", GsResultC)]


class HostTraceItemC(C.Structure):
    _fields_ = [("in_", c_double_p), ("out", c_double_p), ("grid", Grid),
                ("steps", C.POINTER(StepC)), ("n_steps", C.c_int32)]


class KernelStatC(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_uint64), ("total_ms", C.c_double),
                ("bytes", C.c_double)]


class PlanStatsC(C.Structure):
    _fields_ = [("plans", C.c_uint64), ("bytes", C.c_uint64), ("hits", C.c_uint64),
                ("builds", C.c_uint64)]


class ScheduleInfoC(C.Structure):
    _fields_ = [("mx", C.c_uint32), ("rx", C.c_uint32), ("my", C.c_uint32), ("ry", C.c_uint32),
                ("nx", C.c_uint32), ("ny", C.c_uint32), ("lanes", C.c_uint32),
                ("pass_a", C.c_char * 8), ("pass_b", C.c_char * 8), ("pass_c", C.c_char * 8),
                ("ms_default", C.c_double), ("ms_best", C.c_double)]


# (name, restype, argtypes) for every symbol of include/osgpu.h
SIGNATURES = [
    ("osgpu_init", C.c_int, [C.c_int32]),
    ("osgpu_shutdown", C.c_int, []),
    ("osgpu_last_error", C.c_int, [C.c_char_p, C.c_size_t]),
    ("osgpu_sync_status", C.c_int, []),
    ("osgpu_version", C.c_char_p, []),
    ("osgpu_launch_count", C.c_uint64, []),
    ("osgpu_field_create", C.c_int, [C.c_uint64, C.c_uint64, C.c_int32, C.POINTER(C.c_void_p)]),
    ("osgpu_field_upload", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("osgpu_field_download", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("osgpu_field_info", C.c_int,
     [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
      C.POINTER(C.c_int32)]),
    ("osgpu_field_destroy", C.c_int, [C.c_void_p]),
    ("osgpu_asm_sampling_report", C.c_int,
     [C.POINTER(Grid), C.c_double, C.POINTER(AsmConfigC), C.POINTER(AsmReportC)]),
    ("osgpu_asm_propagate", C.c_int,
     [c_double_p, c_double_p, C.POINTER(Grid), C.c_double, C.POINTER(AsmConfigC), C.c_int32,
      C.POINTER(AsmReportC)]),
    ("osgpu_asm_propagate_device", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(Grid), C.c_double, C.POINTER(AsmConfigC),
      C.c_void_p, C.POINTER(AsmReportC)]),
    ("osgpu_fresnel_sampling_report", C.c_int,
     [C.POINTER(Grid), C.c_double, C.POINTER(FresnelConfigC), C.POINTER(FresnelReportC)]),
    ("osgpu_fresnel_propagate", C.c_int,
     [c_double_p, c_double_p, C.POINTER(Grid), C.c_double, C.POINTER(FresnelConfigC), C.c_int32,
      C.POINTER(FresnelReportC)]),
    ("osgpu_fresnel_propagate_convolution", C.c_int,
     [c_double_p, c_double_p, C.POINTER(Grid), C.c_double, C.POINTER(FresnelConfigC), C.c_int32,
      C.POINTER(FresnelReportC)]),
    ("osgpu_fraunhofer_regime_report", C.c_int,
     [C.POINTER(Grid), C.c_double, C.POINTER(FraunhoferConfigC), C.POINTER(FraunhoferReportC)]),
    ("osgpu_fraunhofer_propagate", C.c_int,
     [c_double_p, c_double_p, C.POINTER(Grid), C.c_double, C.POINTER(FraunhoferConfigC),
      C.c_int32, C.POINTER(FraunhoferReportC)]),
    ("osgpu_rs_sampling_report", C.c_int,
     [C.POINTER(Grid), C.c_double, C.POINTER(RsConfigC), C.POINTER(RsReportC)]),
    ("osgpu_rs_propagate", C.c_int,
     [c_double_p, c_double_p, C.POINTER(Grid), C.c_double, C.POINTER(RsConfigC), C.c_int32,
      C.POINTER(RsReportC)]),
    ("osgpu_apply_elements", C.c_int,
     [c_double_p, c_double_p, C.POINTER(Grid), C.POINTER(ElementC), C.c_int32, C.c_int32]),
    ("osgpu_beamline_trace", C.c_int,
     [c_double_p, c_double_p, C.POINTER(Grid), C.POINTER(StepC), C.c_int32,
      C.POINTER(AsmConfigC), C.c_int32, C.POINTER(AsmReportC)]),
    ("osgpu_beamline_trace_batch_device", C.c_int,
     [C.POINTER(TraceItemC), C.c_int32, C.POINTER(AsmConfigC), C.c_int32, C.c_void_p,
      C.POINTER(AsmReportC), C.c_int32]),
    ("osgpu_lattice_create", C.c_int,
     [c_double_p, C.c_uint64, C.c_uint64, C.POINTER(C.c_void_p)]),
    ("osgpu_lattice_destroy", C.c_int, [C.c_void_p]),
    ("osgpu_beamline_trace_batch", C.c_int,
     [C.POINTER(HostTraceItemC), C.c_int32, C.POINTER(AsmConfigC), C.c_int32,
      C.POINTER(AsmReportC), C.c_int32]),
    ("osgpu_beamline_trace_batch_graph", C.c_int,
     [C.POINTER(TraceItemC), C.c_int32, C.POINTER(AsmConfigC), C.c_int32,
      C.POINTER(C.c_void_p)]),
    ("osgpu_graph_launch", C.c_int, [C.c_void_p, C.c_void_p]),
    ("osgpu_graph_destroy", C.c_int, [C.c_void_p]),
    ("osgpu_source_gaussian_device", C.c_int,
     [C.c_void_p, C.c_int32, C.POINTER(Grid), C.c_double, C.c_double, C.c_double, C.c_double,
      C.c_double, C.c_void_p]),
    ("osgpu_source_plane_wave_device", C.c_int,
     [C.c_void_p, C.c_int32, C.POINTER(Grid), C.c_double, C.c_double, C.c_double, C.c_void_p]),
    ("osgpu_source_uniform_device", C.c_int,
     [C.c_void_p, C.c_int32, C.POINTER(Grid), C.c_double, C.c_double, C.c_void_p]),
    ("osgpu_fft2", C.c_int, [c_double_p, c_double_p, C.c_uint64, C.c_uint64, C.c_int32,
                             C.c_int32]),
    ("osgpu_fft2_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_uint64, C.c_uint64,
                                    C.c_int32, C.c_void_p]),
    ("osgpu_tape_create", C.c_int, [C.c_uint64, C.POINTER(C.c_void_p)]),
    ("osgpu_tape_destroy", C.c_int, [C.c_void_p]),
    ("osgpu_tape_bytes", C.c_uint64, [C.c_void_p]),
    ("osgpu_render_batch_device", C.c_int,
     [C.POINTER(FrameC), C.c_int32, C.POINTER(AsmConfigC), C.c_int32, C.c_void_p, C.c_void_p,
      C.POINTER(AsmReportC), C.c_int32]),
    ("osgpu_push_back_batch_device", C.c_int,
     [C.POINTER(FrameC), C.c_int32, C.POINTER(AsmConfigC), C.c_int32, C.c_void_p, C.c_void_p]),
    ("osgpu_field_power_device", C.c_int,
     [C.c_void_p, C.c_int32, C.c_uint64, C.c_void_p, C.POINTER(C.c_double)]),
    ("osgpu_merit_spot_efficiency_device", C.c_int,
     [C.c_void_p, C.c_int32, C.c_int32, C.c_uint64, C.c_void_p, c_double_p, C.c_void_p,
      C.c_void_p, C.POINTER(C.c_double)]),
    ("osgpu_merit_weighted_efficiency_device", C.c_int,
     [C.c_void_p, C.c_int32, C.c_int32, C.c_uint64, C.c_void_p, c_double_p, C.c_void_p,
      C.c_void_p, C.POINTER(C.c_double)]),
    ("osgpu_merit_mse_device", C.c_int,
     [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.c_void_p, C.c_int32, C.c_int32,
      C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    ("osgpu_merit_encircled_energy_device", C.c_int,
     [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.c_uint64, C.c_double,
      C.c_double, C.c_double, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
      C.POINTER(C.c_double)]),
    ("osgpu_merit_spot_rms_device", C.c_int,
     [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.c_uint64, C.c_double,
      C.c_double, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    ("osgpu_merit_strehl_device", C.c_int,
     [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.c_uint64, C.c_void_p,
      C.c_int32, C.c_int32, C.c_void_p, C.POINTER(C.c_double)]),
    ("osgpu_merit_mtf_device", C.c_int,
     [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.c_uint64, C.c_double,
      C.c_double, C.c_int32, C.c_int32, C.c_void_p, C.POINTER(C.c_double)]),
    ("osgpu_adam_step_device", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_uint64,
      C.POINTER(AdamConfigC), C.c_int32, C.c_double, C.c_double, C.c_void_p]),
    ("osgpu_gs_run_batch_device", C.c_int,
     [C.POINTER(GsItemC), C.c_int32, C.POINTER(GsConfigC), C.POINTER(AsmConfigC),
      C.POINTER(FraunhoferConfigC), C.c_int32, C.c_void_p]),
    ("osgpu_asm_propagate_noalloc", C.c_int,
     [C.c_void_p, C.c_void_p, C.POINTER(Grid), C.c_double, C.POINTER(AsmConfigC), C.c_void_p,
      C.POINTER(AsmReportC)]),
    ("osgpu_psf_spot_rms_device", C.c_int,
     [C.c_void_p, C.c_int32, C.POINTER(Grid), C.c_void_p, C.POINTER(C.c_double)]),
    ("osgpu_psf_mtf_device", C.c_int,
     [C.c_void_p, C.c_int32, C.POINTER(Grid), C.c_void_p, C.POINTER(C.c_double),
      C.POINTER(C.c_double)]),
    ("osgpu_psf_encircled_energy_device", C.c_int,
     [C.c_void_p, C.c_int32, C.POINTER(Grid), C.c_void_p, C.POINTER(C.c_double),
      C.POINTER(C.c_double), C.c_uint64, C.POINTER(C.c_uint64)]),
    ("osgpu_psf_strehl_device", C.c_int,
     [C.c_void_p, C.POINTER(Grid), C.c_void_p, C.POINTER(Grid), C.c_int32, C.c_void_p,
      C.POINTER(C.c_double)]),
    ("osgpu_plan_cache_config", C.c_int, [C.c_int32, C.c_uint64]),
    ("osgpu_plan_cache_clear", C.c_int, []),
    ("osgpu_plan_cache_stats", C.c_int, [C.POINTER(PlanStatsC)]),
    ("osgpu_autotune_config", C.c_int, [C.c_int32]),
    ("osgpu_autotune_asm", C.c_int,
     [C.POINTER(Grid), C.c_double, C.POINTER(AsmConfigC), C.c_int32, C.POINTER(ScheduleInfoC)]),
    ("osgpu_autotune_list", C.c_int,
     [C.POINTER(ScheduleInfoC), C.c_int32, C.POINTER(C.c_int32)]),
    ("osgpu_autotune_clear", C.c_int, []),
    ("osgpu_profile_begin", C.c_int, []),
    ("osgpu_profile_end", C.c_int, [C.POINTER(KernelStatC), C.c_int32, C.POINTER(C.c_int32)]),
]

_lib = None


def lib():
    """Loads (building first if stale) the in-tree libosgpu.so.

    There is no fallback: without the library every product call raises.
    """
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path) or os.environ.get("OSGPU_REBUILD"):
            _build.build()
        L = C.CDLL(path)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error():
    buf = C.create_string_buffer(1024)
    lib().osgpu_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


class OsgpuError(RuntimeError):
    """A non-OK status from the C ABI; ``variant`` is the reference error name."""

    def __init__(self, code, report=None):
        self.code = code
        self.variant = STATUS_NAMES.get(code, f"status{code}")
        self.report = report
        super().__init__(f"{self.variant}: {last_error()}")


def check(code, report=None):
    if code != OK:
        raise OsgpuError(code, report)
