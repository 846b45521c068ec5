"""ctypes binding of the C ABI in include/cpd.h (libcpd.so).

The library is the product: the GPU fitness path is its CUDA code and nothing
here falls back to a Python or CPU implementation. If the shared library is
missing, importing this module raises ImportError.
"""
from __future__ import annotations

import ctypes as C
import os

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.environ.get("CPD_LIBRARY", os.path.join(PKG_ROOT, "_build", "libcpd.so"))

MAX_GLASS = 6
MAX_BINS = 1024
MAX_WAVELENGTHS = 65536
MAX_RAYS = 1 << 22

# cpd_status
OK = 0
NOT_CONVERGED = 1
RAYTRACE_NO_SURFACE_INTERSECTION = 2
RAYTRACE_OUT_OF_BOUNDS = 3
RAYTRACE_TOTAL_INTERNAL_REFLECTION = 4
RAYTRACE_ANGULAR_RESPONSE_TOO_WEAK = 5
INVALID_ARGUMENT = 6
CUDA_ERROR = 7
TIMEOUT = 8
NO_CAPACITY = 9
NOT_IMPLEMENTED = 10
RAYTRACE_ERRORS = (RAYTRACE_NO_SURFACE_INTERSECTION, RAYTRACE_OUT_OF_BOUNDS,
                   RAYTRACE_TOTAL_INTERNAL_REFLECTION, RAYTRACE_ANGULAR_RESPONSE_TOO_WEAK)

TRACE_HYBRID = 0
TRACE_FP32 = 1
TRACE_FP64 = 2
SAMPLING_ADAPTIVE = 0x10  # OR-ed into a trace mode: the per-wavelength SEM stop
SAMPLING_EXACT = 0x20     # with SAMPLING_ADAPTIVE: every wavelength on the exact path
TP_FIXED_N = 0x1          # cpd_transmission_probability_ex: all max_m rays per wavelength


class SpectrometerParams(C.Structure):
    _fields_ = [
        ("nglass", C.c_int32),
        ("ar_coated", C.c_int32),
        ("glass", (C.c_double * 6) * MAX_GLASS),
        ("angles", C.c_double * (MAX_GLASS + 1)),
        ("lengths", C.c_double * MAX_GLASS),
        ("curvature", C.c_double),
        ("height", C.c_double),
        ("width", C.c_double),
        ("bin_count", C.c_uint32),
        ("det_flipped", C.c_int32),
        ("bin_size", C.c_double),
        ("linear_slope", C.c_double),
        ("linear_intercept", C.c_double),
        ("det_length", C.c_double),
        ("max_incident_angle", C.c_double),
        ("det_angle", C.c_double),
        ("det_position", C.c_double * 2),
        ("wavelength_bounds", C.c_double * 2),
        ("beam_width", C.c_double),
        ("beam_y_mean", C.c_double),
    ]


class Design(C.Structure):
    _fields_ = [
        ("nglass", C.c_int32),
        ("bin_count", C.c_uint32),
        ("ar_coated", C.c_int32),
        ("reserved", C.c_int32),
        ("glass", (C.c_double * 6) * MAX_GLASS),
        ("face_point", (C.c_double * 2) * MAX_GLASS),
        ("face_normal", (C.c_double * 2) * MAX_GLASS),
        ("height", C.c_double),
        ("exit_center", C.c_double * 2),
        ("exit_radius", C.c_double),
        ("exit_bound_center", C.c_double * 2),
        ("exit_bound_r2", C.c_double),
        ("bin_size", C.c_double),
        ("linear_slope", C.c_double),
        ("linear_intercept", C.c_double),
        ("min_ci", C.c_double),
        ("det_length", C.c_double),
        ("det_normal", C.c_double * 2),
        ("det_position", C.c_double * 2),
        ("det_direction", C.c_double * 2),
        ("wavelength_bounds", C.c_double * 2),
        ("beam_width", C.c_double),
        ("beam_y_mean", C.c_double),
        ("size", C.c_double),
        ("deviation", C.c_double),
    ]


class Fitness(C.Structure):
    _fields_ = [
        ("size", C.c_double),
        ("info", C.c_double),
        ("deviation", C.c_double),
        ("h_cond", C.c_double),
        ("h_det", C.c_double),
        ("max_sem", C.c_double),
        ("rays", C.c_uint64),
        ("hits", C.c_uint64),
        ("retraced", C.c_uint64),
        ("fast_rays", C.c_uint64),
        ("wavelengths", C.c_uint32),
        ("status", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchItem(C.Structure):
    _fields_ = [("seed", C.c_double), ("max_n", C.c_uint32), ("max_eval", C.c_uint32)]


class LoopConfig(C.Structure):
    _fields_ = [("hist_budget_bytes", C.c_uint64), ("max_cells", C.c_uint32), ("max_rows", C.c_uint32),
                ("ring_capacity", C.c_uint32), ("ctas_per_sm", C.c_uint32), ("idle_ms", C.c_uint32),
                ("ray_tile", C.c_uint32)]


class LoopReport(C.Structure):
    _fields_ = [("designs_done", C.c_uint64), ("device_designs", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("max_designs_in_flight", C.c_uint64), ("pending_designs", C.c_uint64),
                ("table_resets", C.c_uint64), ("inline_retraced", C.c_uint64), ("slab_bytes", C.c_uint64),
                ("ctas", C.c_uint32), ("idle_exits", C.c_uint32), ("stop_exits", C.c_uint32),
                ("reserved", C.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


_dp = C.POINTER(C.c_double)
_up = C.POINTER(C.c_uint32)
_ctxp = C.c_void_p

# (name, restype, argtypes) of every symbol include/cpd.h declares.
SIGNATURES = [
    ("cpd_abi_version", C.c_int, []),
    ("cpd_status_string", C.c_char_p, [C.c_int]),
    ("cpd_position_detector_array", C.c_int, [C.POINTER(SpectrometerParams), C.c_double, _dp, C.POINTER(C.c_int32)]),
    ("cpd_design_build", C.c_int, [C.POINTER(SpectrometerParams), C.POINTER(Design)]),
    ("cpd_design_build_batch", C.c_int, [C.c_void_p, C.c_uint32, C.c_double, C.c_void_p, C.POINTER(C.c_int32)]),
    ("cpd_exit_ray", C.c_int, [C.POINTER(Design), C.c_double, C.c_double, _dp]),
    ("cpd_ray_trace", C.c_int, [C.POINTER(Design), C.c_double, C.c_double, _dp, _up]),
    ("cpd_fitness_cpu", C.c_int, [C.POINTER(Design), C.c_uint64, C.c_uint64, C.POINTER(Fitness)]),
    ("cpd_norminv", C.c_double, [C.c_double]),
    ("cpd_glass_index", C.c_double, [_dp, C.c_double]),
    ("cpd_entropy_log2", C.c_int, [C.c_uint64, _dp]),
    ("cpd_context_create", C.c_int, [C.c_int, C.POINTER(_ctxp)]),
    ("cpd_context_destroy", None, [_ctxp]),
    ("cpd_fitness_gpu", C.c_int, [_ctxp, C.POINTER(Design), _dp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                  C.POINTER(Fitness)]),
    ("cpd_fitness_gpu_ex", C.c_int, [_ctxp, C.POINTER(Design), _dp, C.c_uint32, C.c_uint32, C.c_uint32,
                                     C.c_uint32, C.c_uint32, C.POINTER(Fitness)]),
    ("cpd_fitness_gpu_points", C.c_int, [_ctxp, C.POINTER(Design), _dp, C.c_uint32, _dp, C.c_uint32, C.c_uint32,
                                         C.POINTER(Fitness), _dp]),
    ("cpd_fitness_gpu_points_static", C.c_int, [C.POINTER(Design), _dp, C.c_uint32, _dp, C.c_uint32, C.c_uint32,
                                                C.POINTER(Fitness), _dp]),
    ("cpd_transmission_probability", C.c_int, [_ctxp, C.POINTER(Design), _dp, C.c_uint32, C.c_uint32, _dp]),
    ("cpd_transmission_probability_ex", C.c_int, [_ctxp, C.POINTER(Design), _dp, C.c_uint32, C.c_uint32,
                                                  C.c_uint32, _dp, _up]),
    ("cpd_trace_rays", C.c_int, [_ctxp, C.POINTER(Design), _dp, _dp, C.c_uint32, C.c_uint32, _up, _dp,
                                 C.POINTER(C.c_uint8)]),
    ("cpd_fitness_gpu_batch", C.c_int, [_ctxp, C.POINTER(Design), C.POINTER(BatchItem), C.c_uint32, C.c_uint32,
                                        C.POINTER(Fitness)]),
    ("cpd_fitness_gpu_batch_params", C.c_int, [_ctxp, C.c_void_p, C.c_void_p, C.c_uint32, C.c_double, C.c_uint32,
                                               C.c_void_p]),
    ("cpd_design_build_device", C.c_int, [_ctxp, C.c_void_p, C.c_uint32, C.c_double, C.c_void_p,
                                          C.POINTER(C.c_int32)]),
    ("cpd_autotune_batch", C.c_int, [_ctxp, C.POINTER(Design), C.POINTER(BatchItem), C.c_uint32, C.c_uint32, _up,
                                     _up, _dp]),
    ("cpd_set_autotune", C.c_int, [_ctxp, C.c_int]),
    ("cpd_set_launch_shape", C.c_int, [_ctxp, C.c_uint32, C.c_uint32]),
    ("cpd_get_launch_shape", C.c_int, [_ctxp, _up, _up]),
    ("cpd_last_timing", C.c_int, [_ctxp, _dp, _up]),
    ("cpd_measure_fp32_peak", C.c_int, [_ctxp, C.c_uint32, _dp]),
    ("cpd_measure_sfu_peak", C.c_int, [_ctxp, C.c_uint32, _dp]),
    ("cpd_set_profiling", C.c_int, [_ctxp, C.c_int]),
    ("cpd_last_kernel_times", C.c_int, [_ctxp, _dp]),
    ("cpd_last_transfer_bytes", C.c_int, [_ctxp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    ("cpd_server_create", C.c_int, [_ctxp, C.c_uint64, C.c_uint32, C.c_uint32, C.POINTER(C.c_void_p)]),
    ("cpd_server_submit", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                    C.POINTER(C.c_uint64)]),
    ("cpd_server_submit_params", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_double, C.c_uint32,
                                           C.POINTER(C.c_uint64)]),
    ("cpd_server_wait", C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_double, _dp]),
    ("cpd_server_stats", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                   C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    ("cpd_server_destroy", None, [C.c_void_p]),
    ("cpd_loop_create", C.c_int, [_ctxp, C.POINTER(LoopConfig), C.POINTER(C.c_void_p)]),
    ("cpd_loop_submit", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                  C.POINTER(C.c_uint64)]),
    ("cpd_loop_wait", C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_double, _dp]),
    ("cpd_loop_stats", C.c_int, [C.c_void_p, C.POINTER(LoopReport)]),
    ("cpd_loop_destroy", None, [C.c_void_p]),
]

# numpy mirrors of the records, for whole-generation arrays passed by pointer
import numpy as _np  # noqa: E402

PARAMS_DTYPE = _np.dtype(SpectrometerParams)
DESIGN_DTYPE = _np.dtype(Design)
FITNESS_DTYPE = _np.dtype(Fitness)
BATCH_ITEM_DTYPE = _np.dtype(BatchItem)


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"libcpd.so not found at {LIB_PATH}: build it first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


lib = _load()


def status_string(code: int) -> str:
    return lib.cpd_status_string(code).decode()
