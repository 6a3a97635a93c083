"""ctypes binding of the asdpocs_gb300 C ABI (include/asdpocs_gb300.h).

The library is the only compute path: if ``lib/libasdpocs_gb300.so`` is
missing or cannot be loaded, every call raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_PKG = os.path.dirname(os.path.abspath(__file__))
# ASDPOCS_LIB=checked loads the bounds-checked build (build(checked=True))
LIB_PATH = os.path.join(_PKG, "lib", "libasdpocs_gb300_checked.so"
                        if os.environ.get("ASDPOCS_LIB") == "checked" else "libasdpocs_gb300.so")

_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)
_lock = threading.Lock()
_lib = None


class Para(C.Structure):
    """asdpocs_para: the fields the mex gateways read."""

    _fields_ = [("SO", C.c_double), ("OD", C.c_double), ("vxlsize", C.c_double),
                ("detsize", C.c_double), ("phi", C.c_double), ("nx", C.c_int),
                ("ny", C.c_int), ("nz", C.c_int), ("na", C.c_int), ("nb", C.c_int)]


class Options(C.Structure):
    """asdpocs_options: ASD_POCS_cuda.m option set."""

    _fields_ = [("maxnumIter", C.c_int), ("numOfgradients", C.c_int),
                ("alpha", C.c_double), ("alpha_red", C.c_double), ("beta", C.c_double),
                ("beta_red", C.c_double), ("r_max", C.c_double), ("epsilon", C.c_double),
                ("stopRelChg", C.c_double), ("sino_storage", C.c_int), ("ax_mode", C.c_int)]


# asdpocs_options.sino_storage: device storage of the sinogram
SINO_STORAGE = {"f32": 0, "f16": 1, "bf16": 2}
# asdpocs_options.ax_mode: forward projection of the SART steps
AX_MODE = {"reference": 0, "exact": 1}


class Stats(C.Structure):
    _fields_ = [("IterationNum", C.c_int), ("dataTolerance", C.c_double),
                ("alpha", C.c_double), ("beta", C.c_double), ("dp", C.c_double),
                ("dg", C.c_double)]


class Geometry(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("na", C.c_int),
                ("nb", C.c_int), ("nv", C.c_int), ("SO", C.c_double), ("OD", C.c_double),
                ("vxlsize", C.c_double), ("detsize", C.c_double)]


class Shapes(C.Structure):
    """asdpocs_shapes: a plan's launch shapes (none changes a result bit)."""

    _fields_ = [("tv_walk", C.c_int), ("ax_cols", C.c_int), ("ax_quads", C.c_int),
                ("zcol_segment", C.c_int), ("pdl", C.c_int), ("iteration_ms", C.c_double)]


class ServerConfig(C.Structure):
    _fields_ = [("slots_per_lane", C.c_int), ("hbm_budget_bytes", C.c_ulonglong),
                ("inflight", C.c_int)]


class JobTimes(C.Structure):
    _fields_ = [("queued_ms", C.c_double), ("run_ms", C.c_double),
                ("total_ms", C.c_double)]


# (name, restype, argtypes) of every exported function
SIGNATURES = [
    ("asdpocs_last_error", C.c_char_p, []),
    ("asdpocs_last_status", C.c_int, []),
    ("asdpocs_version", C.c_char_p, []),
    ("asdpocs_checked_errors", C.c_int, [C.POINTER(C.c_ulonglong), C.POINTER(C.c_longlong)]),
    ("Ax_cone_mf_gpu_new", None, [_F, _F, _F, C.c_float, C.c_float, _F, _F, C.c_float,
                                  C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                                  C.c_int, C.c_int, C.c_int]),
    ("Atx_cone_mf_gpu_new", None, [_F, _F, _F, C.c_float, C.c_float, _F, _F, C.c_float,
                                   C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                   C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    ("asdpocs_ax_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                                    C.c_float, C.c_void_p, C.c_void_p, C.c_float,
                                    C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                                    C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("asdpocs_ax_siddon", C.c_int, [_F, _F, _F, C.c_float, C.c_float, _F, _F, C.c_float,
                                    C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                                    C.c_int, C.c_int, C.c_int]),
    ("asdpocs_ax_siddon_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                                           C.c_float, C.c_void_p, C.c_void_p, C.c_float,
                                           C.c_float, C.c_float, C.c_float, C.c_int,
                                           C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("asdpocs_atx_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                                     C.c_float, C.c_void_p, C.c_void_p, C.c_float,
                                     C.c_float, C.c_float, C.c_float, C.c_float,
                                     C.c_float, C.c_int, C.c_int, C.c_int, C.c_int,
                                     C.c_int, C.c_void_p]),
    ("Ax_cone_gpu", C.c_int, [_F, C.c_longlong, C.POINTER(Para), _F, _F]),
    ("Atx_cone_gpu", C.c_int, [_F, C.c_longlong, C.POINTER(Para), _F, _F]),
    ("asdpocs_adjoint_check_para", C.c_int, [_F, C.c_longlong, _F, C.c_longlong,
                                             C.POINTER(Para), _D]),
    ("asdpocs_adjoint_check", C.c_int, [_F, _F, C.c_float, C.c_float, _F, _F, C.c_float,
                                        C.c_float, C.c_float, C.c_float, C.c_float,
                                        C.c_float, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.c_int, _D]),
    ("imgTVGradMin", C.c_int, [_D, _D, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int,
                               _D]),
    ("imgTVGradMin3D", C.c_int, [_D, _D, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                                 C.c_int, _D]),
    ("asdpocs_tv_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                    C.c_double, C.c_int, C.c_int, C.c_void_p]),
    ("asdpocs_tv_device_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                            C.c_int, C.c_double, C.c_int, C.c_int,
                                            C.c_void_p]),
    ("asdpocs_options_default", None, [C.POINTER(Options)]),
    ("asdpocs_store_sinogram", C.c_int, [C.c_void_p, C.c_void_p, C.c_ulonglong, C.c_int]),
    ("asdpocs_plan_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int,
                                      C.POINTER(Geometry), _D, C.POINTER(Options),
                                      C.c_ulonglong, C.c_void_p]),
    ("asdpocs_plan_destroy", C.c_int, [C.c_void_p]),
    ("asdpocs_plan_layout", C.c_int, [C.c_int, C.POINTER(Geometry), _D, C.POINTER(Options),
                                      C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("asdpocs_plan_bytes", C.c_ulonglong, [C.c_void_p]),
    ("asdpocs_plan_set_sinogram", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    ("asdpocs_plan_set_initial", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    ("asdpocs_plan_set_reference", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    ("asdpocs_plan_reset", C.c_int, [C.c_void_p]),
    ("asdpocs_plan_run", C.c_int, [C.c_void_p, C.c_int]),
    ("asdpocs_plan_sync", C.c_int, [C.c_void_p]),
    ("asdpocs_plan_get_image", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    ("asdpocs_plan_get_stats", C.c_int, [C.c_void_p, C.c_int, C.POINTER(Stats), _D]),
    ("asdpocs_plan_sinogram_ptr", C.c_void_p, [C.c_void_p, C.c_int]),
    ("asdpocs_plan_image_ptr", C.c_void_p, [C.c_void_p, C.c_int]),
    ("asdpocs_plan_time_phase", C.c_int, [C.c_void_p, C.c_int, C.c_int, _D]),
    ("asdpocs_plan_autotune", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), _D]),
    ("asdpocs_plan_set_tv_walk", C.c_int, [C.c_void_p, C.c_int]),
    ("asdpocs_plan_streams", C.c_int, [C.c_void_p]),
    ("asdpocs_plan_chord_slots", C.c_int, [C.c_void_p]),
    ("asdpocs_plan_autotune_shapes", C.c_int, [C.c_void_p, C.c_int, C.POINTER(Shapes)]),
    ("asdpocs_plan_get_shapes", C.c_int, [C.c_void_p, C.POINTER(Shapes)]),
    ("asdpocs_plan_set_shapes", C.c_int, [C.c_void_p, C.POINTER(Shapes)]),
    ("asdpocs_phantom_device", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _D, C.c_int,
                                         C.c_double, C.c_void_p]),
    ("asdpocs_poisson_noise_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong,
                                               C.c_double, C.c_ulonglong, C.c_void_p]),
    ("asdpocs_server_config_default", None, [C.POINTER(ServerConfig)]),
    ("asdpocs_server_create", C.c_int, [C.POINTER(C.c_void_p), C.POINTER(ServerConfig)]),
    ("asdpocs_server_submit", C.c_int, [C.c_void_p, C.POINTER(Geometry), _D,
                                        C.POINTER(Options), _F, _F, _F,
                                        C.POINTER(C.c_longlong)]),
    ("asdpocs_server_poll", C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(C.c_int)]),
    ("asdpocs_server_cancel", C.c_int, [C.c_void_p, C.c_longlong]),
    ("asdpocs_server_wait", C.c_int, [C.c_void_p, C.c_longlong, _F, C.POINTER(Stats), _D,
                                      C.POINTER(JobTimes)]),
    ("asdpocs_server_memory", C.c_int, [C.c_void_p, C.POINTER(C.c_ulonglong),
                                        C.POINTER(C.c_ulonglong)]),
    ("asdpocs_server_destroy", C.c_int, [C.c_void_p]),
    ("ASD_POCS_cuda", C.c_int, [_D, _D, C.POINTER(Geometry), C.POINTER(Options), _D, _D,
                                _D, _D, C.POINTER(Stats)]),
    ("SART_cuda_inline", C.c_int, [_D, _D, C.POINTER(Geometry), C.c_double, _D, _D, _D]),
]


class AsdpocsError(RuntimeError):
    """A failed library call; ``status`` is the asdpocs_status code."""

    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


def load():
    """Load (once) and return the library; raises if it is not built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"asdpocs_gb300 CUDA library not built ({LIB_PATH}); run "
                    "`python -m asd_pocs_mex_cuda_demo_gb300.build` -- there is no CPU fallback")
            lib = C.CDLL(LIB_PATH)
            for name, res, args in SIGNATURES:
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def check(rc: int):
    """Raise AsdpocsError for a non-zero status from the library."""
    if rc != 0:
        msg = load().asdpocs_last_error().decode(errors="replace")
        raise AsdpocsError(rc, msg or f"asdpocs status {rc}")
