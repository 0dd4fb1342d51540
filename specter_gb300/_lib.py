"""Loader for the in-tree libspecter_gpu.so (the sm_103a kernels behind include/specter_gpu.h).

There is no CPU fallback: if the library is missing or no CUDA device is present, the
calls that need the GPU raise SpecterError.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libspecter_gpu.so")

OK = 0
ERR_NAMES = {1: "SHAPE", 2: "TABLE", 3: "BC", 4: "OOM", 5: "CUDA", 6: "NONFINITE", 7: "ARG", 9: "STATE"}

# every entry point declared in include/specter_gpu.h
EXPORTS = [
    "specter_last_error", "specter_version", "specter_device_count", "specter_set_device",
    "specter_plan_create", "specter_plan_destroy", "specter_plan_info", "specter_plan_engines", "specter_plan_arrays",
    "specter_plan_synchronize", "specter_plan_stream",
    "specter_field_create", "specter_field_destroy", "specter_field_upload", "specter_field_download",
    "specter_field_copy", "specter_field_zero", "specter_field_device_ptr",
    "specter_fftp3d_real_to_complex", "specter_fftp3d_complex_to_real",
    "specter_fftp2d_real_to_complex_xy", "specter_fftp2d_complex_to_real_xy",
    "specter_fftp1d_real_to_complex_z", "specter_fftp1d_complex_to_real_z",
    "specter_derivk", "specter_laplak", "specter_curlk", "specter_gradre", "specter_advect",
    "specter_fc_filter", "specter_energy", "specter_helicity", "specter_cross", "specter_divergence",
    "specter_variance", "specter_product",
    "specter_bouncheck_z", "specter_bouncheck_z_static", "specter_sol_project", "specter_v_imposebc_and_project",
    "specter_s_imposebc",
    "specter_solver_create", "specter_solver_destroy", "specter_solver_fields", "specter_solver_step",
    "specter_solver_stage", "specter_solver_check",
    "specter_solver_autotune", "specter_plan_tile_caps", "specter_plan_set_option", "specter_plan_get_option",
    "specter_graph_create", "specter_graph_launch", "specter_graph_synchronize", "specter_graph_kernels",
    "specter_graph_destroy", "specter_graph_query", "specter_solver_memory", "specter_device_memory",
    "specter_table_check", "specter_fields_upload", "specter_fields_download",
    "specter_timers", "specter_timers_reset",
    "specter_profile", "specter_profile_report", "specter_launch_count",
    "specter_batch_create", "specter_batch_step", "specter_batch_synchronize", "specter_batch_kernels",
    "specter_batch_destroy",
]


class SpecterError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"SPECTER_ERR_{ERR_NAMES.get(code, code)}: {msg}")
        self.code = code


class SolverParams(C.Structure):
    _fields_ = [("solver", C.c_int), ("ord", C.c_int),
                ("dt", C.c_double), ("nu", C.c_double), ("kappa", C.c_double),
                ("gama", C.c_double), ("xmom", C.c_double), ("xtemp", C.c_double),
                ("v_zsta", C.c_double * 2), ("v_zend", C.c_double * 2), ("fused", C.c_int),
                ("omega", C.c_double * 3), ("nl_fp32", C.c_int)]


_lib = None
VP = C.c_void_p
PD = C.POINTER(C.c_double)


def load(path: str | None = None):
    """Load the shared library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        from . import build as _b
        _b.build()
    L = C.CDLL(path)
    for name in EXPORTS:
        getattr(L, name).restype = C.c_int
    L.specter_last_error.restype = C.c_char_p
    L.specter_plan_create.argtypes = [C.POINTER(C.c_int)] * 3 + [PD, C.c_char_p, C.c_int, C.POINTER(VP)]
    L.specter_energy.argtypes = [VP, VP, VP, VP, C.c_int, PD]
    L.specter_helicity.argtypes = [VP, VP, VP, VP, PD]
    L.specter_cross.argtypes = [VP] * 7 + [C.c_int, PD]
    L.specter_divergence.argtypes = [VP, VP, VP, VP, PD]
    L.specter_variance.argtypes = [VP, VP, C.c_int, PD]
    L.specter_product.argtypes = [VP, VP, VP, PD]
    L.specter_bouncheck_z.argtypes = [VP, VP, VP, PD, PD]
    L.specter_bouncheck_z_static.argtypes = [VP, VP, VP, PD, PD]
    L.specter_sol_project.argtypes = [VP] * 5 + [C.c_int] * 3
    L.specter_v_imposebc_and_project.argtypes = [VP] * 5 + [C.c_int, C.c_int, PD, PD]
    L.specter_derivk.argtypes = [VP, VP, VP, C.c_int]
    L.specter_curlk.argtypes = [VP, VP, VP, VP, C.c_int]
    L.specter_solver_create.argtypes = [VP, C.POINTER(SolverParams), C.POINTER(VP)]
    L.specter_solver_step.argtypes = [VP, C.c_int]
    L.specter_solver_stage.argtypes = [VP, C.c_int]
    L.specter_solver_autotune.argtypes = [VP, C.POINTER(C.c_int)]
    L.specter_plan_tile_caps.argtypes = [VP, C.POINTER(C.c_int)]
    L.specter_plan_set_option.argtypes = [VP, C.c_char_p, C.c_int]
    L.specter_plan_get_option.argtypes = [VP, C.c_char_p, C.POINTER(C.c_int)]
    L.specter_graph_create.argtypes = [C.POINTER(VP), C.c_int, C.c_int, C.POINTER(VP)]
    L.specter_graph_launch.argtypes = [VP]
    L.specter_graph_synchronize.argtypes = [VP]
    L.specter_graph_kernels.argtypes = [VP, C.POINTER(C.c_longlong)]
    L.specter_graph_destroy.argtypes = [VP]
    L.specter_graph_query.argtypes = [VP, C.POINTER(C.c_int)]
    L.specter_solver_memory.argtypes = [VP, C.POINTER(C.c_ulonglong)]
    L.specter_device_memory.argtypes = [C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong)]
    L.specter_table_check.argtypes = [C.c_char_p, C.c_int, C.c_int, PD]
    L.specter_fields_upload.argtypes = [C.c_int, C.POINTER(VP), C.POINTER(VP)]
    L.specter_fields_download.argtypes = [C.c_int, C.POINTER(VP), C.POINTER(VP)]
    L.specter_field_create.argtypes = [VP, C.c_int, C.POINTER(VP)]
    L.specter_field_upload.argtypes = [VP, VP]
    L.specter_field_download.argtypes = [VP, VP]
    _lib = L
    return L


def check(code: int) -> None:
    if code != OK:
        msg = _lib.specter_last_error() if _lib is not None else b""
        raise SpecterError(code, (msg or b"").decode(errors="replace"))
