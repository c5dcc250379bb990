"""ctypes binding of libpbi4gpu.so (declared in include/pbi4gpu.h).

There is no CPU fallback: if the library cannot be loaded, or a call fails,
a Pbi4GpuError is raised with the library's message.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import build as _build

PBI4G_OK = 0
PREC_FP32, PREC_FP64, PREC_FP16SPLIT, PREC_BF16, PREC_TF32SPLIT = 0, 1, 2, 3, 4
PRECISIONS = {"fp32": PREC_FP32, "fp64": PREC_FP64, "fp16split": PREC_FP16SPLIT, "bf16": PREC_BF16,
              "tf32split": PREC_TF32SPLIT}

# every entry point the header declares (checked by tests/test_capi.py)
EXPORTS = [
    "pbi4g_last_error", "pbi4g_version", "pbi4g_set_dropin_precision",
    "pbi4g_assign_single_grid", "pbi4g_assign_double_grid", "pbi4g_fcomb", "pbi4g_reduce_array",
    "pbi4g_compute_q2k", "pbi4g_compute_q4k", "pbi4g_measure_pk", "pbi4g_measure_pk_multipoles",
    "pbi4g_count_triangles", "pbi4g_measure_bk", "pbi4g_measure_bk_multipoles", "pbi4g_measure_bk_cross",
    "pbi4g_plan_footprint", "pbi4g_plan_create", "pbi4g_plan_destroy", "pbi4g_plan_set_stream",
    "pbi4g_plan_shape", "pbi4g_plan_map_grid", "pbi4g_plan_map_work", "pbi4g_plan_map_slabs", "pbi4g_plan_tensor_units",
    "pbi4g_plan_triangle_counts", "pbi4g_plan_density",
    "pbi4g_plan_powerspectrum",
    "pbi4g_plan_bispectrum", "pbi4g_plan_run_device", "pbi4g_plan_run_host", "pbi4g_plan_get_delta_half",
    "pbi4g_plan_kernel_launches", "pbi4g_plan_enable_timing", "pbi4g_plan_stage_times", "pbi4g_fft_plan_check",
    "pbi4g_catalog_positions",
    "pbi4g_measure_pk_multipoles_noalloc", "pbi4g_plan_set_delta_half", "pbi4g_plan_set_counts",
    "pbi4g_plan_check", "pbi4g_plan_graph_build", "pbi4g_plan_graph_run_host",
    "pbi4g_device_allocs", "pbi4g_debug_fail_alloc", "pbi4g_plan_debug_wait_limit",
    "pbi4g_scratch_footprint", "pbi4g_scratch_create", "pbi4g_scratch_destroy", "pbi4g_plan_use_scratch",
]
NSTAGES = 12
STAGES = ["assign", "grid_convert", "fft_r2c", "fcomb", "pk_binning", "triangle_counts", "shell_maps_z",
          "shell_maps_y", "triangle_sums", "bk_rows", "shell_maps_x", "assign_sort"]


class Pbi4GpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"pbi4gpu error {code}: {msg}")
        self.code = code


class Config(ctypes.Structure):
    """pbi4g_config of include/pbi4gpu.h."""
    _fields_ = [
        ("grid", ctypes.c_int32), ("box", ctypes.c_float), ("nintp", ctypes.c_int32),
        ("interlacing", ctypes.c_int32), ("multipoles", ctypes.c_int32), ("los", ctypes.c_double * 3),
        ("kbin_ps", ctypes.c_float), ("kcenter_ps", ctypes.c_float), ("nbins_ps", ctypes.c_int32),
        ("do_bispectrum", ctypes.c_int32), ("kbin_bs", ctypes.c_float), ("kcenter_bs", ctypes.c_float),
        ("nbins_bs", ctypes.c_int32), ("iopen", ctypes.c_int32), ("precision", ctypes.c_int32),
        ("map_budget_mb", ctypes.c_int32), ("reserved", ctypes.c_int32 * 6),
    ]


_P = ctypes.c_void_p
_i32, _i64, _f32 = ctypes.c_int32, ctypes.c_int64, ctypes.c_float

_SIGS = {
    "pbi4g_set_dropin_precision": [_i32],
    "pbi4g_assign_single_grid": [_i32, _i32, _i64, _P, _P, _P],
    "pbi4g_assign_double_grid": [_i32, _i32, _i64, _P, _P, _P],
    "pbi4g_fcomb": [_i32, _i32, _i32, _f32, _P, _P],
    "pbi4g_reduce_array": [_i32, _P, _i32, _P],
    "pbi4g_compute_q2k": [_i32, _f32, _P, _i32, _i32, _P],
    "pbi4g_compute_q4k": [_i32, _f32, _P, _i32, _i32, _i32, _i32, _P],
    "pbi4g_measure_pk": [_i32, _f32, _f32, _f32, _i32, _P, _P, _P],
    "pbi4g_measure_pk_multipoles": [_i32, _f32, _f32, _f32, _i32, _P, _P, _P, _P],
    "pbi4g_count_triangles": [_i32, _i32, _f32, _f32, _i32, _i32, _i32, _i64, _P],
    "pbi4g_measure_bk": [_i32, _i32, _f32, _f32, _i32, _f32, _i32, _i64, _i64, _P, _P, _P],
    "pbi4g_measure_bk_multipoles": [_i32, _i32, _f32, _f32, _i32, _f32, _i32, _i64, _i64, _P, _P, _P, _P, _P],
    "pbi4g_measure_bk_cross": [_i32, _i32, _f32, _f32, _i32, _f32, _i32, _i64, _i64, _P, _P, _P, _P],
    "pbi4g_plan_footprint": [ctypes.POINTER(Config), _i64, ctypes.POINTER(_i64)],
    "pbi4g_plan_create": [ctypes.POINTER(Config), ctypes.POINTER(_P)],
    "pbi4g_plan_destroy": [_P],
    "pbi4g_plan_set_stream": [_P, _P],
    "pbi4g_plan_shape": [_P, ctypes.POINTER(_i32), ctypes.POINTER(_i64), ctypes.POINTER(_i32)],
    "pbi4g_plan_map_grid": [_P, ctypes.POINTER(_i32), ctypes.POINTER(_i32)],
    "pbi4g_plan_map_work": [_P, _P, _P],
    "pbi4g_plan_map_slabs": [_P, ctypes.POINTER(_i32), ctypes.POINTER(_i32)],
    "pbi4g_plan_tensor_units": [_P, ctypes.POINTER(_i32), ctypes.POINTER(_i32)],
    "pbi4g_plan_check": [_P],
    "pbi4g_plan_graph_build": [_P, _i32, _i64],
    "pbi4g_plan_graph_run_host": [_P, _i32, _P, _P, _P, _P],
    "pbi4g_plan_triangle_counts": [_P, _P],
    "pbi4g_plan_density": [_P, _i64, _P, _P],
    "pbi4g_plan_powerspectrum": [_P, _P],
    "pbi4g_plan_bispectrum": [_P, _P],
    "pbi4g_plan_run_device": [_P, _i64, _P, _P, _P, _P],
    "pbi4g_plan_run_host": [_P, _i64, _P, _P, _P, _P],
    "pbi4g_plan_get_delta_half": [_P, _P],
    "pbi4g_plan_enable_timing": [_P, _i32],
    "pbi4g_plan_stage_times": [_P, _P, _P],
    "pbi4g_fft_plan_check": [_i32, _i32, _P, _P],
    "pbi4g_catalog_positions": [_i64, _P, _P, _i32, _P, _i32, ctypes.c_double, ctypes.c_double, ctypes.c_double, _P,
                                _P],
    "pbi4g_measure_pk_multipoles_noalloc": [_i32, _f32, _f32, _f32, _i32, _P, _P, _P, _P, _P],
    "pbi4g_plan_set_delta_half": [_P, _i64, _P],
    "pbi4g_plan_set_counts": [_P, _P],
    "pbi4g_debug_fail_alloc": [_i32],
    "pbi4g_plan_debug_wait_limit": [_P, _i64],
    "pbi4g_scratch_footprint": [_i32, _i64, _i32, ctypes.POINTER(_i64)],
    "pbi4g_scratch_create": [_i32, _i64, _i32, ctypes.POINTER(_P)],
    "pbi4g_scratch_destroy": [_P],
    "pbi4g_plan_use_scratch": [_P, _P],
}

_lock = threading.Lock()
_lib = None


def lib(build_if_missing: bool = True):
    """Load libpbi4gpu.so (compiling it first if it is missing and nvcc exists)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise Pbi4GpuError(-1, f"{path} is missing; run pbi4_gb300.build.build()")
            _build.build()
        L = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
        L.pbi4g_last_error.restype = ctypes.c_char_p
        L.pbi4g_last_error.argtypes = []
        L.pbi4g_version.restype = ctypes.c_int
        L.pbi4g_plan_kernel_launches.restype = ctypes.c_int64
        L.pbi4g_plan_kernel_launches.argtypes = [_P]
        L.pbi4g_device_allocs.restype = ctypes.c_int64
        L.pbi4g_device_allocs.argtypes = []
        for name, args in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = ctypes.c_int
        _lib = L
        return L


def check(rc: int) -> None:
    if rc != PBI4G_OK:
        msg = lib().pbi4g_last_error()
        raise Pbi4GpuError(rc, msg.decode() if msg else "")


def ptr(a) -> int | None:
    """Address of a numpy array (host) or anything with data_ptr() (a CUDA tensor)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if isinstance(a, int):
        return a
    raise TypeError(f"cannot take the address of {type(a)}")
