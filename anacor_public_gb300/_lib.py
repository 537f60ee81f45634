"""ctypes binding of libanacor_gb300.so.

The library is loaded from the package's in-tree ``_build`` directory.  If it
is missing the import of the binding raises: there is no host fallback for
the absorption path.
"""
from __future__ import annotations

import ctypes as ct
import os

import numpy as np

from . import build as _build

_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i8p = np.ctypeslib.ndpointer(dtype=np.int8, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_i8ppp = ct.POINTER(ct.POINTER(ct.POINTER(ct.c_int8)))

# every symbol declared in include/anacor_gb300.h
EXPORTS = (
    "ray_tracing_overall", "ray_tracing_single", "ib_test", "ray_tracing_gpu_overall",
    "anacor_last_status", "anacor_last_error", "anacor_version", "anacor_absorption",
    "anacor_plan_create", "anacor_plan_set_reflections", "anacor_plan_run", "anacor_plan_result",
    "anacor_plan_device_result", "anacor_plan_n_refl", "anacor_plan_launch_info", "anacor_plan_destroy",
    "anacor_plan_count_steps",
    "anacor_batch_run", "anacor_rotated_vectors", "anacor_leg_detail", "anacor_absorption_noalloc",
    "anacor_plan_configure", "anacor_plan_config", "anacor_plan_autotune", "anacor_batch_create",
    "anacor_batch_configure", "anacor_batch_autotune", "anacor_batch_launch", "anacor_batch_capture",
    "anacor_batch_replay", "anacor_batch_wait", "anacor_batch_info", "anacor_batch_destroy",
    "anacor_surrogate_create", "anacor_surrogate_destroy", "anacor_surrogate_param_count",
    "anacor_surrogate_members", "anacor_surrogate_params", "anacor_surrogate_fourier", "anacor_surrogate_scale",
    "anacor_surrogate_inputs", "anacor_surrogate_inputs_device", "anacor_surrogate_set_data",
    "anacor_surrogate_train", "anacor_surrogate_gradients", "anacor_surrogate_predict",
    "anacor_surrogate_predict_device", "anacor_surrogate_audit_flags", "anacor_surrogate_save",
    "anacor_surrogate_load", "anacor_tc_gemm_check",
    "anacor_gridding_directions", "anacor_gridding_create", "anacor_gridding_build", "anacor_gridding_info",
    "anacor_gridding_axes", "anacor_gridding_device_map", "anacor_gridding_map", "anacor_gridding_set_map",
    "anacor_gridding_interpolate", "anacor_gridding_interpolate_async", "anacor_gridding_destroy",
    "ray_tracing_single_gridding", "ib_single_gridding", "nearest_neighbor_interpolate_overall",
    "anacor_plan_create_sampled", "anacor_plan_n_voxels", "anacor_plan_voxels", "anacor_sample_voxels",
    "anacor_plan_run_bisection", "anacor_bisection", "anacor_gridding_prepare", "anacor_gridding_run",
    "anacor_distance_field", "anacor_batch_kernels", "anacor_octant_fields", "anacor_block_guard_check",
    "anacor_surrogate_set_inference", "anacor_wait_guard_check",
)

_LIB = None


class AnacorError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"anacor status {status}: {msg}")
        self.status = status


def library_path() -> str:
    return _build.LIB


def load(path: str | None = None) -> ct.CDLL:
    """Load (once) and type the library.  Raises if it has not been built."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    path = path or _build.LIB
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m anacor_public_gb300.build` "
                          "(the absorption path has no CPU fallback)")
    L = ct.CDLL(path)
    # drop-ins, argtypes as AnACor/utils/utils_mp.py:59-148
    L.ray_tracing_overall.restype = ct.POINTER(ct.c_double)
    L.ray_tracing_overall.argtypes = [ct.c_int64, ct.c_int64, np.ctypeslib.ndpointer(dtype=np.int64), ct.c_int64,
                                      np.ctypeslib.ndpointer(dtype=np.float64),
                                      np.ctypeslib.ndpointer(dtype=np.float64),
                                      np.ctypeslib.ndpointer(dtype=np.float64),
                                      np.ctypeslib.ndpointer(dtype=np.float64),
                                      np.ctypeslib.ndpointer(dtype=np.float64), ct.c_int64,
                                      np.ctypeslib.ndpointer(dtype=np.float64),
                                      np.ctypeslib.ndpointer(dtype=np.float64), _i8ppp,
                                      np.ctypeslib.ndpointer(dtype=np.int64), ct.c_int, ct.c_int, ct.c_int,
                                      ct.c_int]
    L.ray_tracing_single.restype = ct.c_double
    L.ray_tracing_single.argtypes = [np.ctypeslib.ndpointer(dtype=np.int64), ct.c_int64,
                                     np.ctypeslib.ndpointer(dtype=np.float64),
                                     np.ctypeslib.ndpointer(dtype=np.float64),
                                     np.ctypeslib.ndpointer(dtype=np.float64),
                                     np.ctypeslib.ndpointer(dtype=np.float64), _i8ppp,
                                     np.ctypeslib.ndpointer(dtype=np.int64), ct.c_int, ct.c_int64, ct.c_int]
    L.ib_test.restype = ct.c_double
    L.ib_test.argtypes = [np.ctypeslib.ndpointer(dtype=np.int64), ct.c_int64,
                          np.ctypeslib.ndpointer(dtype=np.float64), np.ctypeslib.ndpointer(dtype=np.float64),
                          np.ctypeslib.ndpointer(dtype=np.float64), np.ctypeslib.ndpointer(dtype=np.float64),
                          _i8ppp, np.ctypeslib.ndpointer(dtype=np.int64), ct.c_int, ct.c_int64, ct.c_int]
    L.ray_tracing_gpu_overall.restype = ct.POINTER(ct.c_float)
    L.ray_tracing_gpu_overall.argtypes = [ct.c_size_t, ct.c_size_t, np.ctypeslib.ndpointer(dtype=np.int32),
                                          ct.c_size_t] + [np.ctypeslib.ndpointer(dtype=np.float32)] * 5 + [
        ct.c_size_t, np.ctypeslib.ndpointer(dtype=np.float32), np.ctypeslib.ndpointer(dtype=np.float32), _i8ppp,
        ct.POINTER(ct.c_int8), np.ctypeslib.ndpointer(dtype=np.int32), ct.c_int, ct.c_int, ct.c_int]
    L.anacor_last_status.restype = ct.c_int
    L.anacor_last_status.argtypes = []
    L.anacor_last_error.restype = ct.c_char_p
    L.anacor_last_error.argtypes = []
    L.anacor_version.restype = ct.c_char_p
    L.anacor_version.argtypes = []
    L.anacor_absorption.restype = ct.c_int
    L.anacor_absorption.argtypes = [_i8p, _i64p, _i64p, ct.c_int64, _f64p, _f64p, ct.c_int64, _f64p, _f64p, _f64p,
                                    _f64p, _f64p, ct.c_int, ct.c_int, _f64p]
    L.anacor_plan_create.restype = ct.c_void_p
    L.anacor_plan_create.argtypes = [_i8p, _i64p, _i64p, ct.c_int64, _f64p, _f64p, ct.c_int, ct.c_int]
    L.anacor_plan_set_reflections.restype = ct.c_int
    L.anacor_plan_set_reflections.argtypes = [ct.c_void_p, _f64p, _f64p, ct.c_int64, _f64p, _f64p, _f64p]
    L.anacor_plan_run.restype = ct.c_int
    L.anacor_plan_run.argtypes = [ct.c_void_p, ct.c_void_p]
    L.anacor_plan_result.restype = ct.c_int
    L.anacor_plan_result.argtypes = [ct.c_void_p, _f64p, ct.c_void_p]
    L.anacor_plan_device_result.restype = ct.c_void_p
    L.anacor_plan_device_result.argtypes = [ct.c_void_p]
    L.anacor_plan_n_refl.restype = ct.c_int64
    L.anacor_plan_n_refl.argtypes = [ct.c_void_p]
    L.anacor_plan_launch_info.restype = ct.c_int
    L.anacor_plan_launch_info.argtypes = [ct.c_void_p, ct.POINTER(ct.c_int), ct.POINTER(ct.c_int)]
    L.anacor_plan_count_steps.restype = ct.c_int
    L.anacor_plan_count_steps.argtypes = [ct.c_void_p, ct.POINTER(ct.c_uint64)]
    L.anacor_plan_destroy.restype = None
    L.anacor_plan_destroy.argtypes = [ct.c_void_p]
    L.anacor_batch_run.restype = ct.c_int
    L.anacor_batch_run.argtypes = [ct.POINTER(ct.c_void_p), ct.c_int, ct.c_void_p]
    L.anacor_rotated_vectors.restype = ct.c_int
    L.anacor_rotated_vectors.argtypes = [_f64p, _f64p, _f64p, _f64p, _f64p, ct.c_int64, _f64p, _f64p]
    L.anacor_leg_detail.restype = ct.c_int
    L.anacor_leg_detail.argtypes = [_i8p, _i64p, _i64p, ct.c_int64, _f64p, _f64p, _f64p, ct.c_int,
                                    _i32p, _i32p, _i32p, _i32p, _i32p, _f64p, _i32p]
    L.anacor_wait_guard_check.restype = ct.c_int
    L.anacor_wait_guard_check.argtypes = [ct.c_uint, ct.POINTER(ct.c_int32)]
    L.anacor_surrogate_set_inference.restype = ct.c_int
    L.anacor_surrogate_set_inference.argtypes = [ct.c_void_p, ct.c_int]
    L.anacor_block_guard_check.restype = ct.c_int
    L.anacor_block_guard_check.argtypes = [ct.c_int, ct.POINTER(ct.c_int32)]
    L.anacor_absorption_noalloc.restype = ct.c_int
    L.anacor_absorption_noalloc.argtypes = [ct.c_void_p, _i64p, ct.c_void_p, ct.c_int64, _f64p, _f64p, ct.c_int64,
                                            _f64p, _f64p, _f64p, _f64p, _f64p, ct.c_int, ct.c_int, ct.c_void_p,
                                            ct.c_void_p]
    L.anacor_plan_configure.restype = ct.c_int
    L.anacor_plan_configure.argtypes = [ct.c_void_p, ct.c_int, ct.c_int, ct.c_int]
    L.anacor_batch_kernels.restype = ct.c_int
    L.anacor_batch_kernels.argtypes = [ct.c_void_p]
    L.anacor_octant_fields.restype = ct.c_int
    L.anacor_octant_fields.argtypes = [_i8p, _i64p, np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")]
    L.anacor_distance_field.restype = ct.c_int
    L.anacor_distance_field.argtypes = [_i8p, _i64p, np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")]
    L.anacor_plan_config.restype = ct.c_int
    L.anacor_plan_config.argtypes = [ct.c_void_p, ct.POINTER(ct.c_int), ct.POINTER(ct.c_int), ct.POINTER(ct.c_int)]
    L.anacor_plan_autotune.restype = ct.c_int
    L.anacor_plan_autotune.argtypes = [ct.c_void_p, ct.c_int64, ct.POINTER(ct.c_float)]
    L.anacor_batch_create.restype = ct.c_void_p
    L.anacor_batch_create.argtypes = [ct.POINTER(ct.c_void_p), ct.c_int]
    for name in ("anacor_batch_launch", "anacor_batch_capture", "anacor_batch_replay", "anacor_batch_wait"):
        getattr(L, name).restype = ct.c_int
        getattr(L, name).argtypes = [ct.c_void_p, ct.c_void_p]
    L.anacor_batch_configure.restype = ct.c_int
    L.anacor_batch_configure.argtypes = [ct.c_void_p, ct.c_int]
    L.anacor_batch_autotune.restype = ct.c_int
    L.anacor_batch_autotune.argtypes = [ct.c_void_p, ct.c_int64]
    L.anacor_batch_info.restype = ct.c_int
    L.anacor_batch_info.argtypes = [ct.c_void_p, ct.POINTER(ct.c_int), ct.POINTER(ct.c_longlong),
                                    ct.POINTER(ct.c_int)]
    L.anacor_batch_destroy.restype = None
    L.anacor_batch_destroy.argtypes = [ct.c_void_p]
    # learned surrogate
    _vp, _int = ct.c_void_p, ct.c_int
    sigs = {
        "anacor_surrogate_create": (_vp, [_int, ct.c_uint32, ct.c_float]),
        "anacor_surrogate_destroy": (None, [_vp]),
        "anacor_surrogate_param_count": (ct.c_int64, []),
        "anacor_surrogate_members": (_int, [_vp]),
        "anacor_surrogate_params": (_int, [_vp, _f32p, _int]),
        "anacor_surrogate_fourier": (_int, [_vp, _f32p, _int]),
        "anacor_surrogate_scale": (_int, [_vp, ct.POINTER(ct.c_double), ct.POINTER(ct.c_double), _int]),
        "anacor_surrogate_inputs": (_int, [_f64p, _f64p, ct.c_int64, _f64p, _f64p, _f64p, _f32p]),
        "anacor_surrogate_inputs_device": (_int, [_vp, _vp, ct.c_int64, _f64p, _f64p, _f64p, _vp, _vp]),
        "anacor_surrogate_set_data": (_int, [_vp, _f32p, _f64p, ct.c_int64]),
        "anacor_surrogate_train": (_int, [_vp, _int, _int, ct.c_float, ct.c_float, _int, _vp]),
        "anacor_surrogate_gradients": (_int, [_vp, _f32p, _f32p, _int, _vp, _vp]),
        "anacor_surrogate_predict": (_int, [_vp, _f32p, ct.c_int64, _f32p, _f32p, _vp]),
        "anacor_surrogate_predict_device": (_int, [_vp, _vp, ct.c_int64, _vp, _vp, _vp, _vp]),
        "anacor_surrogate_audit_flags": (_int, [_vp, ct.c_int64, ct.c_uint32, ct.c_double, ct.c_float, _vp, _vp]),
        "anacor_surrogate_save": (_int, [_vp, ct.c_char_p]),
        "anacor_surrogate_load": (_int, [_vp, ct.c_char_p]),
        "anacor_tc_gemm_check": (_int, [_f32p, _f32p, _int, _int, _int, _int, _int, _f32p]),
    }
    # gridding (absorption map)
    sigs.update({
        "anacor_gridding_directions": (_int, [_int, _int, _f64p, _f64p, _f64p]),
        "anacor_gridding_create": (_vp, [_vp, _int, _int, _int]),
        "anacor_gridding_build": (_int, [_vp, _vp, _vp, _vp]),
        "anacor_gridding_info": (_int, [_vp, ct.POINTER(ct.c_int64), ct.POINTER(ct.c_int64), ct.POINTER(_int),
                                        ct.POINTER(_int)]),
        "anacor_gridding_axes": (_int, [_vp, _f64p, _f64p]),
        "anacor_gridding_device_map": (_vp, [_vp, ct.POINTER(ct.c_int64)]),
        "anacor_gridding_map": (_int, [_vp, _f32p]),
        "anacor_gridding_set_map": (_int, [_vp, _f32p]),
        "anacor_gridding_interpolate": (_int, [_vp, _f64p, _f64p, ct.c_int64, _f64p, _f64p, _f64p, _int, _f64p]),
        "anacor_gridding_interpolate_async": (_int, [_vp, _f64p, _f64p, ct.c_int64, _f64p, _f64p, _f64p, _int,
                                                     _vp, _vp]),
        "anacor_gridding_destroy": (None, [_vp]),
        "anacor_gridding_prepare": (_int, [_vp, _f64p, _f64p, ct.c_int64, _f64p, _f64p, _f64p, _int]),
        "anacor_gridding_run": (_int, [_vp, _vp, _vp]),
        # drop-ins, argtypes as AnACor/utils/utils_gridding.py:104-134 and :547-573
        "ray_tracing_single_gridding": (ct.c_double, [np.ctypeslib.ndpointer(dtype=np.int64),
                                                      np.ctypeslib.ndpointer(dtype=np.float64), ct.c_double,
                                                      ct.c_double, np.ctypeslib.ndpointer(dtype=np.float64),
                                                      np.ctypeslib.ndpointer(dtype=np.float64), _i8ppp,
                                                      np.ctypeslib.ndpointer(dtype=np.int64), _int, _int, _int]),
        "ib_single_gridding": (ct.c_double, [np.ctypeslib.ndpointer(dtype=np.int64),
                                             np.ctypeslib.ndpointer(dtype=np.float64), ct.c_double, ct.c_double,
                                             np.ctypeslib.ndpointer(dtype=np.float64),
                                             np.ctypeslib.ndpointer(dtype=np.float64), _i8ppp,
                                             np.ctypeslib.ndpointer(dtype=np.int64), _int, _int, _int, _int]),
        "nearest_neighbor_interpolate_overall": (ct.POINTER(ct.c_double), [
            ct.c_int64, ct.c_int64, np.ctypeslib.ndpointer(dtype=np.int64), ct.c_int64,
            np.ctypeslib.ndpointer(dtype=np.float64), np.ctypeslib.ndpointer(dtype=np.float64),
            np.ctypeslib.ndpointer(dtype=np.float64), np.ctypeslib.ndpointer(dtype=np.float64),
            np.ctypeslib.ndpointer(dtype=np.float64), ct.c_int64, np.ctypeslib.ndpointer(dtype=np.float64),
            np.ctypeslib.ndpointer(dtype=np.float64), _int, _int, np.ctypeslib.ndpointer(dtype=np.float64),
            np.ctypeslib.ndpointer(dtype=np.float64), np.ctypeslib.ndpointer(dtype=np.float64), ct.c_int64,
            ct.c_int64, ct.c_double, ct.c_double, ct.c_double, ct.c_double, _int]),
    })
    # GPU voxel sampling, bisection
    sigs.update({
        "anacor_plan_run_bisection": (_int, [_vp, _int, _vp]),
        "anacor_bisection": (_int, [_i8p, _i64p, _i64p, ct.c_int64, _f64p, _f64p, ct.c_int64, _f64p, _f64p, _f64p,
                                    _f64p, _f64p, _int, _f64p]),
        "anacor_plan_create_sampled": (_vp, [_i8p, _i64p, _int, _int, ct.c_int64, ct.c_double, _int, _f64p, _f64p,
                                             _int, _int]),
        "anacor_plan_n_voxels": (ct.c_int64, [_vp]),
        "anacor_plan_voxels": (_int, [_vp, _i64p]),
        "anacor_sample_voxels": (_int, [_i8p, _i64p, _int, _int, ct.c_int64, ct.c_double, _int, _vp, ct.c_int64,
                                        ct.POINTER(ct.c_int64)]),
    })
    for name, (res, args) in sigs.items():
        getattr(L, name).restype = res
        getattr(L, name).argtypes = args
    L.free.restype = None
    L.free.argtypes = [ct.c_void_p]
    if path == _build.LIB:
        _LIB = L
    return L


def last_error(L=None) -> tuple[int, str]:
    L = L or load()
    return int(L.anacor_last_status()), (L.anacor_last_error() or b"").decode()


def check(status: int, L=None) -> None:
    if status != 0:
        st, msg = last_error(L)
        raise AnacorError(status, msg)
