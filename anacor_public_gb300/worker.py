"""Host-side mirror of AnACor's worker layer for the absorption path.

``python_2_c_3d``   int8*** row table over a C-contiguous volume
                    (AnACor/utils/utils_os.py:45-68), built in one pass.
``kp_rotation``     Rodrigues matrix (AnACor/utils/utils_os.py:26-43).
``parse_reflections`` s1 vectors and rotation angles of reflection rows
                    (AnACor/utils/utils_mp.py:151-164) in one pass instead of
                    two ast.literal_eval calls per row.
``worker_function`` same arguments and outputs as the GPU/OpenMP branch of
                    AnACor/utils/utils_mp.py:39-212,418-432: parses ``s1`` and
                    the rotation angle of every selected reflection, calls
                    ``ray_tracing_overall`` of this library through ctypes and
                    writes ``{dataset}_refl_{up}.json`` / ``{dataset}_time_{up}.json``.
"""
from __future__ import annotations

import ctypes as ct
import json
import os
import time
from ast import literal_eval

import numpy as np

from . import _lib


def python_2_c_3d(label_list: np.ndarray):
    """Row-pointer table (int8***) over ``label_list``; returns (pointer, keep-alive)."""
    if label_list.dtype != np.int8 or not label_list.flags.c_contiguous:
        raise ValueError("label_list must be a C-contiguous int8 array")
    Z, Y, X = label_list.shape
    base = label_list.ctypes.data
    ptr_size = ct.sizeof(ct.c_void_p)
    rows = (ct.c_void_p * (Z * Y))()
    addr = base + np.arange(Z * Y, dtype=np.uint64) * np.uint64(X)
    ct.memmove(rows, addr.astype(np.uint64).tobytes(), Z * Y * ptr_size)
    planes = (ct.c_void_p * Z)()
    paddr = np.uint64(ct.addressof(rows)) + np.arange(Z, dtype=np.uint64) * np.uint64(Y * ptr_size)
    ct.memmove(planes, paddr.astype(np.uint64).tobytes(), Z * ptr_size)
    return ct.cast(planes, ct.POINTER(ct.POINTER(ct.POINTER(ct.c_int8)))), (rows, planes, label_list)


def kp_rotation(axis, theta):
    x, y, z = axis
    c, s = np.cos(theta), np.sin(theta)
    return np.array([[c + (x ** 2) * (1 - c), x * y * (1 - c) - z * s, y * s + x * z * (1 - c)],
                     [z * s + x * y * (1 - c), c + (y ** 2) * (1 - c), -x * s + y * z * (1 - c)],
                     [-y * s + x * z * (1 - c), x * s + y * z * (1 - c), c + (z ** 2) * (1 - c)]])


def ray_tracing_overall(label_list, coord_list, s1, omega, xray, omega_axis, F, voxel_size, coefficients,
                        full_iteration=0, store_paths=0, num_workers=1, is_exp=1, low=0):
    """Call the library's ray_tracing_overall as AnACor's worker does; returns A_h."""
    L = _lib.load()
    label_list = np.ascontiguousarray(label_list, dtype=np.int8)
    tab, keep = python_2_c_3d(label_list)
    n = len(omega)
    res = L.ray_tracing_overall(low, low + n, np.ascontiguousarray(coord_list, dtype=np.int64), len(coord_list),
                                np.ascontiguousarray(s1, dtype=np.float64), np.ascontiguousarray(omega, dtype=np.float64),
                                np.ascontiguousarray(xray, dtype=np.float64),
                                np.ascontiguousarray(omega_axis, dtype=np.float64),
                                np.ascontiguousarray(F, dtype=np.float64), n,
                                np.ascontiguousarray(voxel_size, dtype=np.float64),
                                np.ascontiguousarray(coefficients, dtype=np.float64), tab,
                                np.array(label_list.shape, dtype=np.int64), int(full_iteration), int(store_paths),
                                int(num_workers), int(is_exp))
    if not res:
        st, msg = _lib.last_error(L)
        raise _lib.AnacorError(st, msg)
    out = np.ctypeslib.as_array(res, shape=(n,)).copy() if n else np.zeros(0)
    L.free(ct.cast(res, ct.c_void_p))
    del keep
    return out


def _numbers(values, width: int) -> np.ndarray:
    """Rows of `width` numbers from their JSON/Python literal strings (or
    sequences) as float64.  Each number goes through float(), the conversion
    ast.literal_eval applies to a numeric literal, so the values are identical."""
    if not values:
        return np.zeros((0, width))
    if all(isinstance(v, str) for v in values):
        text = ",".join(values).translate(_STRIP)
        out = np.fromiter(map(float, text.split(",")), dtype=np.float64, count=len(values) * width)
        return out.reshape(-1, width)
    return np.array([literal_eval(v) if isinstance(v, str) else v for v in values], dtype=np.float64).reshape(
        -1, width)


_STRIP = str.maketrans("", "", "[]() \t\n")


def parse_reflections(selected_data, offset: float = 0.0):
    """(s1 [n][3], omega [n]) of reflection rows as the reference's worker
    reads them: s1 = row["s1"], omega = row["xyzobs.mm.value"][2] + offset
    (degrees) converted to radians (AnACor/utils/utils_mp.py:151-164)."""
    s1 = _numbers([row["s1"] for row in selected_data], 3)
    obs = _numbers([row["xyzobs.mm.value"] for row in selected_data], 3)
    omega = obs[:, 2] + offset / 180 * np.pi
    return s1, omega


def worker_function(t1, low, dataset, selected_data, label_list, voxel_size, coefficients, F, coord_list,
                    omega_axis, axes_data, save_dir, args, offset, full_iteration, store_paths, printing,
                    num_cls, logger):
    """Same contract as AnACor/utils/utils_mp.py:39 for the --gpu / --openmp branch."""
    xray = -np.array(axes_data[1]["direction"])
    up = low + len(selected_data)
    arr_scattering, arr_omega = parse_reflections(selected_data, offset)
    if logger is not None:
        logger.info("GB300 absorption path is used for ray tracing")
    corr = list(ray_tracing_overall(label_list, coord_list, arr_scattering, arr_omega, xray, omega_axis, F,
                                    voxel_size, coefficients, full_iteration, store_paths,
                                    getattr(args, "num_workers", 1), 1, low))
    t2 = time.time()
    with open(os.path.join(save_dir, "{}_refl_{}.json".format(dataset, up)), "w") as fz:
        json.dump(corr, fz, indent=2)
    with open(os.path.join(save_dir, "{}_time_{}.json".format(dataset, up)), "w") as f1:
        json.dump(t2 - t1, f1, indent=2)
    return corr
