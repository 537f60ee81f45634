"""ctypes access to the checker libraries (test infrastructure only).

* ``Oracle``     -- ``oracle/_build/liboracle.so``, the C restatement in
                    ``oracle/anacor_oracle.c``.  Available wherever gcc is.
* ``Reference``  -- ``oracle/_ref/ray_tracing_cpu.so``, the reference's own C
                    sources compiled by ``make -C oracle ref``.  Only where the
                    reference sources were present at build time.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, as the checker.  The product library never does.
"""
from __future__ import annotations

import contextlib
import ctypes as ct
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "ray_tracing_cpu.so")

_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i8p = np.ctypeslib.ndpointer(dtype=np.int8, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")

STATUS = {0: "ok", 1: "no exit face", 2: "face/angle assert", 3: "bad arguments", 4: "out of memory"}


def build_oracle(ref_src: str | None = None) -> None:
    """Build the C restatement; with ``ref_src`` (the reference checkout's
    ``AnACor/src`` directory) also the reference library from its sources."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref_src:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFSRC={os.path.abspath(ref_src)}"], check=True)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Oracle:
    """The C restatement; FP64 throughout, bit-exact with the reference."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        lib = ct.CDLL(path)
        lib.oracle_overall.restype = ct.c_int
        lib.oracle_overall.argtypes = [_i64p, ct.c_int64, _f64p, _f64p, _f64p, _f64p, _f64p, ct.c_int64,
                                       _f64p, _f64p, _i8p, _i64p, ct.c_int, ct.c_int, ct.c_int, _f64p]
        lib.oracle_single.restype = ct.c_int
        lib.oracle_single.argtypes = [_i64p, ct.c_int64, _f64p, _f64p, _f64p, _f64p, _i8p, _i64p,
                                      ct.c_int, ct.c_int, _f64p]
        lib.oracle_leg_detail.restype = ct.c_int
        lib.oracle_leg_detail.argtypes = [_i64p, ct.c_int64, _f64p, _f64p, _f64p, _i8p, _i64p, ct.c_int,
                                          _i64p, _i64p, _i64p, _i64p, _i64p, _f64p, _i32p]
        lib.oracle_rotate.restype = None
        lib.oracle_rotate.argtypes = [_f64p, ct.c_double, _f64p, _f64p, _f64p, _f64p, _f64p]
        lib.oracle_reflection_dirs.restype = None
        lib.oracle_reflection_dirs.argtypes = [_f64p, _f64p, _f64p]
        lib.oracle_ib.restype = ct.c_int
        lib.oracle_ib.argtypes = [_i64p, ct.c_int64, _f64p, _f64p, _f64p, _f64p, _i8p, _i64p, ct.c_int, _f64p,
                                  ct.c_void_p]
        lib.oracle_cube_face.restype = ct.c_int64
        lib.oracle_cube_face.argtypes = [_i64p, _f64p, _i64p, ct.c_int]
        lib.oracle_ib_gridding.restype = ct.c_int
        lib.oracle_ib_gridding.argtypes = [_i64p, ct.c_int64, _f64p, ct.c_double, ct.c_double, _f64p, _f64p, _i8p,
                                           _i64p, ct.c_int, ct.c_int, _f64p]
        self.lib = lib

    def ib_gridding(self, coords, rotated_s1, theta, phi, voxel, mu, label, num_cls=4, is_exp=0) -> np.ndarray:
        """ib_single_gridding's value for every voxel of `coords` and one
        direction: [n] doubles.  Raises on a status."""
        coords = _c(coords, np.int64).reshape(-1, 3)
        out = np.zeros(len(coords))
        st = self.lib.oracle_ib_gridding(coords, len(coords), _c(rotated_s1, np.float64), float(theta), float(phi),
                                         _c(voxel, np.float64), _c(mu, np.float64), _c(label, np.int8),
                                         np.array(label.shape, dtype=np.int64), int(num_cls), int(is_exp), out)
        if st:
            raise RuntimeError(f"oracle_ib_gridding: {STATUS.get(st, st)}")
        return out

    def overall(self, s, threads: int = 0, full_iteration: int = 0, is_exp: int = 1) -> np.ndarray:
        out = np.zeros(s.n_refl, dtype=np.float64)
        st = self.lib.oracle_overall(_c(s.coords, np.int64), len(s.coords), _c(s.s1, np.float64),
                                     _c(s.omega, np.float64), _c(s.xray, np.float64), _c(s.omega_axis, np.float64),
                                     _c(s.F, np.float64), s.n_refl, _c(s.voxel, np.float64), _c(s.mu, np.float64),
                                     _c(s.label, np.int8), _c(s.shape, np.int64), full_iteration, is_exp,
                                     threads, out)
        if st:
            raise RuntimeError(f"oracle_overall: {STATUS.get(st, st)}")
        return out

    def rotate(self, s, i: int):
        xr = np.zeros(3)
        sr = np.zeros(3)
        self.lib.oracle_rotate(_c(s.omega_axis, np.float64), float(s.omega[i]), _c(s.F, np.float64),
                               _c(s.xray, np.float64), _c(s.s1[i], np.float64), xr, sr)
        return xr, sr

    def reflection_dirs(self, s1_rot, xray_rot) -> np.ndarray:
        out = np.zeros(10)
        self.lib.oracle_reflection_dirs(_c(s1_rot, np.float64), _c(xray_rot, np.float64), out)
        return out

    def single(self, coords, s1_rot, xray_rot, voxel, mu, label, full_iteration=0, is_exp=1) -> float:
        out = np.zeros(1)
        st = self.lib.oracle_single(_c(coords, np.int64), len(coords), _c(s1_rot, np.float64),
                                    _c(xray_rot, np.float64), _c(voxel, np.float64), _c(mu, np.float64),
                                    _c(label, np.int8), np.array(label.shape, dtype=np.int64),
                                    full_iteration, is_exp, out)
        if st:
            raise RuntimeError(f"oracle_single: {STATUS.get(st, st)}")
        return float(out[0])

    def ib(self, coords, s1_rot, xray_rot, voxel, mu, label, num_cls=4, lengths=False):
        """ib_test's A_h (bisection paths) of one reflection; with lengths, also
        the per-voxel [n][2][4] lengths.  Raises on a status."""
        n = len(coords)
        out = np.zeros(1)
        L = np.zeros((n, 2, 4)) if lengths else None
        st = self.lib.oracle_ib(_c(coords, np.int64), n, _c(s1_rot, np.float64), _c(xray_rot, np.float64),
                                _c(voxel, np.float64), _c(mu, np.float64), _c(label, np.int8),
                                np.array(label.shape, dtype=np.int64), int(num_cls), out,
                                L.ctypes.data if L is not None else None)
        if st:
            raise RuntimeError(f"oracle_ib: {STATUS.get(st, st)}")
        return (float(out[0]), L) if lengths else float(out[0])

    def leg_detail(self, coords, s1_rot, xray_rot, voxel, label, full_iteration=0) -> dict:
        n = len(coords)
        face = np.zeros((n, 2), np.int64)
        ln = np.zeros((n, 2), np.int64)
        nseg = np.zeros((n, 2), np.int64)
        first = np.zeros((n, 2, 3), np.int64)
        last = np.zeros((n, 2, 3), np.int64)
        L = np.zeros((n, 2, 4), np.float64)
        status = np.zeros((n, 2), np.int32)
        st = self.lib.oracle_leg_detail(_c(coords, np.int64), n, _c(s1_rot, np.float64), _c(xray_rot, np.float64),
                                        _c(voxel, np.float64), _c(label, np.int8),
                                        np.array(label.shape, dtype=np.int64), full_iteration,
                                        face, ln, nseg, first, last, L, status)
        if st:
            raise RuntimeError(f"oracle_leg_detail: {STATUS.get(st, st)}")
        return dict(face=face, len=ln, nseg=nseg, first=first, last=last, L=L, status=status)


# ---------------------------------------------------------------- reference

class _Path2(ct.Structure):
    # Path2_c, AnACor/src/ray_tracing.h:41-49
    _fields_ = [("ray", ct.POINTER(ct.c_int64)), ("posi", ct.POINTER(ct.c_int64)),
                ("classes", ct.POINTER(ct.c_int64)), ("len_path_2", ct.c_int64),
                ("len_classes_posi", ct.c_int64), ("len_classes", ct.c_int64)]


class _ThetaPhi(ct.Structure):
    _fields_ = [("theta", ct.c_double), ("phi", ct.c_double)]


def row_table(label: np.ndarray):
    """int8*** row-pointer table over a C-contiguous volume, as
    ``AnACor/utils/utils_os.py:45-68`` builds it (vectorised)."""
    assert label.flags.c_contiguous and label.dtype == np.int8
    Z, Y, X = label.shape
    base = label.ctypes.data
    rows = (ct.c_void_p * (Z * Y))(*[base + (z * Y + y) * X for z in range(Z) for y in range(Y)])
    planes = (ct.c_void_p * Z)(*[ct.addressof(rows) + z * Y * ct.sizeof(ct.c_void_p) for z in range(Z)])
    ptr = ct.cast(planes, ct.POINTER(ct.POINTER(ct.POINTER(ct.c_int8))))
    return ptr, (rows, planes, label)


@contextlib.contextmanager
def silence_stdout():
    """The reference printf()s once per reflection; send fd 1 to /dev/null."""
    import sys
    sys.stdout.flush()
    saved = os.dup(1)
    devnull = os.open(os.devnull, os.O_WRONLY)
    try:
        os.dup2(devnull, 1)
        yield
    finally:
        try:
            ct.CDLL(None).fflush(None)
        except Exception:
            pass
        os.dup2(saved, 1)
        os.close(saved)
        os.close(devnull)


class Reference:
    """The reference C library built from its own sources (``make -C oracle ref``)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = ct.CDLL(path)
        # argtypes as AnACor/utils/utils_mp.py:59-79
        lib.ray_tracing_overall.restype = ct.POINTER(ct.c_double)
        lib.ray_tracing_overall.argtypes = [ct.c_int64, ct.c_int64, _i64p, ct.c_int64, _f64p, _f64p, _f64p, _f64p,
                                            _f64p, ct.c_int64, _f64p, _f64p,
                                            ct.POINTER(ct.POINTER(ct.POINTER(ct.c_int8))), _i64p, ct.c_int,
                                            ct.c_int, ct.c_int, ct.c_int]
        lib.ray_tracing_single.restype = ct.c_double
        lib.ray_tracing_single.argtypes = [_i64p, ct.c_int64, _f64p, _f64p, _f64p, _f64p,
                                           ct.POINTER(ct.POINTER(ct.POINTER(ct.c_int8))), _i64p, ct.c_int,
                                           ct.c_int64, ct.c_int]
        lib.cube_face.restype = ct.c_int64
        lib.cube_face.argtypes = [_i64p, _f64p, _i64p, ct.c_int]
        lib.cal_coord.restype = _Path2
        lib.cal_coord.argtypes = [ct.c_double, ct.c_double, _i64p, ct.c_int64, _i64p,
                                  ct.POINTER(ct.POINTER(ct.POINTER(ct.c_int8))), ct.c_int64]
        lib.cal_path2_plus.restype = ct.POINTER(ct.c_double)
        lib.cal_path2_plus.argtypes = [_Path2, _f64p]
        lib.dials_2_thetaphi_22.restype = _ThetaPhi
        lib.dials_2_thetaphi_22.argtypes = [_f64p, ct.c_int64]
        lib.dials_2_myframe.restype = None
        lib.dials_2_myframe.argtypes = [_f64p, _f64p]
        lib.ray_tracing_single_gridding.restype = ct.c_double
        lib.ray_tracing_single_gridding.argtypes = [_i64p, _f64p, ct.c_double, ct.c_double, _f64p, _f64p,
                                                    ct.POINTER(ct.POINTER(ct.POINTER(ct.c_int8))), _i64p, ct.c_int,
                                                    ct.c_int, ct.c_int]
        lib.ib_single_gridding.restype = ct.c_double
        lib.ib_single_gridding.argtypes = [_i64p, _f64p, ct.c_double, ct.c_double, _f64p, _f64p,
                                           ct.POINTER(ct.POINTER(ct.POINTER(ct.c_int8))), _i64p, ct.c_int, ct.c_int,
                                           ct.c_int, ct.c_int]
        lib.ib_test.restype = ct.c_double
        lib.ib_test.argtypes = [_i64p, ct.c_int64, _f64p, _f64p, _f64p, _f64p,
                                ct.POINTER(ct.POINTER(ct.POINTER(ct.c_int8))), _i64p, ct.c_int, ct.c_int64,
                                ct.c_int]
        lib.free.argtypes = [ct.c_void_p]
        self.lib = lib

    def ib_test(self, coords, s1_rot, xray_rot, voxel, mu, label, num_cls=4) -> float:
        """ib_test (AnACor/src/ray_tracing.c:25-163), bisection paths."""
        label = _c(label, np.int8)
        tab, keep = row_table(label)
        with silence_stdout():
            r = self.lib.ib_test(_c(coords, np.int64), len(coords), _c(s1_rot, np.float64).copy(),
                                 _c(xray_rot, np.float64).copy(), _c(voxel, np.float64), _c(mu, np.float64), tab,
                                 np.array(label.shape, dtype=np.int64), 0, 0, int(num_cls))
        del keep
        return float(r)

    def single_gridding(self, coords, rotated_s1, theta, phi, voxel, mu, label, full_iteration=0, is_exp=0):
        """ray_tracing_single_gridding (AnACor/src/ray_tracing.c:484-534) for
        every voxel of `coords` and one direction: [n] doubles."""
        label = _c(label, np.int8)
        tab, keep = row_table(label)
        shape = np.array(label.shape, dtype=np.int64)
        out = np.empty(len(coords))
        s = _c(rotated_s1, np.float64)
        for k, c in enumerate(_c(coords, np.int64)):
            out[k] = self.lib.ray_tracing_single_gridding(np.ascontiguousarray(c), s.copy(), float(theta),
                                                          float(phi), _c(voxel, np.float64), _c(mu, np.float64),
                                                          tab, shape, full_iteration, 0, is_exp)
        del keep
        return out

    def ib_single_gridding(self, coords, rotated_s1, theta, phi, voxel, mu, label, num_cls=4, is_exp=0):
        """ib_single_gridding (AnACor/src/ray_tracing.c:427-482) for every
        voxel of `coords` and one direction: [n] doubles."""
        label = _c(label, np.int8)
        tab, keep = row_table(label)
        shape = np.array(label.shape, dtype=np.int64)
        out = np.empty(len(coords))
        s = _c(rotated_s1, np.float64)
        with silence_stdout():
            for k, c in enumerate(_c(coords, np.int64)):
                out[k] = self.lib.ib_single_gridding(np.ascontiguousarray(c), s.copy(), float(theta), float(phi),
                                                     _c(voxel, np.float64), _c(mu, np.float64), tab, shape, 0, 0,
                                                     int(num_cls), is_exp)
        del keep
        return out

    def overall(self, s, num_workers: int = 1, full_iteration: int = 0) -> np.ndarray:
        label = _c(s.label, np.int8)
        tab, keep = row_table(label)
        n = s.n_refl
        with silence_stdout():
            res = self.lib.ray_tracing_overall(0, n, _c(s.coords, np.int64), len(s.coords), _c(s.s1, np.float64),
                                               _c(s.omega, np.float64), _c(s.xray, np.float64),
                                               _c(s.omega_axis, np.float64), _c(s.F, np.float64), n,
                                               _c(s.voxel, np.float64), _c(s.mu, np.float64), tab,
                                               _c(s.shape, np.int64), full_iteration, 0, num_workers, 1)
        out = np.array([res[i] for i in range(n)], dtype=np.float64)
        self.lib.free(ct.cast(res, ct.c_void_p))
        del keep
        return out

    def single(self, coords, s1_rot, xray_rot, voxel, mu, label, full_iteration=0) -> float:
        label = _c(label, np.int8)
        tab, keep = row_table(label)
        with silence_stdout():
            r = self.lib.ray_tracing_single(_c(coords, np.int64), len(coords), _c(s1_rot, np.float64),
                                            _c(xray_rot, np.float64), _c(voxel, np.float64), _c(mu, np.float64),
                                            tab, np.array(label.shape, dtype=np.int64), full_iteration, 0, 1)
        del keep
        return float(r)

    def leg_detail(self, coords, s1_rot, xray_rot, voxel, label, full_iteration=0) -> dict:
        """Per-voxel cube_face -> cal_coord -> cal_path2_plus through the
        reference's exported primitives (the sequence of ray_tracing.c:199-266).
        The caller must pass only voxels the oracle accepts: the reference
        aborts the process on an assert."""
        label = _c(label, np.int8)
        tab, keep = row_table(label)
        shape = np.array(label.shape, dtype=np.int64)
        a_in = _c(xray_rot, np.float64).copy()
        a_out = _c(s1_rot, np.float64).copy()
        tp_out = self.lib.dials_2_thetaphi_22(a_out, 0)
        tp_in = self.lib.dials_2_thetaphi_22(a_in, 1)
        d_in = np.zeros(3)
        d_out = np.zeros(3)
        self.lib.dials_2_myframe(_c(xray_rot, np.float64).copy(), d_in)
        self.lib.dials_2_myframe(_c(s1_rot, np.float64).copy(), d_out)
        n = len(coords)
        res = dict(face=np.zeros((n, 2), np.int64), len=np.zeros((n, 2), np.int64),
                   nseg=np.zeros((n, 2), np.int64), first=np.zeros((n, 2, 3), np.int64),
                   last=np.zeros((n, 2, 3), np.int64), L=np.zeros((n, 2, 4)))
        for k in range(n):
            c = _c(coords[k], np.int64).copy()
            for leg, (d, tp, inc) in enumerate(((d_in, tp_in, 1), (d_out, tp_out, 0))):
                f = self.lib.cube_face(c, d, shape, inc)
                p = self.lib.cal_coord(tp.theta, tp.phi, c, f, shape, tab, full_iteration)
                L = self.lib.cal_path2_plus(p, _c(voxel, np.float64))
                res["face"][k, leg] = f
                res["len"][k, leg] = p.len_path_2
                res["nseg"][k, leg] = p.len_classes_posi
                if p.len_path_2 > 1:
                    res["first"][k, leg] = [p.ray[0], p.ray[1], p.ray[2]]
                    m = 3 * (p.len_path_2 - 1)
                    res["last"][k, leg] = [p.ray[m], p.ray[m + 1], p.ray[m + 2]]
                res["L"][k, leg] = [L[0], L[1], L[2], L[3]]
                for ptr in (p.ray, p.posi, p.classes, L):
                    self.lib.free(ct.cast(ptr, ct.c_void_p))
        del keep
        return res
