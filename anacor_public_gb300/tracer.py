"""Python front end of the GPU absorption path (numpy in, numpy out).

``absorption(...)``   one-shot A_h for a sample (uploads, runs, downloads);
``Plan``              device-resident sample for repeated or timed runs;
``batch_run(plans)``  one persistent launch over several samples;
``leg_detail(...)``   per-voxel march detail of one reflection (parity checks);
``rotated_vectors``   the host set-up's rotated incident / diffracted vectors.

All compute happens in libanacor_gb300.so on the current CUDA device.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def absorption(label, coords, s1, omega, xray, omega_axis, F, voxel, mu, full_iteration=0, is_exp=1):
    L = _lib.load()
    label = _c(label, np.int8)
    s1 = _c(s1, np.float64).reshape(-1, 3)
    n = s1.shape[0]
    out = np.zeros(max(n, 1), dtype=np.float64)
    st = L.anacor_absorption(label, np.array(label.shape, dtype=np.int64), _c(coords, np.int64).reshape(-1, 3),
                             len(coords), s1, _c(omega, np.float64), n, _c(xray, np.float64),
                             _c(omega_axis, np.float64), _c(F, np.float64).reshape(-1), _c(voxel, np.float64),
                             _c(mu, np.float64), int(full_iteration), int(is_exp), out)
    _lib.check(st, L)
    return out[:n]


def bisection(label, coords, s1, omega, xray, omega_axis, F, voxel, mu, num_cls=4):
    """A_h of every reflection with bisection paths (the reference's ib_test)."""
    L = _lib.load()
    label = _c(label, np.int8)
    s1 = _c(s1, np.float64).reshape(-1, 3)
    n = s1.shape[0]
    out = np.zeros(max(n, 1), dtype=np.float64)
    st = L.anacor_bisection(label, np.array(label.shape, dtype=np.int64), _c(coords, np.int64).reshape(-1, 3),
                            len(coords), s1, _c(omega, np.float64), n, _c(xray, np.float64),
                            _c(omega_axis, np.float64), _c(F, np.float64).reshape(-1), _c(voxel, np.float64),
                            _c(mu, np.float64), int(num_cls), out)
    _lib.check(st, L)
    return out[:n]


def sample_absorption(s, **kw):
    return absorption(s.label, s.coords, s.s1, s.omega, s.xray, s.omega_axis, s.F, s.voxel, s.mu, **kw)


class Plan:
    """A sample resident in device memory: volume, voxel list, reflection tables."""

    def __init__(self, label, coords, voxel, mu, full_iteration=0, is_exp=1):
        self._L = _lib.load()
        label = _c(label, np.int8)
        self.shape = label.shape
        self.n_vox = len(coords)
        h = self._L.anacor_plan_create(label, np.array(label.shape, dtype=np.int64),
                                       _c(coords, np.int64).reshape(-1, 3), len(coords), _c(voxel, np.float64),
                                       _c(mu, np.float64), int(full_iteration), int(is_exp))
        if not h:
            st, msg = _lib.last_error(self._L)
            raise _lib.AnacorError(st, msg)
        self._h = ct.c_void_p(h)
        self.n_refl = 0

    @classmethod
    def from_volume(cls, label, voxel, mu, crystal_code: int = 3, method: str = "all", sampling_size: int = 5000,
                    sampling_ratio: float | None = None, stride: int = 1, full_iteration=0, is_exp=1):
        """A plan whose crystal-voxel list is chosen on the GPU from the volume
        (uploaded once): method "all", "even" (the reference's default
        sampling) or "stride" (z, y, x multiples of `stride`)."""
        self = cls.__new__(cls)
        self._L = _lib.load()
        label = _c(label, np.int8)
        self.shape = label.shape
        m = {"all": 0, "even": 1, "stride": 2}[method]
        h = self._L.anacor_plan_create_sampled(label, np.array(label.shape, dtype=np.int64), int(crystal_code), m,
                                               int(sampling_size), float(sampling_ratio or 0.0), int(stride),
                                               _c(voxel, np.float64), _c(mu, np.float64), int(full_iteration),
                                               int(is_exp))
        if not h:
            st, msg = _lib.last_error(self._L)
            raise _lib.AnacorError(st, msg)
        self._h = ct.c_void_p(h)
        self.n_vox = int(self._L.anacor_plan_n_voxels(self._h))
        self.n_refl = 0
        return self

    def voxels(self) -> np.ndarray:
        """The plan's voxel list [n][3] int64 (z, y, x)."""
        out = np.zeros((max(self.n_vox, 1), 3), dtype=np.int64)
        _lib.check(self._L.anacor_plan_voxels(self._h, out), self._L)
        return out[:self.n_vox]

    @classmethod
    def from_sample(cls, s, **kw):
        p = cls(s.label, s.coords, s.voxel, s.mu, **kw)
        p.set_reflections(s.s1, s.omega, s.xray, s.omega_axis, s.F)
        return p

    def set_reflections(self, s1, omega, xray, omega_axis, F):
        s1 = _c(s1, np.float64).reshape(-1, 3)
        st = self._L.anacor_plan_set_reflections(self._h, s1, _c(omega, np.float64), s1.shape[0],
                                                 _c(xray, np.float64), _c(omega_axis, np.float64),
                                                 _c(F, np.float64).reshape(-1))
        _lib.check(st, self._L)
        self.n_refl = s1.shape[0]

    def run(self, stream: int | None = None):
        """Enqueue the march on `stream` (a raw cudaStream_t handle) or the plan's own stream."""
        _lib.check(self._L.anacor_plan_run(self._h, ct.c_void_p(stream or 0)), self._L)

    def run_bisection(self, num_cls: int = 4, stream: int | None = None):
        """Enqueue the bisection variant (the reference's ib_test per reflection)."""
        _lib.check(self._L.anacor_plan_run_bisection(self._h, int(num_cls), ct.c_void_p(stream or 0)), self._L)

    def result(self, stream: int | None = None) -> np.ndarray:
        out = np.zeros(max(self.n_refl, 1), dtype=np.float64)
        _lib.check(self._L.anacor_plan_result(self._h, out, ct.c_void_p(stream or 0)), self._L)
        return out[:self.n_refl]

    def device_result_ptr(self) -> int:
        return int(self._L.anacor_plan_device_result(self._h) or 0)

    def count_steps(self) -> int:
        """Sum of len_path_2 over every ray (one extra run with counting on)."""
        n = ct.c_uint64()
        _lib.check(self._L.anacor_plan_count_steps(self._h, ct.byref(n)), self._L)
        return int(n.value)

    def configure(self, variant: int = 0, tile: int = 0, order: int = -1):
        """Execution parameters.  variant: 1..4 the warp-cooperative march
        compiled for 1..4 CTAs per SM, 5..8 the march on the chessboard distance
        field, 9..12 on the 8 octant fields, 13..16 on the octant fields stored
        in 4x4x4 bricks (fields need labels in 0..7), 0 the process default; tile: voxels per work item (0 unchanged); order: voxel
        order (0 the caller's, 1 Morton, 2..7 blocked, -1 unchanged).  Results
        do not depend on them beyond the FP32 summation order of A_h."""
        _lib.check(self._L.anacor_plan_configure(self._h, int(variant), int(tile), int(order)), self._L)

    def config(self) -> dict:
        v, t, m = ct.c_int(), ct.c_int(), ct.c_int()
        _lib.check(self._L.anacor_plan_config(self._h, ct.byref(v), ct.byref(t), ct.byref(m)), self._L)
        return {"variant": v.value, "tile": t.value, "order": m.value}

    def autotune(self, sample_refl: int = 0) -> float:
        """Pick the fastest (variant, tile, order) on a reflection sample; returns
        the estimated ms for all reflections."""
        ms = ct.c_float()
        _lib.check(self._L.anacor_plan_autotune(self._h, int(sample_refl), ct.byref(ms)), self._L)
        return float(ms.value)

    def launch_info(self):
        g, k = ct.c_int(), ct.c_int()
        _lib.check(self._L.anacor_plan_launch_info(self._h, ct.byref(g), ct.byref(k)), self._L)
        return g.value, k.value

    def close(self):
        if getattr(self, "_h", None):
            self._L.anacor_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Several plans in one persistent launch; optionally captured in a CUDA graph."""

    def __init__(self, plans):
        self._L = _lib.load()
        self.plans = list(plans)
        arr = (ct.c_void_p * len(self.plans))(*[p._h.value for p in self.plans])
        h = self._L.anacor_batch_create(arr, len(self.plans))
        if not h:
            st, msg = _lib.last_error(self._L)
            raise _lib.AnacorError(st, msg)
        self._h = ct.c_void_p(h)

    def configure(self, variant: int = 0):
        """Variant of the whole launch (as Plan.configure): 1..4 every sample
        on the cooperative march, 5..16 every sample on its field of that kind
        (one launch; samples whose labels allow no field run in a second,
        cooperative one)."""
        _lib.check(self._L.anacor_batch_configure(self._h, int(variant)), self._L)

    def autotune(self, sample_refl: int = 0):
        _lib.check(self._L.anacor_batch_autotune(self._h, int(sample_refl)), self._L)

    def launch(self, stream: int | None = None):
        _lib.check(self._L.anacor_batch_launch(self._h, ct.c_void_p(stream or 0)), self._L)

    def capture(self, stream: int):
        """Capture one launch into a CUDA graph (needs a non-default stream)."""
        _lib.check(self._L.anacor_batch_capture(self._h, ct.c_void_p(stream)), self._L)

    def replay(self, stream: int | None = None):
        _lib.check(self._L.anacor_batch_replay(self._h, ct.c_void_p(stream or 0)), self._L)

    def wait(self, stream: int | None = None):
        _lib.check(self._L.anacor_batch_wait(self._h, ct.c_void_p(stream or 0)), self._L)

    def info(self) -> dict:
        g, n, v = ct.c_int(), ct.c_longlong(), ct.c_int()
        _lib.check(self._L.anacor_batch_info(self._h, ct.byref(g), ct.byref(n), ct.byref(v)), self._L)
        return {"grid": g.value, "items": n.value, "variant": v.value,
                "kernels": int(self._L.anacor_batch_kernels(self._h))}

    def results(self, stream: int | None = None):
        return [p.result(stream) for p in self.plans]

    def close(self):
        if getattr(self, "_h", None):
            self._L.anacor_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_run(plans, stream: int | None = None):
    L = _lib.load()
    arr = (ct.c_void_p * len(plans))(*[p._h.value for p in plans])
    _lib.check(L.anacor_batch_run(arr, len(plans), ct.c_void_p(stream or 0)), L)


def choose_stride(label, voxel, mu, s1, omega, xray, omega_axis, F, strides=(2, 4, 8), tol: float = 1e-3,
                  sample_refl: int = 64, crystal_code: int = 3) -> dict:
    """Crystal-voxel sampling stride of a sample, chosen by what it costs in A_h.

    The stride changes the answer, not only the speed, so it is chosen
    against the every-voxel result: on the first `sample_refl` reflections
    each candidate stride (the z, y, x multiples-of-stride lattice, sampled
    on the GPU) is run and compared with stride 1; the largest stride whose
    maximum relative deviation stays within `tol` wins (1 when none does).
    Returns {"stride", "tol", "candidates": {stride: {"voxels", "ms_per_refl",
    "median_dev", "max_dev"}}}."""
    import time
    k = min(int(sample_refl), len(omega))
    s1 = _c(s1, np.float64).reshape(-1, 3)[:k]
    omega = _c(omega, np.float64)[:k]
    res, base = {}, None
    for st in (1,) + tuple(int(x) for x in strides):
        p = Plan.from_volume(label, voxel, mu, crystal_code, method="stride" if st > 1 else "all", stride=st)
        try:
            if p.n_vox == 0:
                continue
            p.set_reflections(s1, omega, xray, omega_axis, F)
            p.run()
            a = p.result()
            t0 = time.perf_counter()
            p.run()
            a = p.result()
            ms = (time.perf_counter() - t0) * 1e3 / max(k, 1)
        finally:
            p.close()
        if st == 1:
            base = a
            res[1] = {"voxels": int(p.n_vox), "ms_per_refl": ms, "median_dev": 0.0, "max_dev": 0.0}
            continue
        dev = np.abs(a - base) / np.abs(base)
        res[st] = {"voxels": int(p.n_vox), "ms_per_refl": ms, "median_dev": float(np.median(dev)),
                   "max_dev": float(np.max(dev))}
    ok = [st for st, r in res.items() if st > 1 and r["max_dev"] <= tol]
    return {"stride": max(ok) if ok else 1, "tol": float(tol), "candidates": res}


def sample_voxels(label, crystal_code: int = 3, method: str = "all", sampling_size: int = 5000,
                  sampling_ratio: float | None = None, stride: int = 1) -> np.ndarray:
    """Crystal-voxel list of a volume selected on the GPU (see Plan.from_volume)."""
    p = Plan.from_volume(label, np.ones(3), np.zeros(4), crystal_code, method, sampling_size, sampling_ratio, stride)
    try:
        return p.voxels()
    finally:
        p.close()


def rotated_vectors(omega_axis, omega, F, xray, s1):
    L = _lib.load()
    s1 = _c(s1, np.float64).reshape(-1, 3)
    n = s1.shape[0]
    rx = np.zeros((max(n, 1), 3))
    rs = np.zeros((max(n, 1), 3))
    _lib.check(L.anacor_rotated_vectors(_c(omega_axis, np.float64), _c(omega, np.float64),
                                        _c(F, np.float64).reshape(-1), _c(xray, np.float64), s1, n, rx, rs), L)
    return rx[:n], rs[:n]


def leg_detail(label, coords, s1_rot, xray_rot, voxel, full_iteration=0) -> dict:
    L = _lib.load()
    label = _c(label, np.int8)
    coords = _c(coords, np.int64).reshape(-1, 3)
    n = len(coords)
    m = max(n, 1)
    face = np.zeros((m, 2), np.int32)
    ln = np.zeros((m, 2), np.int32)
    nseg = np.zeros((m, 2), np.int32)
    first = np.zeros((m, 2, 3), np.int32)
    last = np.zeros((m, 2, 3), np.int32)
    Ls = np.zeros((m, 2, 4), np.float64)
    status = np.zeros((m, 2), np.int32)
    st = L.anacor_leg_detail(label, np.array(label.shape, dtype=np.int64), coords, n, _c(s1_rot, np.float64),
                             _c(xray_rot, np.float64), _c(voxel, np.float64), int(full_iteration), face, ln, nseg,
                             first, last, Ls, status)
    _lib.check(st, L)
    return dict(face=face[:n], len=ln[:n], nseg=nseg[:n], first=first[:n], last=last[:n], L=Ls[:n],
                status=status[:n])


def distance_field(label) -> np.ndarray:
    """The packed distance field that kernel variants 5..8 march on:
    (label & 7) | (min(D, 31) << 3) per voxel, D the chessboard distance to the
    nearest voxel with another label, 0 for label-0 voxels."""
    L = _lib.load()
    label = _c(label, np.int8)
    out = np.zeros(label.shape, np.uint8)
    _lib.check(L.anacor_distance_field(label, np.array(label.shape, dtype=np.int64), out), L)
    return out


def octant_fields(label) -> np.ndarray:
    """The 8 octant fields of kernel variants 9..12, [octant][Z][Y][X] uint8:
    (label & 7) | (min(r + 1, 31) << 3), r the largest corner box toward the
    octant's signs (octant = (sx<0) | (sy<0)<<1 | (sz<0)<<2) holding one label."""
    L = _lib.load()
    label = _c(label, np.int8)
    out = np.zeros((8,) + label.shape, np.uint8)
    _lib.check(L.anacor_octant_fields(label, np.array(label.shape, dtype=np.int64), out), L)
    return out
