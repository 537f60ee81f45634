"""Gridding (absorption-map) mode on the GPU.

The reference's approximate accelerator (AnACor/utils/utils_gridding.py):
build once, for every direction of a (theta, phi) grid (360 x 180 by
default) and every crystal voxel, the diffracted leg's sum_m mu_m L_m; then
each reflection's A_h is a mean over voxels of exp(-(z_incident +
z_diffracted)) with z looked up in the map (nearest grid point by default,
or bilinear).

``GriddingMap(plan, n_theta, n_phi)``  the map of a plan's sample, built and
                                     kept on the GPU;
``directions(n_theta, n_phi)``       the grid rows (vector and polar angles).

A map can also be built from the caller's own per-direction vectors and
angles (the reference computes them with numpy), so that it reproduces a map
made from exactly those inputs.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _lib, tracer


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def directions(n_theta: int = 360, n_phi: int = 180):
    """(rotated_s1 [G][3], theta [G], phi [G]) of the grid rows, as the library
    generates them (row = i_phi * n_theta + i_theta)."""
    L = _lib.load()
    G = n_theta * n_phi
    s1 = np.zeros((G, 3))
    th = np.zeros(G)
    ph = np.zeros(G)
    _lib.check(L.anacor_gridding_directions(int(n_theta), int(n_phi), s1, th, ph), L)
    return s1, th, ph


class GriddingMap:
    """Absorption map of a plan's sample (the plan must outlive the map)."""

    def __init__(self, plan: tracer.Plan, n_theta: int = 360, n_phi: int = 180, method: int = 2):
        self._L = _lib.load()
        self.plan = plan
        h = self._L.anacor_gridding_create(plan._h, int(n_theta), int(n_phi), int(method))
        if not h:
            raise _lib.AnacorError(*_lib.last_error(self._L))
        self._h = ct.c_void_p(h)
        self.n_theta, self.n_phi, self.method = int(n_theta), int(n_phi), int(method)
        g, n, lt, lp = ct.c_int64(), ct.c_int64(), ct.c_int(), ct.c_int()
        _lib.check(self._L.anacor_gridding_info(self._h, ct.byref(g), ct.byref(n), ct.byref(lt), ct.byref(lp)),
                   self._L)
        self.n_dirs, self.n_vox, self.len_theta, self.len_phi = g.value, n.value, lt.value, lp.value

    def build(self, rotated_s1=None, theta=None, phi=None):
        """Build the map, from the library's grid or from explicit per-direction
        vectors and angles."""
        if rotated_s1 is None:
            _lib.check(self._L.anacor_gridding_build(self._h, None, None, None), self._L)
            return self
        s1 = _c(rotated_s1, np.float64).reshape(-1, 3)
        th = _c(theta, np.float64)
        ph = _c(phi, np.float64)
        if s1.shape[0] != self.n_dirs or th.shape[0] != self.n_dirs or ph.shape[0] != self.n_dirs:
            raise ValueError("one vector and one (theta, phi) per grid direction")
        _lib.check(self._L.anacor_gridding_build(self._h, s1.ctypes.data, th.ctypes.data, ph.ctypes.data),
                   self._L)
        return self

    def axes(self):
        """The padded interpolation axes (theta, phi), radians."""
        t = np.zeros(self.len_theta)
        p = np.zeros(self.len_phi)
        _lib.check(self._L.anacor_gridding_axes(self._h, t, p), self._L)
        return t, p

    def map(self) -> np.ndarray:
        """[n_dirs][n_vox] float32 in the caller's voxel order."""
        m = np.zeros((self.n_dirs, max(self.n_vox, 1)), dtype=np.float32)
        _lib.check(self._L.anacor_gridding_map(self._h, m), self._L)
        return m[:, :self.n_vox]

    def set_map(self, m: np.ndarray):
        m = _c(m, np.float32).reshape(self.n_dirs, self.n_vox)
        _lib.check(self._L.anacor_gridding_set_map(self._h, m), self._L)

    def device_map(self):
        """(device pointer, row stride in floats) of the map."""
        ld = ct.c_int64()
        p = self._L.anacor_gridding_device_map(self._h, ct.byref(ld))
        return int(p or 0), ld.value

    def interpolate(self, s1, omega, xray, omega_axis, F, method: str | int = "nearest") -> np.ndarray:
        m = {"nearest": 1, "linear": 2}.get(method, method)
        s1 = _c(s1, np.float64).reshape(-1, 3)
        n = s1.shape[0]
        out = np.zeros(max(n, 1))
        _lib.check(self._L.anacor_gridding_interpolate(self._h, s1, _c(omega, np.float64), n, _c(xray, np.float64),
                                                       _c(omega_axis, np.float64), _c(F, np.float64).reshape(-1),
                                                       int(m), out), self._L)
        return out[:n]

    def interpolate_async(self, s1, omega, xray, omega_axis, F, d_out: int, stream: int | None = None,
                          method: str | int = "nearest"):
        m = {"nearest": 1, "linear": 2}.get(method, method)
        s1 = _c(s1, np.float64).reshape(-1, 3)
        _lib.check(self._L.anacor_gridding_interpolate_async(self._h, s1, _c(omega, np.float64), s1.shape[0],
                                                             _c(xray, np.float64), _c(omega_axis, np.float64),
                                                             _c(F, np.float64).reshape(-1), int(m),
                                                             ct.c_void_p(d_out), ct.c_void_p(stream or 0)),
                   self._L)

    def prepare(self, s1, omega, xray, omega_axis, F, method: str | int = "nearest"):
        """Compute and keep on the device the lookups of these reflections."""
        m = {"nearest": 1, "linear": 2}.get(method, method)
        s1 = _c(s1, np.float64).reshape(-1, 3)
        _lib.check(self._L.anacor_gridding_prepare(self._h, s1, _c(omega, np.float64), s1.shape[0],
                                                   _c(xray, np.float64), _c(omega_axis, np.float64),
                                                   _c(F, np.float64).reshape(-1), int(m)), self._L)

    def run(self, d_out: int, stream: int | None = None):
        """Interpolation kernel over the prepared reflections into device d_out."""
        _lib.check(self._L.anacor_gridding_run(self._h, ct.c_void_p(d_out), ct.c_void_p(stream or 0)), self._L)

    def close(self):
        if getattr(self, "_h", None):
            self._L.anacor_gridding_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sample_map(s, n_theta: int = 360, n_phi: int = 180, method: int = 2, plan: tracer.Plan | None = None):
    """(plan, built map) of a synthetic sample."""
    p = plan or tracer.Plan(s.label, s.coords, s.voxel, s.mu)
    return p, GriddingMap(p, n_theta, n_phi, method).build()


__all__ = ["GriddingMap", "directions", "sample_map"]
