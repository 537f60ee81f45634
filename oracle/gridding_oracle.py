"""CPU restatement of the reference's gridding mode (test infrastructure only).

Follows, in numpy:
* the grid of ``mp_create_gridding`` and the directions and angles of
  ``worker_function_create_gridding`` (AnACor/utils/utils_gridding.py:140-152,
  270-276) with ``thetaphi_2_myframe`` / ``myframe_2_dials`` /
  ``dials_2_thetaphi`` (AnACor/utils/utils_rt.py:321-350, 483-503);
* the wrap padding and padded axes of ``mp_interpolation_gridding``
  (utils_gridding.py:408-440);
* ``nearest_neighbor_custom`` / ``nearest_neighbor_interpolate`` and the
  per-reflection loop of ``nearest_neighbor_interpolate_overall``
  (AnACor/src/gridding_interpolation.c:16-45, 100-163), and GSL's bilinear
  2-D interpolation (the published algorithm: bracketing index by bisection,
  then (1-t)(1-u) z00 + t(1-u) z10 + (1-t)u z01 + tu z11) for the reference's
  ``interpolate`` (:48-76).

The map values themselves come from the oracle's leg detail or from the
reference library's ``ray_tracing_single_gridding`` (oracle.Reference).
Only the tests use this module, as the checker.
"""
from __future__ import annotations

import numpy as np


def thetaphi_2_myframe(theta, phi):
    z = np.cos(theta) * np.sin(phi)
    x = -np.cos(theta) * np.cos(phi)
    y = -np.sin(theta)
    return np.array([z, y, x])


def myframe_2_dials(v):
    P = np.linalg.inv(np.array([[1, 0, 0], [0, 0, 1], [0, 1, 0]]))
    return P.dot(v)


def dials_2_thetaphi(v, L1=False):
    if L1:
        v = -v
    if v[1] == 0:
        theta = np.arctan(-v[2] / (-np.sqrt(v[0] ** 2 + v[1] ** 2) + 0.001))
        phi = np.arctan(-v[0] / (v[1] + 0.001))
    elif v[1] < 0:
        theta = np.arctan(-v[2] / np.sqrt(v[0] ** 2 + v[1] ** 2))
        phi = np.arctan(-v[0] / v[1])
    else:
        if v[2] < 0:
            theta = np.pi - np.arctan(-v[2] / np.sqrt(v[0] ** 2 + v[1] ** 2))
        else:
            theta = -np.pi - np.arctan(-v[2] / np.sqrt(v[0] ** 2 + v[1] ** 2))
        phi = -np.arctan(-v[0] / (-v[1]))
    return theta, phi


def directions(n_theta: int, n_phi: int):
    """(rotated_s1 [G][3], theta [G], phi [G]) of the reference's map rows."""
    tl = np.linspace(-180, 180, n_theta, endpoint=False)
    pl = np.linspace(-90, 90, n_phi, endpoint=False)
    tg, pg = np.meshgrid(tl, pl)
    data = np.stack((tg.ravel(), pg.ravel()), axis=-1) / 180 * np.pi
    s1 = np.array([myframe_2_dials(thetaphi_2_myframe(t, p)) for t, p in data])
    ang = np.array([dials_2_thetaphi(v) for v in s1])
    return s1, ang[:, 0].copy(), ang[:, 1].copy()


def padded(map_gn: np.ndarray, n_theta: int, n_phi: int):
    """The reference's interpolation input from a [G][N] map:
    (grid [N][len_phi][len_theta], theta_list, phi_list)."""
    n = map_gn.shape[1]
    g = map_gn.astype(np.float64).reshape((n_phi, n_theta, n))
    tp = int(np.round((g.shape[1] // 6) / 2))
    pp = int(np.round(g.shape[0] // 6 / 2))
    g = np.concatenate((g[:, -tp:, :], g, g[:, :tp, :]), axis=1)
    g = np.concatenate((g[-pp:, :, :], g, g[:pp, :, :]), axis=0)
    g = np.ascontiguousarray(np.transpose(g, (2, 0, 1)))
    len_t = int(n_theta + tp * 2)
    len_p = int(n_phi + pp * 2)
    tl = np.linspace(-np.round(180 * 7 / 6), np.round(180 * 7 / 6), len_t, endpoint=False) / 180 * np.pi
    pl = np.linspace(-np.round(90 * 7 / 6), np.round(90 * 7 / 6), len_p, endpoint=False) / 180 * np.pi
    return g, tl, pl


def _nearest(theta, phi, nx, ny, tmin, tmax, pmin, pmax):
    ts = (tmax - tmin) / (nx - 1)
    ps = (pmax - pmin) / (ny - 1)
    ti = int((theta - tmin) / ts)
    pi = int((phi - pmin) / ps)
    ti = min(max(ti, 0), nx - 1)
    pi = min(max(pi, 0), ny - 1)
    return ti, pi


def _bracket(xa, x):
    lo, hi = 0, len(xa) - 1
    while hi > lo + 1:
        mid = (hi + lo) // 2
        if xa[mid] > x:
            hi = mid
        else:
            lo = mid
    return lo


def _bilinear(grid, tl, pl, theta, phi):
    """GSL bilinear value of every voxel's grid at (theta, phi): [N]."""
    xi, yi = _bracket(tl, theta), _bracket(pl, phi)
    t = (theta - tl[xi]) / (tl[xi + 1] - tl[xi])
    u = (phi - pl[yi]) / (pl[yi + 1] - pl[yi])
    z00, z10 = grid[:, yi, xi], grid[:, yi, xi + 1]
    z01, z11 = grid[:, yi + 1, xi], grid[:, yi + 1, xi + 1]
    return (1.0 - t) * (1.0 - u) * z00 + t * (1.0 - u) * z10 + (1.0 - t) * u * z01 + t * u * z11


def interpolate(grid, tl, pl, rotated_xray, rotated_s1, method: int = 1) -> float:
    """A_h of one reflection from the padded map (method 1 nearest, 2 bilinear);
    angles with the reference C's dials_2_thetaphi_22 are passed in through the
    rotated vectors and computed here with the same formulas."""
    th2, ph2 = dials_2_thetaphi(np.asarray(rotated_s1, dtype=np.float64))
    th1, ph1 = dials_2_thetaphi(np.asarray(rotated_xray, dtype=np.float64), L1=True)
    ny, nx = grid.shape[1], grid.shape[2]
    if method == 1:
        a = _nearest(th1, ph1, nx, ny, tl.min(), tl.max(), pl.min(), pl.max())
        b = _nearest(th2, ph2, nx, ny, tl.min(), tl.max(), pl.min(), pl.max())
        z1 = grid[:, a[1], a[0]]
        z2 = grid[:, b[1], b[0]]
    else:
        z1 = _bilinear(grid, tl, pl, th1, ph1)
        z2 = _bilinear(grid, tl, pl, th2, ph2)
    acc = 0.0
    for v in np.exp(-(z1 + z2)):
        acc += float(v)
    return acc / grid.shape[0]


def map_value(L_leg: np.ndarray, mu: np.ndarray, is_exp: int = 0) -> np.ndarray:
    """cal_rate with a zero incident leg, per voxel: float32 of
    mu_li L_li + mu_lo L_lo + mu_cr L_cr + mu_bu L_bu (left to right)."""
    L = np.asarray(L_leg, dtype=np.float64)
    a = ((mu[0] * (0.0 + L[:, 0]) + mu[1] * (0.0 + L[:, 1])) + mu[2] * (0.0 + L[:, 2])) + mu[3] * (0.0 + L[:, 3])
    return (np.exp(-a) if is_exp else a).astype(np.float32)


__all__ = ["directions", "padded", "interpolate", "map_value", "dials_2_thetaphi"]
