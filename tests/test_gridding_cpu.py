"""Gridding mode, host side and oracle pins (no GPU).

* the library's grid directions and angles against the reference's numpy
  construction (utils_gridding.py:140-152, 270-276), restated in
  oracle/gridding_oracle.py;
* the oracle's map value (leg detail + cal_rate with a zero incident leg)
  bit for bit against the reference library's own ray_tracing_single_gridding
  (compiled from its sources into oracle/_ref) on the same vector and angles.
"""
import os

import numpy as np
import pytest

from anacor_public_gb300 import gridding
from oracle import gridding_oracle as go
from oracle.oracle import REF_SO, Oracle, Reference


def _ang_diff(a, b):
    d = np.abs(np.asarray(a) - np.asarray(b))
    return np.minimum(d, np.abs(d - 2 * np.pi))


@pytest.mark.parametrize("nt,np_", [(36, 18), (72, 36), (360, 180)])
def test_directions_match_reference_numpy(nt, np_):
    s1, th, ph = gridding.directions(nt, np_)
    s1r, thr, phr = go.directions(nt, np_)
    # libm cos/sin of the two stacks may differ in the last bit
    assert np.abs(s1 - s1r).max() <= 4.5e-16
    assert _ang_diff(th, thr).max() < 1e-12
    assert _ang_diff(ph, phr).max() < 1e-12
    # rows are i_phi * n_theta + i_theta, unit vectors
    assert s1.shape == (nt * np_, 3)
    assert np.allclose(np.linalg.norm(s1, axis=1), 1.0, atol=1e-15)


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference library not built (oracle/_ref)")
def test_oracle_map_value_matches_reference(small):
    ref = Reference()
    orc = Oracle()
    s1, th, ph = go.directions(36, 18)
    rng = np.random.default_rng(0)
    dirs = rng.choice(len(s1), 12, replace=False)
    vox = small.coords[rng.choice(len(small.coords), 60, replace=False)]
    checked = 0
    for d in dirs:
        # the angles the reference's C computes for this vector (its assert is 1e-6)
        tp = ref.lib.dials_2_thetaphi_22(np.ascontiguousarray(s1[d]).copy(), 0)
        assert abs(tp.theta - th[d]) < 1e-6 and abs(tp.phi - ph[d]) < 1e-6
        det = orc.leg_detail(vox, s1[d], s1[d], small.voxel, small.label)
        ok = det["status"][:, 1] == 0
        want = go.map_value(det["L"][ok, 1, :], small.mu)
        # the reference aborts on asserting voxels: only call it where the oracle accepts
        got = ref.single_gridding(vox[ok], s1[d], tp.theta, tp.phi, small.voxel, small.mu, small.label)
        assert np.array_equal(got.astype(np.float32), want)
        a = ((small.mu[0] * (0.0 + det["L"][ok, 1, 0]) + small.mu[1] * (0.0 + det["L"][ok, 1, 1]))
             + small.mu[2] * (0.0 + det["L"][ok, 1, 2])) + small.mu[3] * (0.0 + det["L"][ok, 1, 3])
        assert np.array_equal(got, a)
        checked += int(ok.sum())
    assert checked > 500


def test_padded_axes_restatement():
    g = np.arange(36 * 18 * 5, dtype=np.float32).reshape(36 * 18, 5)
    grid, tl, pl = go.padded(g, 36, 18)
    # round((36 // 6) / 2) = 3 and round((18 // 6) / 2) = 2 (half to even)
    assert grid.shape == (5, 18 + 4, 36 + 6)
    assert tl[0] == -210.0 / 180 * np.pi and pl[0] == -105.0 / 180 * np.pi
    # wrap: padded (phi 0, theta 0) is original (phi 16, theta 33)
    assert grid[2, 0, 0] == g.reshape(18, 36, 5)[16, 33, 2]
