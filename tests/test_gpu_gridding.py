"""Gridding mode on the GPU against the oracle.

Tolerances: map values (float32 of the FP64 sum_m mu_m L_m) bit for bit; the
per-voxel drop-in's FP64 value bit for bit; interpolated A_h within 1e-6
relative (FP32 exp after FP64 range reduction and a compensated FP32 mean,
as for the plain kernel).
"""
import ctypes as ct
import os

import numpy as np
import pytest

from anacor_public_gb300 import _lib, build, gridding, synth, tracer
from oracle import gridding_oracle as go
from oracle.oracle import Oracle, row_table

pytestmark = pytest.mark.gpu
NT, NP = 72, 36


@pytest.fixture(scope="module")
def built(small):
    build.build()
    plan = tracer.Plan(small.label, small.coords, small.voxel, small.mu)
    g = gridding.GriddingMap(plan, NT, NP).build()
    m = g.map()
    yield plan, g, m
    g.close()
    plan.close()


def test_map_matches_oracle(small, built):
    _, g, m = built
    orc = Oracle()
    s1, th, ph = gridding.directions(NT, NP)
    rng = np.random.default_rng(1)
    for d in rng.choice(len(s1), 24, replace=False):
        det = orc.leg_detail(small.coords, s1[d], s1[d], small.voxel, small.label)
        assert (det["status"][:, 1] == 0).all()
        want = go.map_value(det["L"][:, 1, :], small.mu)
        assert np.array_equal(m[d], want), d


def test_map_from_explicit_directions(small, built):
    plan, g, m = built
    s1, th, ph = gridding.directions(NT, NP)
    h = gridding.GriddingMap(plan, NT, NP).build(s1, th, ph)
    try:
        assert np.array_equal(h.map(), m)
    finally:
        h.close()


def test_map_method1_is_exp(small, built):
    plan, _, m = built
    h = gridding.GriddingMap(plan, NT, NP, method=1).build()
    try:
        e = h.map()
        want = np.exp(-m.astype(np.float64))
        # float32 of exp(-double): the double and the float32-rounded sum differ below 2^-24
        assert np.allclose(e, want, rtol=3e-7, atol=0)
    finally:
        h.close()


def test_set_map_round_trip(built):
    plan, g, m = built
    h = gridding.GriddingMap(plan, NT, NP)
    try:
        rng = np.random.default_rng(2)
        x = rng.random(m.shape, dtype=np.float32)
        h.set_map(x)
        assert np.array_equal(h.map(), x)
    finally:
        h.close()


def test_axes_match_reference(built):
    _, g, m = built
    t, p = g.axes()
    _, tl, pl = go.padded(m[:, :2], NT, NP)
    assert np.array_equal(t, tl) and np.array_equal(p, pl)


@pytest.mark.parametrize("method", [1, 2])
def test_interpolation_matches_oracle(small, built, method):
    _, g, m = built
    orc = Oracle()
    grid, tl, pl = go.padded(m, NT, NP)
    idx = np.arange(0, small.n_refl, 7)
    got = g.interpolate(small.s1[idx], small.omega[idx], small.xray, small.omega_axis, small.F, method=method)
    for j, i in enumerate(idx):
        xr, sr = orc.rotate(small, int(i))
        want = go.interpolate(grid, tl, pl, xr, sr, method=method)
        assert abs(got[j] - want) <= 1e-6 * abs(want), (i, got[j], want)


def test_dropin_interpolate_overall(small, built):
    plan, g, m = built
    grid, tl, pl = go.padded(m, NT, NP)
    L = _lib.load()
    n = 64
    res = L.nearest_neighbor_interpolate_overall(
        0, n, np.ascontiguousarray(small.coords), len(small.coords), np.ascontiguousarray(small.s1[:n]),
        np.ascontiguousarray(small.omega[:n]), small.xray, small.omega_axis, small.F, n, small.voxel, small.mu,
        4, 1, tl, pl, grid, len(tl), len(pl), tl.min(), tl.max(), pl.min(), pl.max(), 1)
    assert res
    out = np.array([res[i] for i in range(n)])
    L.free(ct.cast(res, ct.c_void_p))
    want = g.interpolate(small.s1[:n], small.omega[:n], small.xray, small.omega_axis, small.F, method=1)
    assert np.allclose(out, want, rtol=1e-6, atol=0)


def test_dropin_single_gridding(small):
    build.build()
    L = _lib.load()
    orc = Oracle()
    s1, th, ph = gridding.directions(36, 18)
    tab, keep = row_table(np.ascontiguousarray(small.label))
    shape = np.array(small.label.shape, dtype=np.int64)
    rng = np.random.default_rng(3)
    for d in rng.choice(len(s1), 5, replace=False):
        vox = small.coords[rng.choice(len(small.coords), 6, replace=False)]
        det = orc.leg_detail(vox, s1[d], s1[d], small.voxel, small.label)
        Lg = det["L"][:, 1, :]
        for k, c in enumerate(vox):
            v = L.ray_tracing_single_gridding(np.ascontiguousarray(c), np.ascontiguousarray(s1[d]), th[d], ph[d],
                                              small.voxel, small.mu, tab, shape, 0, 0, 0)
            mu = small.mu
            a = ((mu[0] * (0.0 + Lg[k, 0]) + mu[1] * (0.0 + Lg[k, 1])) + mu[2] * (0.0 + Lg[k, 2])) \
                + mu[3] * (0.0 + Lg[k, 3])
            assert v == a
    # angles that are not the vector's: the reference asserts, the drop-in reports it
    v = L.ray_tracing_single_gridding(np.ascontiguousarray(small.coords[0]), np.ascontiguousarray(s1[0]),
                                      th[0] + 0.1, ph[0], small.voxel, small.mu, tab, shape, 0, 0, 0)
    assert np.isnan(v) and L.anacor_last_status() == 2
    v = L.ib_single_gridding(np.ascontiguousarray(small.coords[0]), np.ascontiguousarray(s1[0]), th[0] + 0.1,
                             ph[0], small.voxel, small.mu, tab, shape, 0, 0, 4, 0)
    assert np.isnan(v) and L.anacor_last_status() == 2
    del keep


def test_dropin_ib_single_gridding_vs_reference_fixture(small, golden_dir):
    """ib_single_gridding through the drop-in: bit for bit with the reference's
    own values (64 voxels x 8 directions, num_cls 4 and 3, exponent and exp)."""
    build.build()
    L = _lib.load()
    g = np.load(os.path.join(golden_dir, "small_ib_grid.npz"))
    tab, keep = row_table(np.ascontiguousarray(small.label))
    shape = np.array(small.label.shape, dtype=np.int64)
    for ncls in (4, 3):
        for ex in (0, 1):
            want = g[f"v{ncls}_{ex}"]
            for j in range(len(g["dirs"])):
                th, ph = g["angles"][j]
                for k, c in enumerate(g["coords"]):
                    v = L.ib_single_gridding(np.ascontiguousarray(c), np.ascontiguousarray(g["s1"][j]), th, ph,
                                             small.voxel, small.mu, tab, shape, 0, 0, ncls, ex)
                    assert v == want[j, k], (ncls, ex, j, k, v, want[j, k], L.anacor_last_error())
    del keep


def test_gridding_accuracy_vs_plain(small, built):
    _, g, _ = built
    plain = tracer.sample_absorption(small)
    near = g.interpolate(small.s1, small.omega, small.xray, small.omega_axis, small.F, method=1)
    lin = g.interpolate(small.s1, small.omega, small.xray, small.omega_axis, small.F, method=2)
    en = np.abs(near - plain) / plain
    el = np.abs(lin - plain) / plain
    # a 5-degree grid: percent-level approximations, bilinear better than nearest
    assert np.median(en) < 0.05 and np.median(el) < np.median(en)


def test_prepare_run_equals_interpolate(small, built):
    import torch
    _, g, _ = built
    n = small.n_refl
    want = g.interpolate(small.s1, small.omega, small.xray, small.omega_axis, small.F, method=1)
    g.prepare(small.s1, small.omega, small.xray, small.omega_axis, small.F, method=1)
    d = torch.empty(n, dtype=torch.float64, device="cuda")
    g.run(d.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy(), want)
