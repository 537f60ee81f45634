"""Oracle pins of the bisection and gridding modes against fixtures made by
the reference library itself (tests/golden/make_golden.py --modes), bit for
bit, and live against the reference where it is built here."""
import os

import numpy as np
import pytest

from anacor_public_gb300 import synth
from oracle import gridding_oracle as go
from oracle.oracle import REF_SO, Oracle, Reference


@pytest.fixture(scope="module")
def fx(golden_dir):
    return np.load(os.path.join(golden_dir, "small_ib.npz")), np.load(os.path.join(golden_dir, "small_grid.npz"))


def test_oracle_bisection_matches_reference_fixture(small, oracle, fx):
    ib, _ = fx
    for ncls, key in ((4, "ib4"), (3, "ib3")):
        got = []
        for i in ib["refl"]:
            xr, sr = oracle.rotate(small, int(i))
            got.append(oracle.ib(small.coords, sr, xr, small.voxel, small.mu, small.label, ncls))
        assert np.array_equal(np.array(got), ib[key]), key


def test_oracle_map_value_matches_reference_fixture(small, oracle, fx):
    _, g = fx
    for k, s1 in enumerate(g["s1"]):
        th, ph = g["angles"][k]
        det = oracle.leg_detail(g["coords"], s1, s1, small.voxel, small.label)
        assert (det["status"][:, 1] == 0).all()
        L = det["L"][:, 1, :]
        mu = small.mu
        a = ((mu[0] * (0.0 + L[:, 0]) + mu[1] * (0.0 + L[:, 1])) + mu[2] * (0.0 + L[:, 2])) + mu[3] * (0.0 + L[:, 3])
        assert np.array_equal(a, g["value"][k])


def test_oracle_ib_single_gridding_matches_reference_fixture(small, oracle, golden_dir):
    g = np.load(os.path.join(golden_dir, "small_ib_grid.npz"))
    from tests.golden.make_golden import sample_digest
    assert str(g["digest"]) == sample_digest(small)
    for ncls in (4, 3):
        for ex in (0, 1):
            got = np.array([oracle.ib_gridding(g["coords"], g["s1"][j], g["angles"][j, 0], g["angles"][j, 1],
                                               small.voxel, small.mu, small.label, ncls, ex)
                            for j in range(len(g["dirs"]))])
            assert np.array_equal(got, g[f"v{ncls}_{ex}"]), (ncls, ex)


def test_oracle_ib_single_gridding_reports_the_reference_assert(small, oracle):
    s1, th, ph = go.directions(36, 18)
    with pytest.raises(RuntimeError, match="assert"):
        oracle.ib_gridding(small.coords[:4], s1[7], th[7] + 0.1, ph[7], small.voxel, small.mu, small.label)


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference library not built (oracle/_ref)")
def test_oracle_ib_single_gridding_live_other_directions(small, oracle):
    r = Reference()
    s1, th, ph = go.directions(24, 12)
    vox = small.coords[::97]
    for d in range(5, len(s1), 41):
        assert np.array_equal(oracle.ib_gridding(vox, s1[d], th[d], ph[d], small.voxel, small.mu, small.label, 4, 1),
                              r.ib_single_gridding(vox, s1[d], th[d], ph[d], small.voxel, small.mu, small.label, 4, 1))


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference library not built (oracle/_ref)")
def test_oracle_bisection_live_other_seed():
    s = synth.small_sample(n_refl=40, seed=3)
    o, r = Oracle(), Reference()
    for i in range(0, 40, 4):
        xr, sr = o.rotate(s, i)
        for ncls in (3, 4):
            a = o.ib(s.coords, sr, xr, s.voxel, s.mu, s.label, ncls)
            assert a == r.ib_test(s.coords, sr, xr, s.voxel, s.mu, s.label, ncls)


def test_bisection_is_an_approximation_of_the_march(small, oracle):
    # the method itself: bisection paths versus the exact march (percent level)
    ex = oracle.overall(small.subset(refl=slice(0, 30, 3)))
    for j, i in enumerate(range(0, 30, 3)):
        xr, sr = oracle.rotate(small, i)
        a = oracle.ib(small.coords, sr, xr, small.voxel, small.mu, small.label, 4)
        assert abs(a - ex[j]) / ex[j] < 0.03
