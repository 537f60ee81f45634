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
