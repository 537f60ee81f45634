"""Bisection variant (the reference's ib_test) on the GPU against the oracle
(pinned to the reference library by tests/test_modes_oracle.py).  Tolerance:
A_h within 1e-6 relative (FP32 exp after FP64 range reduction, compensated
mean); the boundary points and lengths are FP64 with the reference's
operation order."""
import os

import numpy as np
import pytest

from anacor_public_gb300 import _lib, build, synth, tracer
from oracle.oracle import Oracle, row_table

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    build.build()
    return _lib.load()


def test_plan_bisection_matches_oracle(small):
    o = Oracle()
    plan = tracer.Plan.from_sample(small)
    try:
        for ncls in (4, 3):
            plan.run_bisection(ncls)
            got = plan.result()
            for i in range(0, small.n_refl, 9):
                xr, sr = o.rotate(small, i)
                want = o.ib(small.coords, sr, xr, small.voxel, small.mu, small.label, ncls)
                assert abs(got[i] - want) <= 1e-6 * want, (ncls, i, got[i], want)
    finally:
        plan.close()


def test_bisection_golden(small, golden_dir):
    ib = np.load(os.path.join(golden_dir, "small_ib.npz"))
    idx = ib["refl"]
    got = tracer.bisection(small.label, small.coords, small.s1[idx], small.omega[idx], small.xray,
                           small.omega_axis, small.F, small.voxel, small.mu, 4)
    assert np.max(np.abs(got - ib["ib4"]) / ib["ib4"]) <= 1e-6


def test_ib_test_dropin(small, lib):
    o = Oracle()
    tab, keep = row_table(np.ascontiguousarray(small.label))
    for i in (0, 50, 123):
        xr, sr = o.rotate(small, i)
        r = lib.ib_test(np.ascontiguousarray(small.coords), len(small.coords), sr.copy(), xr.copy(), small.voxel,
                        small.mu, tab, small.shape, 0, 0, 4)
        want = o.ib(small.coords, sr, xr, small.voxel, small.mu, small.label, 4)
        assert abs(r - want) <= 1e-6 * want
    del keep


def test_bisection_beamline_subset():
    s = synth.beamline_sample(n_refl=16)
    o = Oracle()
    got = tracer.bisection(s.label, s.coords, s.s1, s.omega, s.xray, s.omega_axis, s.F, s.voxel, s.mu, 4)
    for i in range(0, 16, 5):
        xr, sr = o.rotate(s, i)
        want = o.ib(s.coords, sr, xr, s.voxel, s.mu, s.label, 4)
        assert abs(got[i] - want) <= 1e-6 * want
