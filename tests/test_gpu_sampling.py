"""GPU voxel sampling against numpy restatements of the reference's host
sampling (AnACor/utils/utils_rt.py:27-253): np.where order, the 'even'
method's np.linspace picks, and the stride lattice of the benchmark
configurations.  Integer results: exact equality."""
import numpy as np
import pytest

from anacor_public_gb300 import build, synth, tracer

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib():
    build.build()


def even_reference(label, cr=3, sampling_size=5000, sampling_ratio=None):
    """generate_sampling(method='even') of utils_rt.py:27-84, restated."""
    zz, yy, xx = np.where(label == cr)
    c = np.stack((zz, yy, xx), axis=1)
    if sampling_ratio is not None:
        n = int(len(c) * sampling_ratio / 100)
    else:
        n = len(c) if len(c) < sampling_size else len(c) // sampling_size
    idx = np.linspace(0, len(c), num=n, endpoint=False, dtype=int)
    return c[idx]


def test_all_voxels_match_np_where(small):
    got = tracer.sample_voxels(small.label, method="all")
    assert np.array_equal(got, np.argwhere(small.label == 3))


@pytest.mark.parametrize("size,ratio", [(5000, None), (100, None), (10, None), (5000, 10.0), (5000, 37.5)])
def test_even_matches_reference(small, size, ratio):
    got = tracer.sample_voxels(small.label, method="even", sampling_size=size, sampling_ratio=ratio)
    assert np.array_equal(got, even_reference(small.label, 3, size, ratio))


def test_stride_matches_lattice(small):
    for st in (2, 3, 4):
        got = tracer.sample_voxels(small.label, method="stride", stride=st)
        assert np.array_equal(got, synth.crystal_coords(small.label, st))


def test_other_label_codes(small):
    for code in (1, 2, 4):
        got = tracer.sample_voxels(small.label, crystal_code=code, method="all")
        assert np.array_equal(got, np.argwhere(small.label == code))


def test_beamline_volume_even_and_stride():
    s = synth.beamline_sample(n_refl=64)
    got = tracer.sample_voxels(s.label, method="stride", stride=4)
    assert np.array_equal(got, s.coords)
    got = tracer.sample_voxels(s.label, method="even", sampling_ratio=1.0)
    assert np.array_equal(got, even_reference(s.label, 3, 5000, 1.0))


def test_plan_from_volume_gives_identical_absorption(small):
    a = tracer.Plan.from_sample(small)
    b = tracer.Plan.from_volume(small.label, small.voxel, small.mu, method="all")
    try:
        b.set_reflections(small.s1, small.omega, small.xray, small.omega_axis, small.F)
        a.run()
        b.run()
        assert np.array_equal(a.result(), b.result())
        assert np.array_equal(b.voxels(), small.coords)
    finally:
        a.close()
        b.close()


def test_empty_selection(small):
    got = tracer.sample_voxels(small.label, crystal_code=9, method="all")
    assert got.shape == (0, 3)
