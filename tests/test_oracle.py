"""The oracle (C restatement) pinned against the reference's golden vectors
and, where the reference sources were compiled here, the reference itself."""
import os

import numpy as np
import pytest

from anacor_public_gb300 import synth
from oracle import oracle as orc
from tests.golden.make_golden import (cylinder_directions, cylinder_volume, sample_digest, sphere_directions,
                                      sphere_volume)


def test_generator_reproduces_golden_inputs(small, golden_dir):
    g = np.load(os.path.join(golden_dir, "small_ah.npz"))
    assert str(g["digest"]) == sample_digest(small)


def test_oracle_matches_reference_small_sample_bitwise(oracle, small, golden_dir):
    g = np.load(os.path.join(golden_dir, "small_ah.npz"))
    ah = oracle.overall(small, threads=os.cpu_count() or 1)
    assert np.array_equal(ah, g["ah"])


def test_oracle_matches_reference_leg_detail(oracle, small, golden_dir):
    g = np.load(os.path.join(golden_dir, "small_legs.npz"))
    coords = g["coords"]
    for k, i in enumerate(g["refl"]):
        xr, sr = oracle.rotate(small, int(i))
        d = oracle.leg_detail(coords, sr, xr, small.voxel, small.label)
        assert (d["status"] == 0).all()
        for key in ("face", "len", "nseg", "L"):
            assert np.array_equal(d[key], g[key][k]), key
        moved = d["len"] > 1
        assert np.array_equal(d["last"][moved], g["last"][k][moved])


def test_oracle_matches_reference_beamline_subset(oracle, golden_dir):
    g = np.load(os.path.join(golden_dir, "beamline_ah.npz"))
    b = synth.beamline_sample(n_refl=12)
    assert str(g["digest"]) == sample_digest(b)
    ah = oracle.overall(b, threads=os.cpu_count() or 1)
    assert np.array_equal(ah, g["ah"])


def test_oracle_matches_reference_beamline_workload(oracle, golden_dir):
    """32 of the 256 reference A_h of the 20,000-reflection beamline workload."""
    g = np.load(os.path.join(golden_dir, "beamline_ah256.npz"))
    b = synth.beamline_sample()
    assert str(g["digest"]) == sample_digest(b)
    k = np.arange(0, 256, 8)
    ah = oracle.overall(b.subset(refl=g["refl"][k]), threads=os.cpu_count() or 1)
    assert np.array_equal(ah, g["ah"][k])


def test_oracle_matches_reference_largest_batch_sample(oracle, golden_dir):
    g = np.load(os.path.join(golden_dir, "batch_ah.npz"))
    s = synth.batch_samples(only=int(g["sample"]))[0]
    assert str(g["digest"]) == sample_digest(s)
    ss = s.subset(refl=g["refl"])
    assert np.array_equal(oracle.overall(ss, threads=os.cpu_count() or 1), g["ah"])
    xr, sr = oracle.rotate(ss, 0)
    d = oracle.leg_detail(s.coords[g["leg_voxels"]], sr, xr, s.voxel, s.label)
    for key in ("face", "len", "nseg", "L"):
        assert np.array_equal(d[key], g[f"leg_{key}"][0]), key


def test_oracle_sphere_known_answers(oracle, golden_dir):
    g = np.load(os.path.join(golden_dir, "sphere_kat.npz"))
    vol = sphere_volume(24)
    voxel = np.array([0.5] * 3)
    dirs = sphere_directions(g["two_theta"])
    # discretisation error of the reference's method grows with mu*r
    tol = {0.1: 0.01, 0.5: 0.04, 1.0: 0.07}
    for k, mur in enumerate(g["mur"]):
        mu = np.array([0.0, 0.0, mur / (24 * 0.5), 0.0])
        got = np.array([oracle.single(g["coords"], sr, xr, voxel, mu, vol) for xr, sr in dirs])
        assert np.array_equal(got, g["reference"][k])
        rel = np.abs(got - g["analytic"][k]) / g["analytic"][k]
        assert rel.max() < tol[float(mur)]


def test_oracle_cylinder_known_answers(oracle, golden_dir):
    g = np.load(os.path.join(golden_dir, "cylinder_kat.npz"))
    vol = cylinder_volume(24, 2)
    voxel = np.array([0.5] * 3)
    dirs = cylinder_directions(g["two_theta"])
    tol = {0.1: 0.01, 0.5: 0.04, 1.0: 0.07}
    for k, mur in enumerate(g["mur"]):
        mu = np.array([0.0, 0.0, mur / (24 * 0.5), 0.0])
        got = np.array([oracle.single(g["coords"], sr, xr, voxel, mu, vol) for xr, sr in dirs])
        assert np.array_equal(got, g["reference"][k])
        rel = np.abs(got - g["analytic"][k]) / g["analytic"][k]
        assert rel.max() < tol[float(mur)]


@pytest.mark.skipif(not os.path.exists(orc.REF_SO), reason="reference sources not compiled here")
def test_oracle_matches_reference_full_iteration(oracle, small):
    ref = orc.Reference()
    s = small.subset(refl=slice(0, 20))
    a = oracle.overall(s, threads=4, full_iteration=1)
    b = ref.overall(s, num_workers=4, full_iteration=1)
    assert np.array_equal(a, b)


@pytest.mark.skipif(not os.path.exists(orc.REF_SO), reason="reference sources not compiled here")
def test_oracle_matches_reference_other_seeds():
    ref = orc.Reference()
    o = orc.Oracle()
    for seed in (5, 6):
        s = synth.make_sample(shape=(64, 72, 80), semi_axes=(14, 10, 8), shell=5, torus=(18, 2.5), bubble_r=2.5,
                              n_refl=40, seed=seed)
        assert np.array_equal(o.overall(s, threads=4), ref.overall(s, num_workers=4))


def test_oracle_reports_reference_abort_cases(oracle, small):
    # a rotated beam with an exactly-zero DIALS-y component takes the
    # reference's +0.001 branch; its face/angle check fails (the reference
    # aborts the process there), the oracle returns a status instead
    xr = np.array([-0.6, 0.0, 0.8])
    sr = np.array([0.3, 0.5, 0.81])
    with pytest.raises(RuntimeError, match="assert"):
        oracle.single(small.coords[:50], sr, xr, small.voxel, small.mu, small.label)
