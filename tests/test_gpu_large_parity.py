"""GPU parity at the large workloads, for every march kind.

Fixtures come from the reference library compiled from its own sources
(``tests/golden/make_golden.py --large``); the volumes are regenerated here from
their seeds and pinned by the fixtures' input digests:

* the 20,000-reflection beamline workload (512x512x400, stride-4 voxels):
  A_h of 256 reflections over every voxel;
* the 1024x1024x800 mu x5 workload: A_h of 48 reflections over a seeded
  32,768-voxel subset (the largest exponents of any workload: A_h ~ 0.004-0.01),
  and per-voxel, per-leg detail of 2 reflections on 2,048 voxels;
* the largest-volume sample of the 12-sample batch (347x288x578): A_h of 48
  reflections over all its voxels, per-leg detail of 1 reflection.

Tolerances: A_h within 1e-6 relative of the reference (FP64 throughout there);
exit face, len_path_2, segment count, path end points and the four per-material
lengths bit-identical; the four marches (warp-cooperative, centred distance
field, octant fields, octant fields in 4^3 bricks) visit the same label
steps (sum of len_path_2 equal).
"""
import os
import sys

import numpy as np
import pytest

from anacor_public_gb300 import _lib, build, synth, tracer
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu
RTOL = 1e-6
HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)
from make_golden import sample_digest  # noqa: E402

# one variant per march kind, at the 4-CTA and 2-CTA register budgets
VARIANTS = {"cooperative": (4, 2), "centred field": (8, 6), "octant fields": (12, 10),
            "bricked octant fields": (16, 14)}


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def max_rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.abs(b)))


def check_marches(s, gold, label):
    p = tracer.Plan.from_sample(s)
    errs, steps = {}, {}
    try:
        for kind, variants in VARIANTS.items():
            for v in variants:
                p.configure(v)
                p.run()
                errs[(kind, v)] = max_rel(p.result(), gold)
                steps[(kind, v)] = p.count_steps()
    finally:
        p.close()
    print(f"\n{label}: max relative error of A_h vs the reference: " +
          ", ".join(f"{k} v{v} {e:.2e}" for (k, v), e in errs.items()))
    assert max(errs.values()) <= RTOL, errs
    assert len(set(steps.values())) == 1, steps
    return errs


def check_legs(s, f, refl_index, coords):
    o = Oracle()
    for j, k in enumerate(f["leg_refl"]):
        xr, sr = o.rotate(s, int(k))
        g = tracer.leg_detail(s.label, coords, sr, xr, s.voxel)
        assert (g["status"] == 0).all()
        for key in ("face", "len", "nseg", "L"):
            want = f[f"leg_{key}"][j]
            assert np.array_equal(g[key].astype(want.dtype), want), key
        moved = f["leg_len"][j] > 1
        for key in ("first", "last"):
            assert np.array_equal(g[key][moved].astype(np.int64), f[f"leg_{key}"][j][moved]), key
        print(f"reflection {refl_index[int(k)]}: {len(coords)} voxels x 2 legs bit-identical, "
              f"{int(f['leg_len'][j].sum())} label steps, longest leg {int(f['leg_len'][j].max())}")


@pytest.fixture(scope="module")
def beamline():
    s = synth.beamline_sample()
    f = np.load(os.path.join(GOLDEN, "beamline_ah256.npz"))
    assert sample_digest(s) == str(f["digest"])
    return s, f


def test_beamline_256_reflections_every_march(lib, beamline):
    s, f = beamline
    check_marches(s.subset(refl=f["refl"]), f["ah"], "beamline 256 reflections x 22,917 voxels")


@pytest.fixture(scope="module")
def highabs():
    s = synth.high_absorption_sample()
    f = np.load(os.path.join(GOLDEN, "highabs_ah.npz"))
    assert sample_digest(s) == str(f["digest"])
    sub = s.subset(refl=f["refl"], coords=s.coords[f["voxels"]])
    return sub, f


def test_high_absorption_every_march(lib, highabs):
    s, f = highabs
    check_marches(s, f["ah"], "1024x1024x800 mu x5, 48 reflections x 32,768 voxels")


def test_high_absorption_legs_bitwise(lib, highabs):
    s, f = highabs
    check_legs(s, f, f["refl"], s.coords[f["leg_voxels"]])


@pytest.fixture(scope="module")
def batch_largest():
    f = np.load(os.path.join(GOLDEN, "batch_ah.npz"))
    s = synth.batch_samples(only=int(f["sample"]))[0]
    assert sample_digest(s) == str(f["digest"])
    return s.subset(refl=f["refl"]), f


def test_batch_largest_sample_every_march(lib, batch_largest):
    s, f = batch_largest
    check_marches(s, f["ah"], f"batch sample {s.label.shape}, 48 reflections x {len(s.coords)} voxels")


def test_batch_largest_sample_legs_bitwise(lib, batch_largest):
    s, f = batch_largest
    check_legs(s, f, f["refl"], s.coords[f["leg_voxels"]])
