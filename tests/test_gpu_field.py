"""Distance-field march (kernel variants 5..8).

The packed field is checked against a CPU chessboard distance (min/max
filters over growing cubes), and the march that steps over increments the
field proves to keep their label against the oracle and against the
per-increment cooperative march: the same len_path_2 totals, and A_h bit for
bit under the same tile and voxel order (the per-voxel terms and their FP32
summation order are the same).  A_h tolerance against the oracle: 1e-6
relative, as for every other variant.
"""
import os

import numpy as np
import pytest
from scipy import ndimage as nd

from anacor_public_gb300 import _lib, build, synth, tracer

pytestmark = pytest.mark.gpu
RTOL = 1e-6
K_UNSUPPORTED = 6


@pytest.fixture(scope="module", autouse=True)
def lib():
    build.build()


def max_rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)) / np.abs(np.asarray(b))))


def field_cpu(label):
    """(label & 7) | (min(D, 31) << 3), D = 1 + the largest r whose clipped
    cube around the voxel holds one label; 0 for label-0 voxels."""
    lab = label.astype(np.int16)
    D = np.ones(lab.shape, np.int32)
    alive = np.ones(lab.shape, bool)
    for r in range(1, 31):
        # edge replication leaves the min and max of a clipped cube unchanged
        mx = nd.maximum_filter(lab, size=2 * r + 1, mode="nearest")
        mn = nd.minimum_filter(lab, size=2 * r + 1, mode="nearest")
        alive &= (mx == lab) & (mn == lab)
        if not alive.any():
            break
        D[alive] = r + 1
    out = (lab & 7) | (D << 3)
    out[lab == 0] = 0
    return out.astype(np.uint8)


def octant_fields_cpu(label):
    """[octant][Z][Y][X]: (label & 7) | (min(r + 1, 31) << 3), r the largest
    corner box toward the octant's signs holding one label; 0 for label 0."""
    lab = label.astype(np.int16)
    out = np.zeros((8,) + lab.shape, np.uint8)
    for o in range(8):
        signs = (-1 if o & 4 else 1, -1 if o & 2 else 1, -1 if o & 1 else 1)   # z, y, x
        D = np.ones(lab.shape, np.int32)
        alive = np.ones(lab.shape, bool)
        for r in range(1, 31):
            size = r + 1
            # window over offsets 0..r toward each sign
            origin = [-(size // 2) if sg > 0 else (size - 1) - size // 2 for sg in signs]
            mx = nd.maximum_filter(lab, size=size, origin=origin, mode="nearest")
            mn = nd.minimum_filter(lab, size=size, origin=origin, mode="nearest")
            alive &= (mx == lab) & (mn == lab)
            if not alive.any():
                break
            D[alive] = r + 1
        f = (lab & 7) | (D << 3)
        f[lab == 0] = 0
        out[o] = f.astype(np.uint8)
    return out


def blocky_volume(shape, seed, n_boxes=40, labels=(1, 2, 3, 4, 5, 6, 7)):
    rng = np.random.default_rng(seed)
    vol = np.zeros(shape, np.int8)
    for _ in range(n_boxes):
        lo = [int(rng.integers(0, d)) for d in shape]
        hi = [min(d, l + int(rng.integers(1, max(2, d // 2)))) for l, d in zip(lo, shape)]
        vol[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] = rng.choice(labels)
    return vol


@pytest.mark.parametrize("shape,seed", [((20, 33, 47), 1), ((9, 70, 5), 2), ((64, 40, 72), 3), ((1, 1, 90), 4)])
def test_field_matches_cpu(shape, seed):
    vol = blocky_volume(shape, seed)
    assert np.array_equal(tracer.distance_field(vol), field_cpu(vol))


@pytest.mark.parametrize("shape,seed", [((20, 33, 47), 5), ((9, 70, 5), 6), ((1, 1, 90), 7),
                                        ((130, 67, 261), 8), ((150, 90, 260), 9), ((3, 140, 132), 10),
                                        ((40, 50, 1), 11), ((1, 200, 3), 12), ((70, 1, 70), 13)])
def test_octant_fields_match_cpu(shape, seed):
    # several tiles along every axis, rows with and without 4-byte alignment
    vol = blocky_volume(shape, seed)
    assert np.array_equal(tracer.octant_fields(vol), octant_fields_cpu(vol))


def test_octant_fields_of_a_sample_volume(small):
    assert np.array_equal(tracer.octant_fields(small.label), octant_fields_cpu(small.label))


def test_field_of_a_sample_volume(small):
    assert np.array_equal(tracer.distance_field(small.label), field_cpu(small.label))


def test_field_caps_at_31():
    vol = np.full((80, 70, 75), 3, np.int8)
    vol[0, 0, 0] = 1
    f = tracer.distance_field(vol)
    assert (f >> 3).max() == 31 and f[40, 40, 40] == 3 | (31 << 3)
    assert np.array_equal(f, field_cpu(vol))


def test_field_rejects_labels_outside_0_to_7():
    vol = np.ones((8, 9, 10), np.int8)
    vol[3, 4, 5] = 9
    with pytest.raises(_lib.AnacorError) as e:
        tracer.distance_field(vol)
    assert e.value.status == K_UNSUPPORTED
    vol[3, 4, 5] = -1
    with pytest.raises(_lib.AnacorError):
        tracer.distance_field(vol)


@pytest.fixture(scope="module")
def sample():
    return synth.small_sample(n_refl=48, seed=9)


@pytest.fixture(scope="module")
def want(sample, oracle):
    return oracle.overall(sample, threads=os.cpu_count() or 1)


@pytest.mark.parametrize("variant", [5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16])
@pytest.mark.parametrize("tile,order", [(512, 1), (2048, 0), (128, 3)])
def test_field_variants_match_the_oracle_and_the_cooperative_march(sample, want, variant, tile, order):
    p = tracer.Plan.from_sample(sample)
    p.configure(variant, tile, order)
    assert p.config() == {"variant": variant, "tile": tile, "order": order}
    p.run()
    a = p.result()
    assert max_rel(a, want) <= RTOL
    steps = p.count_steps()
    p.configure((variant - 1) % 4 + 1, tile, order)
    p.run()
    assert np.array_equal(p.result(), a)
    assert p.count_steps() == steps
    p.close()


@pytest.mark.parametrize("variant", [8, 12, 16])
def test_field_march_beamline_vs_golden(golden_dir, variant):
    gold = np.load(os.path.join(golden_dir, "beamline_ah.npz"))["ah"]
    b = synth.beamline_sample(n_refl=12)
    p = tracer.Plan.from_sample(b)
    p.configure(variant, 1024, 1)
    p.run()
    a = p.result()
    assert max_rel(a, gold) <= RTOL
    s8 = p.count_steps()
    p.configure(4, 1024, 1)
    p.run()
    assert np.array_equal(p.result(), a)
    assert p.count_steps() == s8
    p.close()


def _run(t, variant):
    p = tracer.Plan.from_sample(t)
    p.configure(variant, 512, 1)
    p.run()
    r = p.result()
    n = p.count_steps()
    p.close()
    return r, n


def test_field_march_on_wall_and_slab_volumes(oracle):
    s = synth.small_sample(n_refl=24)
    vols = []
    v = np.full((20, 24, 28), 1, dtype=np.int8)   # crystal and liquor up to the walls: per-lane legs
    v[4:16, 6:18, 2:26] = 3
    vols.append(v)
    v = np.ones((48, 56, 64), dtype=np.int8)      # more than 16 class changes per leg
    for z in range(48):
        v[z, :, :] = (1, 2, 4, 1, 2)[z % 5]
    v[20:28, 24:32, 28:36] = 3
    vols.append(v)
    v = blocky_volume((40, 44, 48), 7, labels=(1, 2, 4, 5, 6))   # codes 5..7 change no class
    v[14:26, 16:28, 18:30] = 3
    vols.append(v)
    v = blocky_volume((37, 42, 29), 8, labels=(1, 2, 4))   # axes not multiples of the 4^3 bricks
    v[12:25, 14:28, 9:20] = 3
    vols.append(v)
    for vol in vols:
        coords = np.ascontiguousarray(np.argwhere(vol == 3).astype(np.int64))
        t = synth.Sample(label=vol, coords=coords, s1=s.s1, omega=s.omega, xray=s.xray, omega_axis=s.omega_axis,
                         F=s.F, voxel=s.voxel, mu=s.mu)
        ref = oracle.overall(t, threads=4)
        a4, n4 = _run(t, 4)
        for v in (8, 12, 16):
            a8, n8 = _run(t, v)
            assert max_rel(a8, ref) <= RTOL
            assert np.array_equal(a8, a4) and n8 == n4


def test_field_variant_refused_for_wide_labels(sample):
    vol = sample.label.copy()
    vol[0, 0, 0] = 12
    p = tracer.Plan(vol, sample.coords, sample.voxel, sample.mu)
    p.set_reflections(sample.s1[:8], sample.omega[:8], sample.xray, sample.omega_axis, sample.F)
    for v in (8, 12, 16):
        with pytest.raises(_lib.AnacorError) as e:
            p.configure(v, 512, 1)
        assert e.value.status == K_UNSUPPORTED
    p.autotune()
    assert p.config()["variant"] in (2, 3, 4)
    p.close()


def test_batch_runs_samples_without_a_field_in_a_cooperative_launch(oracle):
    import torch
    samples = synth.batch_samples(n_samples=3, max_refl=16, dim_range=(64, 128))
    wide = samples[2].label.copy()
    wide[0, 0, 0] = 9   # no field for this one
    samples[2] = synth.Sample(label=wide, coords=samples[2].coords, s1=samples[2].s1, omega=samples[2].omega,
                              xray=samples[2].xray, omega_axis=samples[2].omega_axis, F=samples[2].F,
                              voxel=samples[2].voxel, mu=samples[2].mu)
    wants = [oracle.overall(s, threads=os.cpu_count() or 1) for s in samples]
    plans = [tracer.Plan.from_sample(s) for s in samples]
    plans[0].configure(8, 512, 1)
    plans[1].configure(12, 512, 1)   # octant fields, in the same field launch
    plans[2].configure(4, 512, 1)
    b = tracer.Batch(plans)
    st = torch.cuda.Stream()
    got = {}
    for v, kernels in ((8, 2), (4, 1), (7, 2), (16, 2), (11, 2)):
        b.configure(v)
        assert b.info()["kernels"] == kernels
        b.launch(st.cuda_stream)
        b.wait(st.cuda_stream)
        got[v] = b.results(st.cuda_stream)
        for g, w in zip(got[v], wants):
            assert max_rel(g, w) <= RTOL
    for g8, g4 in zip(got[8], got[4]):
        assert np.array_equal(g8, g4)
    b.configure(8)
    b.capture(st.cuda_stream)
    b.replay(st.cuda_stream)
    b.wait(st.cuda_stream)
    for g, g8 in zip(b.results(st.cuda_stream), got[8]):
        assert np.array_equal(g, g8)
    b.close()
    for p in plans:
        p.close()


def test_field_variants_with_full_iteration_and_no_exp(small, oracle):
    s = small.subset(refl=slice(0, 24))
    for full, ie in ((1, 1), (0, 0), (1, 0)):
        ref = oracle.overall(s, threads=os.cpu_count() or 1, full_iteration=full, is_exp=ie)
        got = {}
        for v in (4, 8, 12, 16):
            p = tracer.Plan(s.label, s.coords, s.voxel, s.mu, full_iteration=full, is_exp=ie)
            p.set_reflections(s.s1, s.omega, s.xray, s.omega_axis, s.F)
            p.configure(v, 512, 1)
            p.run()
            got[v] = p.result()
            p.close()
            assert max_rel(got[v], ref) <= RTOL, (full, ie, v)
        assert np.array_equal(got[8], got[4]) and np.array_equal(got[12], got[4]) and np.array_equal(got[16], got[4])
