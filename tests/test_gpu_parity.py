"""GPU path vs the oracle: per-ray path detail bit for bit, A_h within 1e-6.

Tolerances: per-voxel, per-material lengths (and every path quantity) must be
bit-identical to the reference's; A_h within 1e-6 relative (FP32 exp and an
FP32 compensated mean, as specified for the plain kernel).
"""
import ctypes as ct
import os

import numpy as np
import pytest

from anacor_public_gb300 import _lib, build, synth, tracer
from oracle.oracle import Oracle, row_table

pytestmark = pytest.mark.gpu
RTOL = 1e-6


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def max_rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))) if a.size else 0.0


def assert_legs_equal(g, o):
    assert (o["status"] == 0).all()
    assert (g["status"] == 0).all()
    for k in ("face", "len", "nseg", "L"):
        assert np.array_equal(g[k].astype(o[k].dtype), o[k]), k
    moved = o["len"] > 1
    assert np.array_equal(g["last"][moved].astype(np.int64), o["last"][moved])
    assert np.array_equal(g["first"][moved].astype(np.int64), o["first"][moved])


def test_leg_detail_small_sample_bitwise(lib, small, oracle):
    for i in range(0, small.n_refl, 10):
        xr, sr = oracle.rotate(small, i)
        g = tracer.leg_detail(small.label, small.coords, sr, xr, small.voxel)
        o = oracle.leg_detail(small.coords, sr, xr, small.voxel, small.label)
        assert_legs_equal(g, o)


def test_leg_detail_beamline_bitwise(lib, oracle):
    b = synth.beamline_sample(n_refl=6)
    for i in range(b.n_refl):
        xr, sr = oracle.rotate(b, i)
        g = tracer.leg_detail(b.label, b.coords, sr, xr, b.voxel)
        o = oracle.leg_detail(b.coords, sr, xr, b.voxel, b.label)
        assert_legs_equal(g, o)


def test_absorption_small_sample_vs_golden(lib, small, golden_dir):
    gold = np.load(os.path.join(golden_dir, "small_ah.npz"))["ah"]
    got = tracer.sample_absorption(small)
    assert max_rel(got, gold) <= RTOL


def test_absorption_beamline_vs_golden(lib, golden_dir):
    gold = np.load(os.path.join(golden_dir, "beamline_ah.npz"))["ah"]
    b = synth.beamline_sample(n_refl=12)
    assert max_rel(tracer.sample_absorption(b), gold) <= RTOL


def test_absorption_is_deterministic(lib, small):
    p = tracer.Plan.from_sample(small)
    p.run()
    a = p.result()
    p.run()
    b = p.result()
    assert np.array_equal(a, b)
    p.close()


def test_full_iteration_and_no_exp(lib, small, oracle):
    s = small.subset(refl=slice(0, 40))
    for full, ie in ((1, 1), (0, 0), (1, 0)):
        got = tracer.sample_absorption(s, full_iteration=full, is_exp=ie)
        ref = oracle.overall(s, threads=os.cpu_count() or 1, full_iteration=full, is_exp=ie)
        assert max_rel(got, ref) <= RTOL, (full, ie)
    xr, sr = oracle.rotate(s, 3)
    assert_legs_equal(tracer.leg_detail(s.label, s.coords, sr, xr, s.voxel, full_iteration=1),
                      oracle.leg_detail(s.coords, sr, xr, s.voxel, s.label, full_iteration=1))


def test_many_class_changes_use_second_pass(lib, oracle):
    # alternating liquor / loop / bubble slabs: legs cross far more than 16
    # material boundaries, so the kernel re-marches to accumulate lengths
    vol = np.ones((48, 56, 64), dtype=np.int8)
    for z in range(48):
        vol[z, :, :] = (1, 2, 4, 1, 2)[z % 5]
    vol[20:28, 24:32, 28:36] = 3
    coords = np.ascontiguousarray(np.argwhere(vol == 3).astype(np.int64))
    s = synth.small_sample(n_refl=24)
    for i in range(s.n_refl):
        xr, sr = oracle.rotate(s, i)
        o = oracle.leg_detail(coords, sr, xr, s.voxel, vol)
        g = tracer.leg_detail(vol, coords, sr, xr, s.voxel)
        assert_legs_equal(g, o)
    assert o["nseg"].max() > 16
    t = synth.Sample(label=vol, coords=coords, s1=s.s1, omega=s.omega, xray=s.xray, omega_axis=s.omega_axis,
                     F=s.F, voxel=s.voxel, mu=s.mu)
    assert max_rel(tracer.sample_absorption(t), oracle.overall(t, threads=4)) <= RTOL


def test_voxels_on_the_volume_boundary(lib, oracle):
    # crystal touching every face: zero-distance exit faces and clamped steps
    vol = np.full((20, 24, 28), 1, dtype=np.int8)
    vol[:, :, :4] = 3
    vol[:3, :, :] = 3
    vol[:, -2:, :] = 3
    coords = np.ascontiguousarray(np.argwhere(vol == 3).astype(np.int64))
    s = synth.small_sample(n_refl=30)
    ok = 0
    for i in range(s.n_refl):
        xr, sr = oracle.rotate(s, i)
        o = oracle.leg_detail(coords, sr, xr, s.voxel, vol)
        g = tracer.leg_detail(vol, coords, sr, xr, s.voxel)
        # legs the reference would abort on carry the same status; every other
        # leg matches bit for bit
        assert np.array_equal(g["status"], o["status"])
        good = o["status"] == 0
        ok += int(good.sum())
        for k in ("face", "len", "nseg", "L"):
            assert np.array_equal(g[k][good].astype(o[k].dtype), o[k][good]), k
        moved = good & (o["len"] > 1)
        assert np.array_equal(g["last"][moved].astype(np.int64), o["last"][moved])
    assert ok >= 1000


def test_diagonal_and_axis_aligned_directions(lib, small, oracle):
    # 45-degree and near-axis rays: positions land on rounding boundaries
    # (FP64 fallback) and ratios exceed the fixed-point range (FP64 march)
    dirs = []
    for v in ([1, 1, 1], [1, -1, 1], [-1, 1, 1e-7], [1e-6, 1, 1], [1, 2, 3], [-2, 1, 1], [1, 1e-9, -1],
              [0.5, 0.5, 0.7071067811865476]):
        v = np.array(v, dtype=np.float64)
        dirs.append(v / np.linalg.norm(v))
    coords = small.coords[::5]
    checked = 0
    for xr in dirs:
        for sr in dirs:
            o = oracle.leg_detail(coords, sr, xr, small.voxel, small.label)
            if (o["status"] != 0).any():
                continue
            checked += 1
            assert_legs_equal(tracer.leg_detail(small.label, coords, sr, xr, small.voxel), o)
    assert checked >= 10


def test_exact_zero_components(lib, small, oracle):
    # rotation about DIALS x with the beam along -z keeps x exactly zero
    s = synth.Sample(label=small.label, coords=small.coords[::3].copy(), s1=small.s1[:30], omega=small.omega[:30],
                     xray=np.array([0.0, 0.0, -1.0]), omega_axis=np.array([1.0, 0.0, 0.0]),
                     F=np.eye(3).reshape(-1).copy(), voxel=small.voxel, mu=small.mu)
    checked = 0
    for i in range(s.n_refl):
        xr, sr = oracle.rotate(s, i)
        o = oracle.leg_detail(s.coords, sr, xr, s.voxel, s.label)
        if (o["status"] != 0).any():
            continue
        checked += 1
        assert_legs_equal(tracer.leg_detail(s.label, s.coords, sr, xr, s.voxel), o)
    assert checked >= 5


def test_reference_abort_case_is_an_error(lib, small):
    xr = np.array([-0.6, 0.0, 0.8])
    sr = np.array([0.3, 0.5, 0.81])
    g = tracer.leg_detail(small.label, small.coords[:64], sr, xr, small.voxel)
    assert (g["status"] == 2).any()
    tab, keep = row_table(small.label)
    r = lib.ray_tracing_single(small.coords, len(small.coords), sr, xr, small.voxel, small.mu, tab, small.shape,
                               0, 0, 1)
    assert np.isnan(r) and lib.anacor_last_status() == 2


def test_out_of_range_coordinate_is_an_error(lib, small):
    bad = small.coords[:10].copy()
    bad[3, 2] = small.label.shape[2]
    s = small.subset(refl=slice(0, 2), coords=bad)
    with pytest.raises(_lib.AnacorError):
        tracer.sample_absorption(s)


def test_empty_inputs(lib, small):
    s = small.subset(refl=slice(0, 0))
    assert tracer.sample_absorption(s).shape == (0,)
    e = small.subset(refl=slice(0, 3), coords=np.zeros((0, 3), np.int64))
    assert np.isnan(tracer.sample_absorption(e)).all()   # the reference's 0/0 mean


@pytest.mark.parametrize("which", ["s1", "xray"])
@pytest.mark.parametrize("bad", [np.nan, np.inf, 0.0])
def test_non_finite_or_zero_direction_is_an_error(lib, small, which, bad):
    """A NaN, infinite or zero-length s1 or incident beam: NULL from the drop-in
    and ANACOR_ERR_DIRECTION (7), a raised error from the flat entry point, and
    the next good call unaffected (host-side input, no kernel sees it)."""
    s = small.subset(refl=slice(0, 6))
    s1 = np.array(s.s1, copy=True)
    xray = np.array(s.xray, copy=True)
    if which == "s1":
        s1[4] = bad
    else:
        xray[:] = bad
    t = synth.Sample(label=s.label, coords=s.coords, s1=s1, omega=s.omega, xray=xray, omega_axis=s.omega_axis,
                     F=s.F, voxel=s.voxel, mu=s.mu)
    tab, keep = row_table(s.label)
    res = lib.ray_tracing_overall(0, 6, t.coords, len(t.coords), t.s1, t.omega, t.xray, t.omega_axis, t.F, 6,
                                  t.voxel, t.mu, tab, t.shape, 0, 0, 1, 1)
    assert not res
    assert lib.anacor_last_status() == 7
    with pytest.raises(_lib.AnacorError) as ei:
        tracer.sample_absorption(t)
    assert ei.value.status == 7
    good = lib.ray_tracing_overall(0, 6, s.coords, len(s.coords), s.s1, s.omega, s.xray, s.omega_axis, s.F, 6,
                                   s.voxel, s.mu, tab, s.shape, 0, 0, 1, 1)
    assert good
    got = [good[i] for i in range(6)]
    lib.free(ct.cast(good, ct.c_void_p))
    assert max_rel(got, tracer.sample_absorption(s)) == 0.0


def test_block_shape_guard(lib):
    """The absorption kernel refuses a block shape its shared arrays are not
    sized for: status bit 1 << ANACOR_ERR_ARGS, no access (128 threads: inside
    the arrays, so even an unguarded kernel would stay in bounds)."""
    word = ct.c_int32(-1)
    assert lib.anacor_block_guard_check(128, ct.byref(word)) == 0, lib.anacor_last_error()
    assert word.value == 1 << 3
    assert lib.anacor_block_guard_check(256, ct.byref(word)) == 0
    assert word.value == 0
    assert lib.anacor_block_guard_check(300, ct.byref(word)) == 3   # refused on the host


# --------------------------------------------------- the reference's ABI --

def test_dropin_ray_tracing_overall_like_anacor_worker(lib, small, golden_dir):
    """Called exactly as AnACor/utils/utils_mp.py:197-212 calls it."""
    gold = np.load(os.path.join(golden_dir, "small_ah.npz"))["ah"]
    tab, keep = row_table(small.label)
    n = small.n_refl
    res = lib.ray_tracing_overall(0, n, small.coords, len(small.coords), small.s1, small.omega, small.xray,
                                  small.omega_axis, small.F, n, small.voxel, small.mu, tab, small.shape, 0, 0, 8, 1)
    assert res, lib.anacor_last_error()
    corr = [res[i] for i in range(n)]
    lib.free(ct.cast(res, ct.c_void_p))
    assert max_rel(corr, gold) <= RTOL


@pytest.fixture(scope="module")
def beamline_500():
    return synth.beamline_sample().subset(refl=slice(0, 500))


@pytest.mark.parametrize("which", ["small", "beamline_500"])
def test_dropin_calls_from_several_host_threads(lib, which, request):
    """Concurrent calls (each host thread has its own pinned staging and
    set-up helper; the device stream and tuning cache are shared; a 105 MB
    pageable volume is page-locked for its upload, one call at a time) return
    the answers of one call, bit for bit, every time."""
    import threading
    smp = request.getfixturevalue(which)
    tab, keep = row_table(smp.label)
    n = smp.n_refl

    def call():
        res = lib.ray_tracing_overall(0, n, smp.coords, len(smp.coords), smp.s1, smp.omega, smp.xray,
                                      smp.omega_axis, smp.F, n, smp.voxel, smp.mu, tab, smp.shape, 0, 0, 4, 1)
        assert res, lib.anacor_last_error()
        out = np.array([res[i] for i in range(n)])
        lib.free(ct.cast(res, ct.c_void_p))
        return out

    want = call()
    got, errors = [], []

    def worker():
        try:
            for _ in range(4):
                got.append(call())
        except Exception as ex:   # reported below
            errors.append(ex)

    threads = [threading.Thread(target=worker) for _ in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not any(t.is_alive() for t in threads)
    assert not errors, errors
    assert len(got) == 12
    for g in got:
        assert np.array_equal(g, want)


def test_dropin_calls_keep_device_memory_steady(lib, small):
    """Repeated calls reuse the library pool's memory: after the first call
    the device's free memory does not move (no leak, no growing reservation)."""
    import torch
    tab, keep = row_table(small.label)
    n = small.n_refl
    free = []
    for _ in range(4):
        res = lib.ray_tracing_overall(0, n, small.coords, len(small.coords), small.s1, small.omega, small.xray,
                                      small.omega_axis, small.F, n, small.voxel, small.mu, tab, small.shape, 0, 0,
                                      4, 1)
        assert res, lib.anacor_last_error()
        lib.free(ct.cast(res, ct.c_void_p))
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
    assert free[1] == free[2] == free[3], free


def test_dropin_non_contiguous_row_table(lib, small, oracle):
    # rows of the table scattered in memory: the library gathers them
    s = small.subset(refl=slice(0, 5))
    Z, Y, X = s.label.shape
    rows = [np.ascontiguousarray(s.label[z, y]).copy() for z in range(Z) for y in range(Y)]
    P = ct.POINTER(ct.c_int8)
    plane = [(P * Y)(*[rows[z * Y + y].ctypes.data_as(P) for y in range(Y)]) for z in range(Z)]
    cube = (ct.POINTER(P) * Z)(*[ct.cast(p, ct.POINTER(P)) for p in plane])
    tab = ct.cast(cube, ct.POINTER(ct.POINTER(P)))
    res = lib.ray_tracing_overall(0, 5, s.coords, len(s.coords), s.s1, s.omega, s.xray, s.omega_axis, s.F, 5,
                                  s.voxel, s.mu, tab, s.shape, 0, 0, 1, 1)
    assert res, lib.anacor_last_error()
    got = [res[i] for i in range(5)]
    lib.free(ct.cast(res, ct.c_void_p))
    assert max_rel(got, oracle.overall(s, threads=4)) <= RTOL


def test_dropin_ray_tracing_single(lib, small, oracle):
    tab, keep = row_table(small.label)
    for i in (0, 7, 99):
        xr, sr = oracle.rotate(small, i)
        got = lib.ray_tracing_single(small.coords, len(small.coords), sr, xr, small.voxel, small.mu, tab,
                                     small.shape, 0, 0, 1)
        want = oracle.single(small.coords, sr, xr, small.voxel, small.mu, small.label)
        assert abs(got - want) <= RTOL * want


def test_dropin_float_abi(lib, small, oracle):
    """ray_tracing_gpu_overall: FP32 arguments widened to FP64 on entry."""
    s = small.subset(refl=slice(0, 16))
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
    tab, keep = row_table(s.label)
    res = lib.ray_tracing_gpu_overall(0, 16, s.coords.astype(np.int32), len(s.coords), f32(s.s1), f32(s.omega),
                                      f32(s.xray), f32(s.omega_axis), f32(s.F), 16, f32(s.voxel), f32(s.mu), tab,
                                      s.label.ctypes.data_as(ct.POINTER(ct.c_int8)), s.shape.astype(np.int32),
                                      0, 0, 1)
    assert res, lib.anacor_last_error()
    got = np.array([res[i] for i in range(16)])
    lib.free(ct.cast(res, ct.c_void_p))
    w = lambda a: np.asarray(a, dtype=np.float32).astype(np.float64)  # noqa: E731
    t = synth.Sample(label=s.label, coords=s.coords, s1=w(s.s1), omega=w(s.omega), xray=w(s.xray),
                     omega_axis=w(s.omega_axis), F=w(s.F), voxel=w(s.voxel), mu=w(s.mu))
    assert max_rel(got, oracle.overall(t, threads=4)) <= 2e-6


def test_batch_of_samples_one_launch(lib, oracle):
    samples = synth.batch_samples(n_samples=3, max_refl=20, dim_range=(64, 128))
    plans = [tracer.Plan.from_sample(s) for s in samples]
    tracer.batch_run(plans)
    for s, p in zip(samples, plans):
        assert max_rel(p.result(), oracle.overall(s, threads=os.cpu_count() or 1)) <= RTOL
        p.close()


@pytest.mark.parametrize("shape", ["sphere", "cylinder"])
def test_known_answer_volumes(lib, golden_dir, shape):
    """The analytic sphere and cylinder sets (reference values and analytic
    transmission factors in tests/golden): ray_tracing_single on the GPU gives
    the reference's A_h within 1e-6 for every mu*r and 2theta."""
    from tests.golden.make_golden import cylinder_directions, cylinder_volume, sphere_directions, sphere_volume
    g = np.load(os.path.join(golden_dir, f"{shape}_kat.npz"))
    if shape == "sphere":
        vol, dirs = sphere_volume(24), sphere_directions(g["two_theta"])
    else:
        vol, dirs = cylinder_volume(24, 2), cylinder_directions(g["two_theta"])
    tab, keep = row_table(vol)
    voxel = np.array([0.5] * 3)
    coords = np.ascontiguousarray(g["coords"])
    for k, mur in enumerate(g["mur"]):
        mu = np.array([0.0, 0.0, mur / (24 * 0.5), 0.0])
        for j, (xr, sr) in enumerate(dirs):
            got = lib.ray_tracing_single(coords, len(coords), np.ascontiguousarray(sr), np.ascontiguousarray(xr),
                                         voxel, mu, tab, np.array(vol.shape, dtype=np.int64), 0, 0, 1)
            want = g["reference"][k][j]
            assert abs(got - want) <= RTOL * want, (shape, mur, j, got, want)
    del keep
