"""Generate the golden fixtures in this directory from the reference library.

Run in a container that holds the reference sources (they are compiled by
``make -C oracle ref`` into ``oracle/_ref/ray_tracing_cpu.so``):

    python tests/golden/make_golden.py

Fixtures (all small):
  small_ah.npz      A_h of every reflection of the 96^3 sample (seed 0, 300
                    reflections, all crystal voxels) from the reference's
                    ray_tracing_overall, plus checksums of the generated inputs.
  small_legs.npz    per-voxel, per-leg detail (exit face, len_path_2, number of
                    class segments, last path point, four lengths) from the
                    reference's cube_face / cal_coord / cal_path2_plus for a
                    voxel subset of 8 reflections.
  beamline_ah.npz   A_h of 12 reflections of the 512x512x400 stride-4 sample.
  small_ib.npz      A_h of 30 reflections of the 96^3 sample from the
                    reference's ib_test (iterative bisection), num_cls 4 and 3.
  small_grid.npz    ray_tracing_single_gridding values (the gridding map) of
                    64 voxels for 8 grid directions of a 36 x 18 grid, with the
                    direction vectors built as the reference's gridding does.
  sphere_kat.npz    A_h of a voxelised sphere at mu*r = 0.1, 0.5, 1 and
                    2theta = linspace(0, 180, 10), from the reference's
                    ray_tracing_single, beside the analytic transmission values
                    that AnACor/verification/sphere_verification_new.py:31-36
                    checks against.
  cylinder_kat.npz  the same for a voxelised cylinder (axis along the
                    volume's first axis, rays perpendicular to it) against the
                    values AnACor/verification/cylinder_verification_new.py:31-33
                    checks against (python make_golden.py --cylinder).

Fixtures at the large workloads (python make_golden.py --large; the volumes
are regenerated from their seeds by the tests, the digests pin them):
  beamline_ah256.npz  A_h of 256 reflections of the 20,000-reflection beamline
                      workload (512x512x400, stride-4 voxels), every voxel.
  highabs_ah.npz      the 1024x1024x800 mu x5 workload (50,000 reflections):
                      A_h of 48 seeded reflections over a seeded 32,768-voxel
                      subset, and the per-voxel, per-leg detail of 2 of them
                      on 2,048 voxels of that subset.
  batch_ah.npz        the largest-volume sample of the 12-sample batch
                      (347x288x578, mu jittered): A_h of 48 seeded reflections
                      over all its stride-sampled voxels, and the per-leg
                      detail of 1 reflection on 2,048 voxels.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from anacor_public_gb300 import synth  # noqa: E402
from oracle import oracle as orc  # noqa: E402

# the reference checkout's C sources, compiled into oracle/_ref
REFERENCE_SRC = os.environ.get("ANACOR_REFERENCE_SRC", "/root/reference/AnACor/src")

# analytic sphere transmission factors at 2theta = linspace(0, 180, 10)
# (AnACor/verification/sphere_verification_new.py:31-36)
SPHERE_ANALYTIC = {
    0.1: [0.86140064, 0.86140064, 0.8616233, 0.86206897, 0.86258949,
          0.86311065, 0.86363244, 0.86415486, 0.86445367, 0.8645284],
    0.5: [0.48181161, 0.4829518, 0.48626307, 0.49164208, 0.49860391,
          0.50645733, 0.51427102, 0.52099614, 0.52565181, 0.52731491],
    1.0: [0.24250067, 0.24500796, 0.25236593, 0.26373395, 0.27777006,
          0.29295445, 0.30770178, 0.32034854, 0.32913142, 0.33233632],
}
SPHERE_RADIUS = 24          # voxels
SPHERE_VOXEL = 0.5          # um

# analytic cylinder transmission factors at 2theta = linspace(0, 180, 10),
# rays perpendicular to the axis (AnACor/verification/cylinder_verification_new.py:31-33)
CYLINDER_ANALYTIC = {
    0.1: [0.84438065, 0.84445195, 0.84473729, 0.84516565, 0.84580902,
          0.84652501, 0.84731401, 0.84796065, 0.8483923, 0.84853627],
    0.5: [0.43485824, 0.43618599, 0.44012147, 0.44646843, 0.45462811,
          0.46373586, 0.47276853, 0.4805613, 0.48593226, 0.48787627],
    1.0: [0.19643664, 0.19926273, 0.2074861, 0.22007527, 0.23551023,
          0.25211779, 0.26819718, 0.28199199, 0.29158769, 0.29510712],
}
CYLINDER_RADIUS = 24        # voxels
CYLINDER_LENGTH = 2         # voxels along the axis (rays never move along it)
CYLINDER_VOXEL = 0.5        # um


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def sample_digest(s) -> str:
    return digest(s.label, s.coords, s.s1, s.omega, s.xray, s.omega_axis, s.F, s.voxel, s.mu)


def sphere_volume(radius: int):
    n = 3 * radius
    c = n / 2 - 1
    g = np.arange(n, dtype=np.float64) - c
    zz, yy, xx = np.meshgrid(g, g, g, indexing="ij", sparse=True)
    vol = np.where(zz ** 2 + yy ** 2 + xx ** 2 < radius ** 2, 3, 0).astype(np.int8)
    return np.ascontiguousarray(vol)


def cylinder_volume(radius: int, length: int):
    """Crystal (label 3) cylinder of `radius` voxels whose axis runs along the
    volume's first axis, in a (length, 3r, 3r) volume."""
    n = 3 * radius
    c = n / 2 - 1
    g = np.arange(n, dtype=np.float64) - c
    yy, xx = np.meshgrid(g, g, indexing="ij")
    disc = np.where(yy ** 2 + xx ** 2 < radius ** 2, 3, 0).astype(np.int8)
    return np.ascontiguousarray(np.repeat(disc[None, :, :], length, axis=0))


def cylinder_directions(two_theta_deg):
    """Rotated incident / diffracted vectors at scattering angle 2theta, both
    perpendicular to the cylinder axis: the volume's first axis is the DIALS
    x component (the march frame swaps DIALS y and z), so both lie in the
    DIALS y-z plane, at a generic angle to its axes."""
    a0 = 0.37
    out = []
    for t in np.deg2rad(two_theta_deg):
        b = np.array([0.0, np.cos(a0), np.sin(a0)])
        s = np.array([0.0, np.cos(a0 + t), np.sin(a0 + t)])
        out.append((b, s))
    return out


def cylinder_kat(ref):
    vol = cylinder_volume(CYLINDER_RADIUS, CYLINDER_LENGTH)
    coords = np.ascontiguousarray(np.argwhere(vol == 3).astype(np.int64))[::5]
    tth = np.linspace(0, 180, 10)
    voxel = np.array([CYLINDER_VOXEL] * 3)
    res = {}
    for mur in (0.1, 0.5, 1.0):
        mu = np.array([0.0, 0.0, mur / (CYLINDER_RADIUS * CYLINDER_VOXEL), 0.0])
        res[mur] = [ref.single(coords, sr, xr, voxel, mu, vol) for xr, sr in cylinder_directions(tth)]
    np.savez_compressed(os.path.join(HERE, "cylinder_kat.npz"), coords=coords, two_theta=tth,
                        mur=np.array([0.1, 0.5, 1.0]),
                        reference=np.array([res[m] for m in (0.1, 0.5, 1.0)]),
                        analytic=np.array([CYLINDER_ANALYTIC[m] for m in (0.1, 0.5, 1.0)]))
    for m in (0.1, 0.5, 1.0):
        err = np.abs(np.array(res[m]) - CYLINDER_ANALYTIC[m]) / np.array(CYLINDER_ANALYTIC[m])
        print("cylinder mu*r", m, "max rel err vs analytic", err.max())


def sphere_directions(two_theta_deg):
    """Rotated incident / diffracted vectors at scattering angle 2theta, in a
    generic orientation (no exactly-zero component)."""
    rot = synth.euler_matrix(0.3, 1.1, 2.0)
    b = np.array([-1.0, 0.0, 0.0])
    out = []
    for t in np.deg2rad(two_theta_deg):
        s = np.array([-np.cos(t), np.sin(t) * 0.6, np.sin(t) * 0.8])
        out.append((rot @ b, rot @ s))
    return out


def bisection_and_gridding(ref):
    """Fixtures of the bisection and gridding modes (python make_golden.py --modes)."""
    from oracle import gridding_oracle as go
    s = synth.small_sample()
    o = orc.Oracle()
    refl = np.arange(0, s.n_refl, 10)
    ib = {}
    for ncls in (4, 3):
        vals = []
        for i in refl:
            xr, sr = o.rotate(s, int(i))
            vals.append(ref.ib_test(s.coords, sr, xr, s.voxel, s.mu, s.label, ncls))
        ib[ncls] = vals
    np.savez_compressed(os.path.join(HERE, "small_ib.npz"), refl=refl, ib4=np.array(ib[4]), ib3=np.array(ib[3]),
                        digest=sample_digest(s))
    s1, th, ph = go.directions(36, 18)
    rng = np.random.default_rng(0)
    dirs = np.sort(rng.choice(len(s1), 8, replace=False))
    vox = np.ascontiguousarray(s.coords[np.sort(rng.choice(len(s.coords), 64, replace=False))])
    vals, angles = [], []
    for d in dirs:
        tp = ref.lib.dials_2_thetaphi_22(np.ascontiguousarray(s1[d]).copy(), 0)
        angles.append((tp.theta, tp.phi))
        vals.append(ref.single_gridding(vox, s1[d], tp.theta, tp.phi, s.voxel, s.mu, s.label))
    np.savez_compressed(os.path.join(HERE, "small_grid.npz"), dirs=dirs, s1=s1[dirs], angles=np.array(angles),
                        coords=vox, value=np.array(vals))
    print("ib", ib[4][:3], "grid", vals[0][:3])
    ib_grid_fixture(ref)


def ib_grid_fixture(ref):
    """ib_single_gridding values of 64 voxels x 8 grid directions of a 36 x 18
    grid, num_cls 4 and 3, exponent and exp (python make_golden.py --ib-grid)."""
    from oracle import gridding_oracle as go
    s = synth.small_sample()
    s1, th, ph = go.directions(36, 18)
    rng = np.random.default_rng(1)
    dirs = np.sort(rng.choice(len(s1), 8, replace=False))
    vox = np.ascontiguousarray(s.coords[np.sort(rng.choice(len(s.coords), 64, replace=False))])
    out = {}
    for ncls in (4, 3):
        for ex in (0, 1):
            out[f"v{ncls}_{ex}"] = np.array([ref.ib_single_gridding(vox, s1[d], th[d], ph[d], s.voxel, s.mu,
                                                                    s.label, ncls, ex) for d in dirs])
    np.savez_compressed(os.path.join(HERE, "small_ib_grid.npz"), dirs=dirs, s1=s1[dirs],
                        angles=np.stack([th[dirs], ph[dirs]], 1), coords=vox, digest=sample_digest(s), **out)
    print("ib grid", out["v4_0"][0][:3])


def _legs(ref, s, k, coords):
    """Reference per-voxel, per-leg detail of reflection k of sample s."""
    xr, sr = orc.Oracle().rotate(s, int(k))
    d = ref.leg_detail(coords, sr, xr, s.voxel, s.label)
    return {key: d[key] for key in ("face", "len", "nseg", "first", "last", "L")}


def large_fixtures(ref):
    nw = os.cpu_count() or 1
    b = synth.beamline_sample()
    rsel = np.arange(256, dtype=np.int64) * (b.n_refl // 256)
    ah = ref.overall(b.subset(refl=rsel), num_workers=nw)
    np.savez_compressed(os.path.join(HERE, "beamline_ah256.npz"), refl=rsel, ah=ah, digest=sample_digest(b))
    print("beamline256", ah[:3])
    del b

    h = synth.high_absorption_sample()
    rng = np.random.default_rng(44)
    vsel = np.sort(rng.choice(len(h.coords), 32768, replace=False)).astype(np.int32)
    rsel = np.sort(rng.choice(h.n_refl, 48, replace=False)).astype(np.int64)
    hs = h.subset(refl=rsel, coords=h.coords[vsel])
    ah = ref.overall(hs, num_workers=nw)
    lsel = np.arange(0, len(vsel), 16)
    legs = [_legs(ref, hs, k, hs.coords[lsel]) for k in (0, 1)]
    np.savez_compressed(os.path.join(HERE, "highabs_ah.npz"), refl=rsel, voxels=vsel, ah=ah, digest=sample_digest(h),
                        leg_refl=np.array([0, 1]), leg_voxels=lsel,
                        **{f"leg_{key}": np.array([g[key] for g in legs]) for key in legs[0]})
    print("highabs", ah[:3])
    del h, hs

    bs = synth.batch_samples()
    k = int(np.argmax([np.prod(x.label.shape) for x in bs]))
    s = bs[k]
    del bs
    rng = np.random.default_rng(45)
    rsel = np.sort(rng.choice(s.n_refl, 48, replace=False)).astype(np.int64)
    ss = s.subset(refl=rsel)
    ah = ref.overall(ss, num_workers=nw)
    lsel = np.linspace(0, len(s.coords), 2048, endpoint=False).astype(np.int64)
    legs = [_legs(ref, ss, 0, s.coords[lsel])]
    np.savez_compressed(os.path.join(HERE, "batch_ah.npz"), sample=k, refl=rsel, ah=ah, digest=sample_digest(s),
                        leg_refl=np.array([0]), leg_voxels=lsel,
                        **{f"leg_{key}": np.array([g[key] for g in legs]) for key in legs[0]})
    print("batch", k, s.label.shape, len(s.coords), ah[:3])


def main():
    orc.build_oracle(ref_src=REFERENCE_SRC)
    ref = orc.Reference()
    if "--large" in sys.argv:
        large_fixtures(ref)
        return
    if "--modes" in sys.argv:
        bisection_and_gridding(ref)
        return
    if "--ib-grid" in sys.argv:
        ib_grid_fixture(ref)
        return
    if "--cylinder" in sys.argv:
        cylinder_kat(ref)
        return

    s = synth.small_sample()
    ah = ref.overall(s, num_workers=os.cpu_count() or 1)
    np.savez_compressed(os.path.join(HERE, "small_ah.npz"), ah=ah, digest=sample_digest(s))

    o = orc.Oracle()
    legs = {k: [] for k in ("refl", "face", "len", "nseg", "last", "L")}
    sel = np.ascontiguousarray(s.coords[::23])
    for i in range(0, s.n_refl, 37):
        xr, sr = o.rotate(s, i)
        d = ref.leg_detail(sel, sr, xr, s.voxel, s.label)
        legs["refl"].append(i)
        for k in ("face", "len", "nseg", "last", "L"):
            legs[k].append(d[k])
    np.savez_compressed(os.path.join(HERE, "small_legs.npz"), coords=sel,
                        **{k: np.array(v) for k, v in legs.items()})

    b = synth.beamline_sample(n_refl=12)
    ahb = ref.overall(b, num_workers=os.cpu_count() or 1)
    np.savez_compressed(os.path.join(HERE, "beamline_ah.npz"), ah=ahb, digest=sample_digest(b))

    vol = sphere_volume(SPHERE_RADIUS)
    coords = np.ascontiguousarray(np.argwhere(vol == 3).astype(np.int64))[::7]
    tth = np.linspace(0, 180, 10)
    res = {}
    voxel = np.array([SPHERE_VOXEL] * 3)
    for mur in (0.1, 0.5, 1.0):
        mu = np.array([0.0, 0.0, mur / (SPHERE_RADIUS * SPHERE_VOXEL), 0.0])
        res[mur] = [ref.single(coords, sr, xr, voxel, mu, vol) for xr, sr in sphere_directions(tth)]
    np.savez_compressed(os.path.join(HERE, "sphere_kat.npz"), coords=coords, two_theta=tth,
                        mur=np.array([0.1, 0.5, 1.0]),
                        reference=np.array([res[m] for m in (0.1, 0.5, 1.0)]),
                        analytic=np.array([SPHERE_ANALYTIC[m] for m in (0.1, 0.5, 1.0)]))
    print("small_ah", ah[:4], "beamline", ahb[:4])
    for m in (0.1, 0.5, 1.0):
        err = np.abs(np.array(res[m]) - SPHERE_ANALYTIC[m]) / np.array(SPHERE_ANALYTIC[m])
        print("sphere mu*r", m, "max rel err vs analytic", err.max())
    bisection_and_gridding(ref)
    cylinder_kat(ref)


if __name__ == "__main__":
    main()
