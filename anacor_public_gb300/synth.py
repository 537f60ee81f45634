"""Seeded synthetic samples for the absorption-correction path.

A sample is what AnACor's driver hands to the native library
(``AnACor/main_lite.py:93-225`` -> ``AnACor/utils/utils_mp.py:197``):

* ``label``    int8 [Z, Y, X] C-contiguous segmentation volume using AnACor's
               label codes (``AnACor/src/ray_tracing_basic.c:350-387``):
               0 vacuum, 1 liquor, 2 loop, 3 crystal, 4 bubble.
* ``coords``   int64 [N, 3] C-contiguous (z, y, x) crystal voxels in ``np.where``
               order (``AnACor/utils/utils_rt.py:50-51``), optionally stride-sampled.
* ``s1``       float64 [R, 3] diffracted unit vectors (DIALS lab frame).
* ``omega``    float64 [R] rotation angles (rad).
* ``xray``     float64 [3] incident propagation direction (``utils_mp.py:47``).
* ``omega_axis`` float64 [3]; ``F`` float64 [9] fixed goniometer matrix.
* ``voxel``    float64 [3] (z, y, x) voxel edge (um); ``mu`` float64 [4] in
               AnACor's coefficient order [liquor, loop, crystal, bubble]
               (``AnACor/main_lite.py:207``).

The recipe: a crystal ellipsoid with seeded Euler orientation, a liquor shell a
fixed number of voxels thicker, a torus loop in a seeded plane through the
centre, two bubble spheres centred inside the liquor, and reflections with
omega ~ U[0, 2pi), 2theta ~ U[5 deg, 120 deg] about the incident beam and a
uniform azimuth.  Every array is built from ``numpy.random.default_rng(seed)``.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

VACUUM, LIQUOR, LOOP, CRYSTAL, BUBBLE = 0, 1, 2, 3, 4

# incident propagation direction and goniometer used for every synthetic sample
XRAY = np.array([-1.0, 0.0, 0.0])
OMEGA_AXIS = np.array([0.0, 1.0, 0.0])
F_IDENTITY = np.eye(3).reshape(-1).copy()


@dataclasses.dataclass
class Sample:
    label: np.ndarray
    coords: np.ndarray
    s1: np.ndarray
    omega: np.ndarray
    xray: np.ndarray
    omega_axis: np.ndarray
    F: np.ndarray
    voxel: np.ndarray
    mu: np.ndarray
    name: str = ""

    @property
    def shape(self) -> np.ndarray:
        return np.array(self.label.shape, dtype=np.int64)

    @property
    def n_refl(self) -> int:
        return int(self.omega.shape[0])

    def subset(self, refl: slice | np.ndarray | None = None, coords=None) -> "Sample":
        return dataclasses.replace(
            self,
            s1=np.ascontiguousarray(self.s1[refl]) if refl is not None else self.s1,
            omega=np.ascontiguousarray(self.omega[refl]) if refl is not None else self.omega,
            coords=np.ascontiguousarray(coords) if coords is not None else self.coords,
        )


def euler_matrix(a: float, b: float, c: float) -> np.ndarray:
    """z-y-z Euler rotation."""
    ca, sa, cb, sb, cc, sc = math.cos(a), math.sin(a), math.cos(b), math.sin(b), math.cos(c), math.sin(c)
    rz1 = np.array([[ca, -sa, 0], [sa, ca, 0], [0, 0, 1]])
    ry = np.array([[cb, 0, sb], [0, 1, 0], [-sb, 0, cb]])
    rz2 = np.array([[cc, -sc, 0], [sc, cc, 0], [0, 0, 1]])
    return rz1 @ ry @ rz2


def build_volume(shape, semi_axes, shell, torus_R, torus_r, bubble_r, rng,
                 n_bubbles: int = 2, slab: int = 32) -> np.ndarray:
    """Paint liquor, loop, bubbles and crystal into an int8 [Z, Y, X] volume.

    Paint order: liquor ellipsoid (crystal semi-axes + ``shell``), torus loop
    over vacuum, bubbles over liquor only, crystal last.  Built in z-slabs so
    the 1024x1024x800 volume needs no full-size float temporaries.
    """
    Z, Y, X = (int(s) for s in shape)
    vol = np.zeros((Z, Y, X), dtype=np.int8)
    centre = np.array([(Z - 1) / 2.0, (Y - 1) / 2.0, (X - 1) / 2.0])
    rot = euler_matrix(*rng.uniform(0.0, 2.0 * math.pi, size=3))
    a = np.asarray(semi_axes, dtype=np.float64)
    aliq = a + shell
    normal = rng.normal(size=3)
    normal /= np.linalg.norm(normal)

    yy = np.arange(Y, dtype=np.float64)[None, :, None] - centre[1]
    xx = np.arange(X, dtype=np.float64)[None, None, :] - centre[2]
    for z0 in range(0, Z, slab):
        z1 = min(Z, z0 + slab)
        zz = np.arange(z0, z1, dtype=np.float64)[:, None, None] - centre[0]
        # body-frame coordinates q = rot^T (p - c)
        q = [rot[0, k] * zz + rot[1, k] * yy + rot[2, k] * xx for k in range(3)]
        liq = (q[0] / aliq[0]) ** 2 + (q[1] / aliq[1]) ** 2 + (q[2] / aliq[2]) ** 2 <= 1.0
        cry = (q[0] / a[0]) ** 2 + (q[1] / a[1]) ** 2 + (q[2] / a[2]) ** 2 <= 1.0
        del q
        # torus around `normal` through the centre
        h = normal[0] * zz + normal[1] * yy + normal[2] * xx
        rho2 = zz * zz + yy * yy + xx * xx - h * h
        rho = np.sqrt(np.maximum(rho2, 0.0))
        tor = (rho - torus_R) ** 2 + h * h <= torus_r ** 2
        del h, rho2, rho
        blk = vol[z0:z1]
        blk[liq] = LIQUOR
        blk[tor & ~liq] = LOOP
        blk[cry] = CRYSTAL
    # bubbles centred on uniformly chosen liquor voxels
    liq_idx = np.flatnonzero(vol.reshape(-1) == LIQUOR)
    if liq_idx.size:
        for _ in range(n_bubbles):
            cz, cy, cx = np.unravel_index(liq_idx[rng.integers(liq_idx.size)], (Z, Y, X))
            rr = int(math.ceil(bubble_r))
            zs, ys, xs = (slice(max(0, c - rr), min(n, c + rr + 1)) for c, n in ((cz, Z), (cy, Y), (cx, X)))
            sub = vol[zs, ys, xs]
            gz, gy, gx = np.meshgrid(np.arange(zs.start, zs.stop) - cz, np.arange(ys.start, ys.stop) - cy,
                                     np.arange(xs.start, xs.stop) - cx, indexing="ij")
            ball = gz * gz + gy * gy + gx * gx <= bubble_r * bubble_r
            sub[ball & (sub == LIQUOR)] = BUBBLE
    return vol


def crystal_coords(vol: np.ndarray, stride: int = 1) -> np.ndarray:
    """(z, y, x) crystal voxels in ``np.where`` order, C-contiguous int64.

    ``stride`` keeps voxels whose three indices are multiples of it.
    """
    if stride > 1:
        sub = vol[::stride, ::stride, ::stride]
        c = np.argwhere(sub == CRYSTAL) * stride
    else:
        c = np.argwhere(vol == CRYSTAL)
    return np.ascontiguousarray(c.astype(np.int64))


def reflections(n: int, rng, xray=XRAY, two_theta=(5.0, 120.0)):
    """omega ~ U[0,2pi); s1 at 2theta ~ U[two_theta] from ``xray``, uniform azimuth."""
    omega = rng.uniform(0.0, 2.0 * math.pi, size=n)
    tth = np.deg2rad(rng.uniform(two_theta[0], two_theta[1], size=n))
    az = rng.uniform(0.0, 2.0 * math.pi, size=n)
    b = np.asarray(xray, dtype=np.float64)
    b = b / np.linalg.norm(b)
    helper = np.array([0.0, 0.0, 1.0]) if abs(b[2]) < 0.9 else np.array([0.0, 1.0, 0.0])
    u = np.cross(b, helper)
    u /= np.linalg.norm(u)
    v = np.cross(b, u)
    s1 = (np.cos(tth)[:, None] * b[None, :]
          + (np.sin(tth) * np.cos(az))[:, None] * u[None, :]
          + (np.sin(tth) * np.sin(az))[:, None] * v[None, :])
    return np.ascontiguousarray(omega), np.ascontiguousarray(s1)


MU_BASE = np.array([0.010, 0.007, 0.012, 0.0])  # [liquor, loop, crystal, bubble] um^-1


def make_sample(shape=(96, 96, 96), scale: float = 1.0, n_refl: int = 300, stride: int = 1,
                seed: int = 0, mu=MU_BASE, voxel=0.3, semi_axes=(20.0, 14.0, 10.0),
                shell=6.0, torus=(30.0, 3.0), bubble_r=3.0, name: str = "") -> Sample:
    rng = np.random.default_rng(seed)
    vol = build_volume(shape, np.asarray(semi_axes) * scale, shell * scale, torus[0] * scale,
                       torus[1] * scale, bubble_r * scale, rng)
    coords = crystal_coords(vol, stride)
    omega, s1 = reflections(n_refl, rng)
    # fixed goniometer setting (the kappa/phi product F of AnACor/main_lite.py:211-225),
    # seeded so that rotated directions have no exactly-zero component
    F = np.ascontiguousarray(euler_matrix(*rng.uniform(0.0, 2.0 * math.pi, size=3)).reshape(-1))
    return Sample(label=vol, coords=coords, s1=s1, omega=omega, xray=XRAY.copy(),
                  omega_axis=OMEGA_AXIS.copy(), F=F,
                  voxel=np.array([voxel, voxel, voxel], dtype=np.float64),
                  mu=np.asarray(mu, dtype=np.float64).copy(), name=name)


def small_sample(n_refl: int = 300, seed: int = 0) -> Sample:
    """96^3 volume, crystal semi-axes 20/14/10, every crystal voxel, 300 reflections."""
    return make_sample(n_refl=n_refl, seed=seed, name="small_96cube_all_voxels")


def beamline_sample(n_refl: int = 20000, stride: int = 4, seed: int = 1) -> Sample:
    """512x512x400 volume (recipe scaled x5), crystal voxels at stride 4, 20k reflections."""
    return make_sample(shape=(512, 512, 400), scale=5.0, n_refl=n_refl, stride=stride, seed=seed,
                       name="beamline_512x512x400_stride4")


def high_absorption_sample(n_refl: int = 50000, stride: int = 1, seed: int = 4) -> Sample:
    """1024x1024x800 volume (recipe scaled x10), every crystal voxel, mu x5."""
    return make_sample(shape=(1024, 1024, 800), scale=10.0, n_refl=n_refl, stride=stride, seed=seed,
                       mu=MU_BASE * 5.0, name="highabs_1024x1024x800")


def batch_samples(n_samples: int = 12, seed: int = 2, refl_range=(2000, 60000),
                  dim_range=(128, 640), max_refl: int | None = None, voxel_budget: int = 60000,
                  strides=(2, 4, 8), only: int | None = None):
    """Independent samples with log-uniform dimensions, crystal diameters 15-40%
    of the smallest dimension, the same label recipe, mu jittered +-30% and
    log-uniform reflection counts.  ``only=k`` builds sample k alone (the
    same sample as in the full list) and returns it in a one-element list.

    The crystal-voxel sampling stride of each sample is the smallest of
    `strides` that keeps its voxel list within `voxel_budget` (the largest
    stride otherwise).  Axes are sorted so the largest is last (the reference's
    path buffer holds x_max*sqrt(3) entries, ``AnACor/src/ray_tracing_basic.c:402-406``).
    """
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_samples):
        dims = np.exp(rng.uniform(math.log(dim_range[0]), math.log(dim_range[1]), size=3)).astype(int)
        dims = np.sort(dims)[::-1].copy()
        dims = np.array([dims[1], dims[2], dims[0]])
        frac = rng.uniform(0.15, 0.40, size=3)
        semi = frac * float(np.min(dims)) / 2.0
        n_refl = int(math.exp(rng.uniform(math.log(refl_range[0]), math.log(refl_range[1]))))
        if max_refl is not None:
            n_refl = min(n_refl, max_refl)
        mu = MU_BASE * rng.uniform(0.7, 1.3, size=4)
        scale = float(np.min(dims)) / 96.0
        sample_seed = int(rng.integers(1 << 30))
        if only is not None and k != only:
            continue
        # the loop grazes the liquor so that rays can cross liquor -> loop
        s = make_sample(shape=tuple(int(d) for d in dims), n_refl=n_refl, seed=sample_seed, mu=mu,
                        semi_axes=tuple(semi), shell=6.0 * scale,
                        torus=(float(np.max(semi)) + 7.0 * scale, 3.0 * scale),
                        bubble_r=3.0 * scale, name=f"batch{k}")
        n_all = int(np.count_nonzero(s.label == CRYSTAL))
        stride = strides[-1]
        for st in strides:
            if n_all / st ** 3 <= voxel_budget:
                stride = st
                break
        s.coords = crystal_coords(s.label, stride)
        s.name = f"batch{k}_stride{stride}"
        out.append(s)
    return out
