"""The distance-field skip rule on the CPU (no GPU): on random labelled volumes
and random rays, every increment a skip steps over carries the label of the
increment the skip starts from, for the centred field (D = chessboard distance
to another label) and for the octant fields (1 + the largest one-label corner
box toward the ray's signs).  The rule is the kernels':

    n = min(D - 1, ((D - 2) * rq) >> 16),  rq = floor(2^16 / qmax) - 1

and the ray is the reference's march: the step axis moves by exactly 1 per
increment, the other two by R(c + i q) with R = floor or round (q = ratio).
"""
import math

import numpy as np
from scipy import ndimage as nd

CAP = 31


def centred_field(lab):
    D = np.ones(lab.shape, np.int32)
    alive = np.ones(lab.shape, bool)
    for r in range(1, CAP):
        mx = nd.maximum_filter(lab, size=2 * r + 1, mode="nearest")
        mn = nd.minimum_filter(lab, size=2 * r + 1, mode="nearest")
        alive &= (mx == lab) & (mn == lab)
        if not alive.any():
            break
        D[alive] = r + 1
    return D


def octant_field(lab, signs):
    D = np.ones(lab.shape, np.int32)
    alive = np.ones(lab.shape, bool)
    for r in range(1, CAP):
        size = r + 1
        origin = [-(size // 2) if sg > 0 else (size - 1) - size // 2 for sg in signs]
        mx = nd.maximum_filter(lab, size=size, origin=origin, mode="nearest")
        mn = nd.minimum_filter(lab, size=size, origin=origin, mode="nearest")
        alive &= (mx == lab) & (mn == lab)
        if not alive.any():
            break
        D[alive] = r + 1
    return D


def volume(shape, seed):
    rng = np.random.default_rng(seed)
    lab = np.zeros(shape, np.int16)
    for _ in range(30):
        lo = [int(rng.integers(0, d)) for d in shape]
        hi = [min(d, l + int(rng.integers(2, max(3, d // 2)))) for l, d in zip(lo, shape)]
        lab[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] = rng.integers(1, 8)
    return lab


def nmax(D, rq):
    return 0 if D < 2 else min(D - 1, ((D - 2) * rq) >> 16)


def test_skips_never_cross_a_label_change():
    rng = np.random.default_rng(11)
    violations = skipped = 0
    for seed in range(3):
        lab = volume((40, 44, 48), seed)
        shape = np.array(lab.shape)
        cen = centred_field(lab)
        octs = {}
        for _ in range(400):
            s = int(rng.integers(0, 3))                      # step axis
            q = rng.uniform(-2.0, 2.0, 3)
            q[s] = rng.choice([-1.0, 1.0])
            use_round = bool(rng.integers(0, 2))
            c = np.array([int(rng.integers(0, d)) for d in shape])
            others = [a for a in range(3) if a != s]
            qmax = max(abs(q[a]) for a in others)
            rq = (1 << 22) if qmax < 1 / 64 else max(0, math.floor(65536.0 / qmax) - 1)
            signs = tuple(1 if q[a] >= 0 else -1 for a in range(3))
            if signs not in octs:
                octs[signs] = octant_field(lab, signs)

            def point(i):
                p = np.empty(3, np.int64)
                for a in range(3):
                    x = c[a] + i * q[a]
                    p[a] = math.floor(x + 0.5) if (use_round and a != s) else math.floor(x)
                return p

            for field in (cen, octs[signs]):
                i = 0
                while True:
                    p = point(i)
                    if np.any(p < 0) or np.any(p >= shape):
                        break
                    n = nmax(int(field[tuple(p)]), rq)
                    for j in range(i + 1, i + n + 1):
                        pj = point(j)
                        if np.any(pj < 0) or np.any(pj >= shape):
                            break
                        skipped += 1
                        violations += int(lab[tuple(pj)] != lab[tuple(p)])
                    i += n + 1
    assert skipped > 10000
    assert violations == 0
