"""Properties of the kernel's arithmetic shortcuts, checked on the CPU.

* per-segment quotient: reciprocal table + one FMA correction equals the
  correctly rounded division for every (span, len) the march can produce;
* 32.32 fixed-point march positions: wherever the ambiguity test passes, the
  fixed-point floor equals the reference's floor/round of fl(c + fl(i*q)).
"""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MARGIN = 1 << 14          # anacor::kAmbiguityMargin
FAST_LIMIT = 65536.0      # anacor::kFastRatioLimit
MAX_DIM = 8191            # anacor::kMaxDim


def test_segment_quotient_exhaustive():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "qc")
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-o", exe,
                        os.path.join(HERE, "helpers", "quotient_check.c"), "-lm"], check=True)
        out = subprocess.run([exe, str(MAX_DIM + 1)], check=True, capture_output=True, text=True).stdout.split()
    n, bad = int(out[0]), int(out[1])
    assert n == sum(d + 1 for d in range(1, MAX_DIM + 2))
    assert bad == 0


def c_round(v):
    return np.sign(v) * np.floor(np.abs(v) + 0.5)


def _clamp(n, dim):
    return np.clip(n, 0, dim - 1)


def _check(c, i, q, use_round, dim):
    """Fixed-point positions vs the reference's FP64 expression."""
    Q = np.rint(np.ldexp(q, 32)).astype(np.int64)
    off = np.int64(1 << 31) if use_round else np.int64(0)
    E = (c.astype(np.int64) << 32) + off + i.astype(np.int64) * Q
    hi = E >> 32
    lo = (E & 0xFFFFFFFF).astype(np.uint64)
    amb = ((lo + MARGIN) & 0xFFFFFFFF) < 2 * MARGIN
    v = c.astype(np.float64) + i.astype(np.float64) * q      # fl(c + fl(i*q)), no FMA in numpy
    ref = c_round(v) if use_round else np.floor(v)
    good = ~amb
    assert np.array_equal(_clamp(hi[good], dim), _clamp(ref[good].astype(np.int64), dim))
    return amb.mean()


def test_fixed_point_positions_random():
    rng = np.random.default_rng(7)
    n = 2_000_000
    for use_round in (False, True):
        for scale in (1e-3, 0.3, 1.0, 7.0, 300.0, FAST_LIMIT * 0.999):
            q = rng.uniform(-scale, scale, size=n)
            c = rng.integers(0, MAX_DIM + 1, size=n)
            i = rng.integers(0, MAX_DIM + 2, size=n)
            frac = _check(c, i, q, use_round, MAX_DIM)
            assert frac < 1e-3


def test_fixed_point_positions_near_boundaries():
    # ratios that put c + i*q at or next to integers and half-integers
    rng = np.random.default_rng(8)
    n = 1_000_000
    k = rng.integers(1, 64, size=n)
    num = rng.integers(-512, 512, size=n)
    base = num / k
    for eps in (0.0, 1e-17, 1e-16, 1e-15, 1e-13, 1e-11):
        q = base * (1 + eps * rng.choice([-1.0, 1.0], size=n))
        i = (k * rng.integers(0, 100, size=n)).astype(np.int64)
        i = np.minimum(i, MAX_DIM + 1)
        c = rng.integers(0, 1000, size=n)
        for use_round in (False, True):
            _check(c, i, q, use_round, 4096)
            _check(c, i, q + 0.5 / np.maximum(i, 1), use_round, 4096)


def test_small_integer_ratios_are_exact():
    # integral |q| <= 128 skips the ambiguity test: the fixed point is exact
    for q in (-128.0, -3.0, -1.0, 0.0, 1.0, 2.0, 128.0):
        c = np.arange(0, 200)
        for i in range(0, 300, 7):
            Q = np.int64(np.rint(np.ldexp(q, 32)))
            E = (c.astype(np.int64) << 32) + np.int64(i) * Q
            assert np.array_equal(E >> 32, np.floor(c + i * q).astype(np.int64))
            assert ((E & 0xFFFFFFFF) == 0).all()
