"""Caller-side I/O of the worker mirror (no GPU): the vectorised reflection
parser against the reference worker's per-row ast.literal_eval
(AnACor/utils/utils_mp.py:151-164), bit for bit, and the row table."""
import ctypes as ct
import json
import time
from ast import literal_eval

import numpy as np

from anacor_public_gb300 import worker


def _rows(n, seed=0, as_tuple=False):
    rng = np.random.default_rng(seed)
    s1 = rng.normal(size=(n, 3))
    obs = rng.uniform(-1e3, 1e3, size=(n, 3))
    obs[:, 2] = rng.uniform(0, 2 * np.pi, n)
    rows = []
    for a, b in zip(s1, obs):
        fa = json.dumps([float(x) for x in a])
        fb = json.dumps([float(x) for x in b])
        if as_tuple:
            fa = "(" + fa[1:-1] + ")"
        rows.append({"s1": fa, "xyzobs.mm.value": fb, "intensity.sum.value": "1.0", "miller_index": "(1, 2, 3)"})
    return rows


def _reference_parse(rows, offset):
    s1, om = [], []
    for row in rows:
        s1.append(literal_eval(row["s1"]))
        a = literal_eval(row["xyzobs.mm.value"])[2]
        a += offset / 180 * np.pi
        om.append(a)
    return np.array(s1), np.array(om)


def test_parse_matches_literal_eval():
    for as_tuple in (False, True):
        rows = _rows(5000, seed=1, as_tuple=as_tuple)
        for offset in (0.0, 12.5, -90.0):
            s1, om = worker.parse_reflections(rows, offset)
            r1, ro = _reference_parse(rows, offset)
            assert np.array_equal(s1, r1) and np.array_equal(om, ro)


def test_parse_non_string_rows_and_empty():
    rows = [{"s1": [0.1, 0.2, 0.3], "xyzobs.mm.value": (1.0, 2.0, 3.0)}]
    s1, om = worker.parse_reflections(rows, 0.0)
    assert np.array_equal(s1, [[0.1, 0.2, 0.3]]) and np.array_equal(om, [3.0])
    s1, om = worker.parse_reflections([], 0.0)
    assert s1.shape == (0, 3) and om.shape == (0,)


def test_parse_is_faster_than_literal_eval():
    rows = _rows(20000, seed=2)
    t0 = time.perf_counter()
    worker.parse_reflections(rows, 1.0)
    t1 = time.perf_counter()
    _reference_parse(rows, 1.0)
    t2 = time.perf_counter()
    assert (t1 - t0) * 3 < (t2 - t1), (t1 - t0, t2 - t1)


def test_row_table_points_at_rows():
    vol = np.arange(3 * 4 * 5, dtype=np.int8).reshape(3, 4, 5)
    tab, keep = worker.python_2_c_3d(vol)
    for z in range(3):
        for y in range(4):
            assert ct.addressof(tab[z][y].contents) == vol.ctypes.data + (z * 4 + y) * 5
            assert tab[z][y][2] == vol[z, y, 2]
