"""The multi-rank job of bench.py: with N ranks every rank takes its slice of
the job with the library's sharding (the reference's --low/--up split), and
the slices tile the job exactly (weak: N x the workload's reflections; strong:
the workload itself).  Host logic only: no GPU and no process group."""
import argparse

import numpy as np

import bench


def _args(scaling):
    return argparse.Namespace(workload="small", refl=30, scaling=scaling)


def test_strong_scaling_slices_tile_the_workload():
    whole, n = bench.job_samples(_args("strong"), 0, 1)
    parts = [bench.job_samples(_args("strong"), r, 4) for r in range(4)]
    assert all(p[1] == n for p in parts)
    s1 = np.concatenate([p[0][0].s1 for p in parts])
    om = np.concatenate([p[0][0].omega for p in parts])
    assert np.array_equal(s1, whole[0].s1) and np.array_equal(om, whole[0].omega)
    assert sorted(p[0][0].n_refl for p in parts) == [7, 7, 8, 8]


def test_weak_scaling_job_is_world_times_the_workload():
    parts = [bench.job_samples(_args("weak"), r, 3) for r in range(3)]
    assert all(p[1] == [90] for p in parts)
    assert [p[0][0].n_refl for p in parts] == [30, 30, 30]
    s1 = np.concatenate([p[0][0].s1 for p in parts])
    assert len(np.unique(s1, axis=0)) == 90          # one job, no rank repeats another's reflections
    assert np.array_equal(parts[0][0][0].coords, parts[2][0][0].coords)   # the same sample on every rank
