"""Reflection sharding across ranks (one process per GPU).

Reflections are independent, so the path shards with no collective on the
data path: rank r of W takes a contiguous slice of the reflection list (the
same split AnACor's driver makes with --low/--up, AnACor/main_lite.py:179-185),
runs it on its own GPU, and the per-reflection results are gathered on the
host afterwards.
"""
from __future__ import annotations

import numpy as np


def reflection_slice(n: int, rank: int, world: int) -> slice:
    """Balanced contiguous slice of n reflections for `rank` of `world`."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad rank / world")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return slice(lo, hi)


def gather_results(local: np.ndarray, n: int, rank: int, world: int, group=None) -> np.ndarray | None:
    """Gather every rank's slice to rank 0 (torch.distributed, any backend).

    Returns the full array on rank 0 and None elsewhere."""
    import torch
    import torch.distributed as dist
    if world == 1:
        return np.asarray(local)
    width = -(-n // world)
    buf = torch.full((width,), float("nan"), dtype=torch.float64)
    buf[:len(local)] = torch.as_tensor(np.asarray(local, dtype=np.float64))
    parts = [torch.empty_like(buf) for _ in range(world)] if rank == 0 else None
    dist.gather(buf, parts, dst=0, group=group)
    if rank != 0:
        return None
    out = np.empty(n, dtype=np.float64)
    for r in range(world):
        sl = reflection_slice(n, r, world)
        out[sl] = parts[r].numpy()[:sl.stop - sl.start]
    return out


def run_sharded(sample, rank: int, world: int, compute, group=None):
    """compute(sub_sample) -> A_h of its reflections; returns the gathered A_h on rank 0."""
    sl = reflection_slice(sample.n_refl, rank, world)
    local = compute(sample.subset(refl=sl)) if sl.stop > sl.start else np.zeros(0)
    return gather_results(local, sample.n_refl, rank, world, group)
