"""Multi-rank path on CPU: two gloo ranks each take a reflection slice and the
gathered result equals the single-process one.  The oracle stands in for the
per-rank GPU compute (no GPU here); the sharding and gather code is the
package's own."""
import os
import socket

import numpy as np
import pytest

from anacor_public_gb300 import shard


def test_slices_cover_and_balance():
    for n in (0, 1, 7, 300, 20001):
        for w in (1, 2, 3, 8):
            sl = [shard.reflection_slice(n, r, w) for r in range(w)]
            assert sl[0].start == 0 and sl[-1].stop == n
            assert all(a.stop == b.start for a, b in zip(sl, sl[1:]))
            sizes = [s.stop - s.start for s in sl]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.reflection_slice(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from anacor_public_gb300 import synth
    from oracle.oracle import Oracle
    s = synth.small_sample(n_refl=21)
    o = Oracle()
    full = shard.run_sharded(s, rank, world, lambda sub: o.overall(sub, threads=2))
    if rank == 0:
        q.put(full)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_gather_the_full_result():
    import torch.multiprocessing as mp
    from anacor_public_gb300 import synth
    from oracle.oracle import Oracle
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    s = synth.small_sample(n_refl=21)
    assert np.array_equal(got, Oracle().overall(s, threads=4))
