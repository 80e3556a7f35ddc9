"""The multi-rank host logic on CPU with gloo, world size 2: instance
sharding without exchange (each rank evaluates its own slice; the gathered
per-group <W> equal a single-process evaluation) and the max-over-ranks timing
of bench.py."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch

    import bench
    from oracle import oracle as O

    w, r, _ = bench.dist_setup()
    assert (w, r) == (world, rank)
    loops = O.vloops(3, 256, 32)
    cx = np.linspace(0.0, 2.0, 10)
    T = np.geomspace(0.05, 2.0, 10)
    lo, hi = bench.shard(len(T), r, w)
    g = O.eval_groups(loops, cx[lo:hi], 0 * cx[lo:hi], T[lo:hi], [1.0],
                      O.field("smooth", fermion=1, nint=4), nthreads=1)
    parts = [None] * w
    dist.all_gather_object(parts, (lo, hi, g))
    t = bench.max_over_ranks(float(rank + 1), w)
    bench.barrier(w)
    if rank == 0:
        q.put((parts, t))
    dist.destroy_process_group()


def test_sharded_eval_equals_single_process():
    from oracle import oracle as O

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    parts, tmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert tmax == 2.0
    loops = O.vloops(3, 256, 32)
    cx = np.linspace(0.0, 2.0, 10)
    T = np.geomspace(0.05, 2.0, 10)
    ref = O.eval_groups(loops, cx, 0 * cx, T, [1.0], O.field("smooth", fermion=1, nint=4))
    got = np.concatenate([g for (_, _, g) in sorted(parts, key=lambda x: x[0])])
    assert [(lo, hi) for lo, hi, _ in sorted(parts, key=lambda x: x[0])] == [(0, 5), (5, 10)]
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("n,world", [(10, 2), (7, 3), (2, 4), (8192, 8)])
def test_shards_cover_all_units_once(n, world):
    import sys

    sys.path.insert(0, ROOT)
    import bench

    spans = [bench.shard(n, r, world) for r in range(world)]
    assert spans[0][0] == 0 and spans[-1][1] == n
    assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
    assert max(h - l for l, h in spans) - min(h - l for l, h in spans) <= 1
