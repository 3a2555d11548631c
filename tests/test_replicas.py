"""
Replicas on several GPUs (myokit_gb300.replicas): sharding of independent
units, and the timing reduction of a replica run over two gloo ranks on the
CPU (the multi-GPU bench path without GPUs).
"""
import os
import socket

import pytest

from myokit_gb300.replicas import combine, shard


def test_shard_covers_units_once():
    for n in (0, 1, 7, 512, 1000):
        for world in (1, 2, 3, 8):
            ranges = [shard(n, world, r) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            for (a, b), (c, d) in zip(ranges, ranges[1:]):
                assert b == c
            sizes = [b - a for a, b in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(10, 2, 2)


def test_combine_single_rank():
    assert combine(12.5, 0.5, 1000) == (12.5, 0.5, 1000)


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        # Rank r: device time 10 + r ms, wall 0.1 * (r + 1) s, 1000 * (r+1)
        res = combine(10.0 + rank, 0.1 * (rank + 1), 1000 * (rank + 1),
                      world, dist, 'cpu')
        out.put((rank, res))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def test_combine_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q))
             for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        ms, wall, units = res[r]
        assert ms == 11.0 and abs(wall - 0.2) < 1e-12 and units == 3000
