"""Replica aggregation across ranks (gloo, world size 2, CPU): the job's
rate is the summed work over the slowest rank's time; shards are balanced
and cover every item once."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from astroemperor_gb300.replicas import job_rate, shard


def test_shards_cover_every_item_once():
    for n, world in ((4096, 1), (4096, 2), (10, 3), (2, 4)):
        seen = []
        for r in range(world):
            sl = shard(n, r, world)
            seen.extend(range(n)[sl])
        assert seen == list(range(n))
        sizes = [len(range(n)[shard(n, r, world)]) for r in range(world)]
        assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    units = 1000.0 * (rank + 1)
    secs = 2.0 + rank
    out[rank] = job_rate(units, secs)
    dist.destroy_process_group()


def test_job_rate_gloo_two_ranks():
    world = 2
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        u, t, v = res[r]
        assert u == 3000.0 and t == 3.0 and v == pytest.approx(1000.0)


def test_job_rate_single_process():
    assert job_rate(10.0, 2.0) == (10.0, 2.0, 5.0)
