"""Replica bookkeeping on CPU: sharding of independent units, and the
max-over-ranks / whole-job throughput reductions with two gloo ranks
(rendezvous on 127.0.0.1)."""
import os
import socket

import pytest

from depix import replicas


def test_shard_covers_every_unit_once():
    for n in (0, 1, 7, 4096, 4097):
        for world in (1, 2, 3, 8):
            parts = [replicas.shard(n, r, world) for r in range(world)]
            units = [u for p in parts for u in p]
            assert units == list(range(n))
            assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
    with pytest.raises(ValueError):
        replicas.shard(10, 2, 2)


def test_single_process_reductions_are_identities():
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.job_throughput(100, 2.0) == 50.0


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        units = len(replicas.shard(4097, rank, world))
        seconds = 1.0 + rank  # rank 1 is the slow one
        out[rank] = (replicas.max_over_ranks(seconds), replicas.job_throughput(units, seconds))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_to_the_slowest_rank():
    import torch.multiprocessing as mp
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0] == res[1]
    slowest, thr = res[0]
    assert slowest == 2.0
    assert thr == pytest.approx(4097 / 2.0)
