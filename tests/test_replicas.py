"""Replica bookkeeping of the multi-GPU runs (one process per GPU, no data exchange), on CPU with gloo ranks."""
import os
import socket

import pytest


def test_shard_covers_every_unit_once():
    from nsl_gb300.replicas import shard

    for n, world in ((64, 2), (64, 8), (7, 3), (3, 4), (0, 2)):
        got = [u for r in range(world) for u in shard(n, r, world)]
        assert got == list(range(n))
        sizes = [len(shard(n, r, world)) for r in range(world)]
        assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    from nsl_gb300.replicas import job_rate, max_over_ranks, shard

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seconds = 1.0 + rank  # the slowest rank defines the job time
    t = max_over_ranks(seconds, dist)
    rate = job_rate(10, seconds, dist)
    mine = list(shard(10, rank, world))
    dist.destroy_process_group()
    out.put((rank, t, rate, mine))


def test_two_gloo_ranks_reduce_time_and_sum_units():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, rate, mine in res:
        assert t == 2.0
        assert rate == 2 * 10 / 2.0
    assert res[0][3] + res[1][3] == list(range(10))
