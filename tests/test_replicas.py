"""Replica (one canvas set per rank) host logic on CPU with gloo, world size 2."""
import os

import pytest
import torch.multiprocessing as mp

from canvaz_film import replicas


def test_shard_covers_every_item_once():
    items = list(range(17))
    parts = [replicas.shard(items, r, 3) for r in range(3)]
    assert sorted(x for p in parts for x in p) == items
    assert all(abs(len(p) - len(items) / 3) < 1 for p in parts)
    with pytest.raises(ValueError):
        replicas.shard(items, 3, 3)


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    jobs = list(range(10))
    mine = replicas.shard(jobs, rank, world)
    cells = 1000 * sum(mine)            # this rank's cell-updates
    seconds = 1.0 + rank                # the slower rank takes 2 s
    rate, units, t = replicas.whole_job_rate(cells, seconds)
    out.put((rank, mine, rate, units, t))
    dist.destroy_process_group()


def test_whole_job_rate_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    (r0, m0, rate0, u0, t0), (r1, m1, rate1, u1, t1) = res
    assert sorted(m0 + m1) == list(range(10))
    assert u0 == u1 == 1000 * sum(range(10))
    assert t0 == t1 == 2.0
    assert rate0 == rate1 == u0 / 2.0
