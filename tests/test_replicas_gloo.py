"""Multi-process host logic on CPU (gloo, world size 2): batch sharding and
the max-over-ranks timing the benchmark reports."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, costs, out):
    import torch.distributed as dist

    from simall_gb300.replicas import max_over_ranks, shard_by_cost

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shard_by_cost(costs, rank, world)
        t = max_over_ranks(10.0 + rank)
        gathered = [None] * world
        dist.all_gather_object(gathered, mine.tolist())
        dist.barrier()
        out.put((rank, mine.tolist(), t, gathered))
    finally:
        dist.destroy_process_group()


def test_shard_and_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp

    world = 2
    costs = (np.exp(np.random.default_rng(3).uniform(np.log(32), np.log(256), 41)) ** 2).round()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, costs, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert all(t == 11.0 for _, _, t, _ in res)          # max over ranks, seen by both
    assert res[0][3] == res[1][3]                        # both ranks agree on the assignment
    taken = sorted(res[0][1] + res[1][1])
    assert taken == list(range(len(costs)))              # every system exactly once
    loads = [costs[r[1]].sum() for r in res]
    assert max(loads) - min(loads) <= costs.max()        # greedy balance bound


def test_shard_single_process_and_errors():
    from simall_gb300.replicas import max_over_ranks, shard_by_cost

    assert shard_by_cost([3, 1, 2], 0, 1).tolist() == [0, 1, 2]
    assert max_over_ranks(4.5) == 4.5
    with pytest.raises(ValueError):
        shard_by_cost([1], 2, 2)
