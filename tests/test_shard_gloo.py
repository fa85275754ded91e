"""Multi-rank sharding on CPU: two gloo ranks split one uneven batch by
estimated cost with no data exchange; together they cover every instance
exactly once, the loads are balanced, and the step time reported is the
maximum over ranks (the one collective)."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path[:0] = [os.path.dirname(here), os.path.join(os.path.dirname(here), "ndarray-conv_gb300")]
    import torch
    import torch.distributed as dist
    from ndconv import shard
    from ndconv.workloads import uneven_batch
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    specs = uneven_batch(400, seed=9)
    cost = lambda s: float(np.prod(s.out_shape())) * float(np.prod(s.kshape))  # noqa: E731
    mine = shard.local_share(specs, rank, world, cost=cost)
    # what every rank took (only for the check; the run itself needs no exchange)
    got = [None] * world
    dist.all_gather_object(got, mine)
    t = torch.tensor([1.0 + rank])  # this rank's step time
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    q.put((rank, got, float(t.item())))
    dist.destroy_process_group()


def test_two_rank_instance_sharding():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, tmax in res:
        assert tmax == 2.0
        flat = sorted(i for part in got for i in part)
        assert flat == list(range(400))
        assert not set(got[0]) & set(got[1])
    from ndconv import shard
    from ndconv.workloads import uneven_batch
    specs = uneven_batch(400, seed=9)
    costs = [float(np.prod(s.out_shape())) * float(np.prod(s.kshape)) for s in specs]
    assert shard.imbalance(costs, res[0][1]) < 1.05


def test_partition_properties():
    from ndconv.shard import partition
    rng = np.random.default_rng(0)
    costs = list(rng.pareto(1.5, 1000))
    for world in (1, 2, 4, 8):
        parts = partition(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(1000))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) <= sum(costs) / world + max(costs) + 1e-9
