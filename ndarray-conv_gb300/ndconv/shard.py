"""Instance sharding for runs on several GPUs (one process per GPU).

The convolution path has no exchange step: instances are independent, so a
batch is split across ranks by estimated cost (longest-processing-time
greedy over the cost model's times) and each rank runs its share with no
collective on the data path.  Only the timing uses a collective (the
maximum over ranks).
"""
import heapq

import numpy as np


def partition(costs, world):
    """Greedy LPT: instance indices per rank, costliest instances first,
    each to the currently least-loaded rank.  Deterministic (ties by rank)."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(p) for p in parts]


def local_share(specs, rank, world, cost=None):
    """This rank's instances of a batch shared by `world` ranks."""
    if world <= 1:
        return list(range(len(specs)))
    if cost is None:
        from .dispatch import plan_info, spec_problem
        cost = lambda s: min(plan_info(spec_problem(s))[:2])  # noqa: E731
    costs = [cost(s) for s in specs]
    return partition(costs, world)[rank]


def imbalance(costs, parts):
    loads = np.array([sum(costs[i] for i in p) for p in parts])
    return float(loads.max() / max(loads.mean(), 1e-30))
