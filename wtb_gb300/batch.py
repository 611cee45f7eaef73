"""Batches of independent exciton systems (strain variants, k-meshes of uneven size).

Systems are independent, so a batch shards across GPUs with no data-path collective: each rank solves
the systems a longest-processing-time-first partition assigns to it (cost model ``system_cost``) and the
results are gathered on the host.  One rank drives one GPU; on that GPU ``api.Batch`` overlaps the
rank's systems on several streams.
"""
from __future__ import annotations

import heapq
from typing import Callable, Sequence


def system_cost(p, w: int | None = None) -> float:
    """Relative cost of one system.  With the orbital count w: the matrix-free operator's Nk^2 w^2 nev
    (its V x Z contraction dominates; the same model orders the work of wtb_batch_bsesolver).  Without it:
    the dense-equivalent dim^3 (the reference's ZHEEV scaling)."""
    if w is None:
        return float(p.dim) ** 3
    nk = float(p.ngrid[0] * p.ngrid[1] * p.ngrid[2])
    return nk * nk * float(w) ** 2 * max(int(p.nev), 1) + nk * p.nc * p.nv * 1e3


def lpt_partition(costs: Sequence[float], nranks: int) -> list[list[int]]:
    """Longest-processing-time-first greedy: largest job to the least loaded rank.  Deterministic:
    ties break on the job index and then the rank index."""
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, r) for r in range(nranks)]
    heapq.heapify(heap)
    parts: list[list[int]] = [[] for _ in range(nranks)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    for p in parts:
        p.sort()
    return parts


def solve_sharded(items: Sequence, solve_one: Callable, rank: int, world: int, cost: Callable = None,
                  gather: Callable = None):
    """Solve the items assigned to ``rank`` and return the results of all ranks in item order.

    ``solve_one(item) -> result``; ``cost(item) -> float``; ``gather(local_dict) -> list of dicts`` (one per
    rank; e.g. torch.distributed.all_gather_object).  With world == 1 nothing is gathered."""
    costs = [cost(it) if cost else 1.0 for it in items]
    parts = lpt_partition(costs, world)
    local = {i: solve_one(items[i]) for i in parts[rank]}
    if world == 1 or gather is None:
        return [local[i] for i in range(len(items))] if world == 1 else local
    everything = {}
    for d in gather(local):
        everything.update(d)
    return [everything[i] for i in range(len(items))]
