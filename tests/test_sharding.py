"""Sharding of independent systems across ranks: LPT partition and host gather, run as 2 gloo ranks."""
import os
import socket

import numpy as np
import pytest

from wtb_gb300.batch import lpt_partition, solve_sharded


def test_lpt_partition_balances_and_covers():
    costs = [27.0, 8.0, 64.0, 1.0, 125.0, 27.0, 8.0]
    parts = lpt_partition(costs, 3)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) == 125.0          # the largest job alone bounds the makespan
    assert lpt_partition(costs, 3) == parts  # deterministic


def test_lpt_single_rank():
    assert lpt_partition([3.0, 1.0], 1) == [[0, 1]]
    with pytest.raises(ValueError):
        lpt_partition([1.0], 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)

    def gather(local):
        out = [None] * world
        dist.all_gather_object(out, local)
        return out

    items = list(range(11))
    res = solve_sharded(items, lambda x: (x * x, rank), rank, world, cost=lambda x: float(x + 1) ** 3,
                        gather=gather)
    q.put((rank, res))
    dist.destroy_process_group()


def test_two_rank_gather_gloo():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see every result in item order, each computed by exactly one rank
    assert out[0] == out[1]
    assert [v for v, _ in out[0]] == [i * i for i in range(11)]
    assert {r for _, r in out[0]} == {0, 1}


def _lowest_transitions(item):
    """CPU stand-in for one system's solve: the oracle's bands on the system's mesh and its lowest nev
    transition energies E_c - E_v (the exciton energies with the Coulomb kernel switched off)."""
    from oracle import wtb_oracle as O

    sysm, p = item
    kpt = O.monhkhorst_pack(p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, sysm.rlat)
    eigv, _, _ = O.bands(sysm, p, kpt)
    de = (eigv[:, p.nv:p.nv + p.nc][:, :, None] - eigv[:, :p.nv][:, None, :]).ravel()
    return np.sort(de)[: p.nev]


def _batch_worker(rank, world, port, q):
    import torch.distributed as dist

    from wtb_gb300 import batch as B
    from wtb_gb300 import synthetic as S

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)

    def gather(local):
        out = [None] * world
        dist.all_gather_object(out, local)
        return out

    items = S.strained_batch(nsys=64)
    cost = [B.system_cost(p, s.w90basis) for s, p in items]
    mine = B.lpt_partition(cost, world)[rank]
    res = solve_sharded(items, _lowest_transitions, rank, world, cost=lambda it: B.system_cost(it[1], it[0].w90basis),
                        gather=gather)
    q.put((rank, mine, [r.tolist() for r in res]))
    dist.destroy_process_group()


def test_strained_batch_sharded_over_two_gloo_ranks():
    """The 64-system strained batch split over 2 ranks by the LPT partition of system_cost, each system solved by
    the rank that owns it, the results gathered on every rank: equal to a 1-rank run, item for item."""
    import torch.multiprocessing as mp

    from wtb_gb300 import batch as B
    from wtb_gb300 import synthetic as S

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_batch_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(2):
        r, mine, res = q.get(timeout=300)
        out[r] = (mine, res)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    items = S.strained_batch(nsys=64)
    ref = solve_sharded(items, _lowest_transitions, 0, 1)
    assert out[0][1] == out[1][1]
    assert len(out[0][1]) == len(items)
    for got, want in zip(out[0][1], ref):
        np.testing.assert_array_equal(np.array(got), want)
    # the two ranks own disjoint halves of the batch whose costs differ by at most the largest system's
    a, b = set(out[0][0]), set(out[1][0])
    assert a.isdisjoint(b) and a | b == set(range(len(items)))
    cost = [B.system_cost(p, s.w90basis) for s, p in items]
    la, lb = sum(cost[i] for i in a), sum(cost[i] for i in b)
    assert abs(la - lb) <= max(cost)
