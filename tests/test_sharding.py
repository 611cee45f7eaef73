"""Sharding of independent systems across ranks: LPT partition and host gather, run as 2 gloo ranks."""
import os
import socket

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
