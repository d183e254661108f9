"""Replicas across ranks (femmd_old_gb300.replicas): the host side of the
multi-GPU path, on CPU with two gloo processes.  The split of replica costs
covers every replica once and is the same on every rank without
communication; the slowest rank's timing, sums and the gather of per-rank
results reach rank 0 in rank order."""
import os
import socket

import pytest

from femmd_old_gb300.replicas import partition


def test_partition_covers_and_balances():
    costs = [19909, 500, 8000, 8000, 1200, 3000, 650, 15000, 777, 4100, 4100, 9000]
    for world in (1, 2, 3, 8):
        parts = partition(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        # greedy heaviest-first: within the largest cost of the ideal share
        assert max(loads) - sum(costs) / world <= max(costs)
        assert parts == partition(costs, world)  # deterministic
    with pytest.raises(ValueError):
        partition(costs, 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from femmd_old_gb300.replicas import Group, partition
    try:
        g = Group(backend="gloo")
        costs = [5000, 300, 12000, 800, 7000, 2500, 2500, 900]
        mine = partition(costs, g.world)[g.rank]
        g.barrier()
        slowest = g.max(10.0 + rank)
        atoms = g.sum(sum(costs[i] for i in mine))
        got = g.gather({"rank": g.rank, "replicas": mine})
        if g.rank == 0:
            q.put(("ok", slowest, atoms, got))
        g.close()
    except Exception as e:  # report instead of hanging the parent
        q.put(("error", repr(e)))


def test_two_gloo_ranks_gather_on_rank_zero():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = q.get(timeout=120)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert res[0] == "ok", res
    _, slowest, atoms, got = res
    assert slowest == 11.0
    assert atoms == sum([5000, 300, 12000, 800, 7000, 2500, 2500, 900])
    assert [d["rank"] for d in got] == [0, 1]
    assert sorted(got[0]["replicas"] + got[1]["replicas"]) == list(range(8))
