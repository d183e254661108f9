"""Host logic of bench.py that needs no GPU: the force mode 'auto' picks per
workload, --gpus N without a launcher becomes a torchrun command on the
loopback rendezvous, and several ranks split the batched ensemble so that
every replica is advanced by exactly one rank (the same split on every rank,
without communication), and which workloads take the cooperative
small-system run."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from femmd_old_gb300 import scene as S  # noqa: E402


def test_auto_force_mode_per_workload():
    assert bench.resolve_mode("lj_1m", "auto") == "fast"
    assert bench.resolve_mode("lj_fluid", "auto") == "fast"
    assert bench.resolve_mode("large_mixed", "auto") == "reference"
    assert bench.resolve_mode("suspension", "auto") == "reference"
    assert bench.resolve_mode("large_mixed", "fast") == "fast"
    assert bench.resolve_mode("lj_1m", "reference") == "reference"


def test_relaunch_command_is_torchrun_on_loopback():
    cmd = bench.relaunch_cmd(4, ["--gpus", "4", "--steps", "5"])
    assert cmd[:3] == [sys.executable, "-m", "torch.distributed.run"]
    assert "--nproc-per-node=4" in cmd
    i = cmd.index("--master-addr")
    assert cmd[i + 1] == "127.0.0.1"
    port = int(cmd[cmd.index("--master-port") + 1])
    assert 0 < port < 65536
    assert cmd[cmd.index(os.path.abspath(bench.__file__)) + 1:] == ["--gpus", "4", "--steps", "5"]


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_ensemble_share_covers_every_replica_once(world):
    ens = S.batched_ensemble()
    shares = [bench.ensemble_share(ens, world, r) for r in range(world)]
    ids = sorted(id(sc) for sh in shares for sc in sh)
    assert ids == sorted(id(sc) for sc in ens)
    atoms = [sum(int(sc.meta["N"]) for sc in sh) for sh in shares]
    total = sum(atoms)
    biggest = max(int(sc.meta["N"]) for sc in ens)
    assert max(atoms) - total / world <= biggest
    assert [bench.ensemble_share(ens, world, r) for r in range(world)] == shares


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _share_worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    try:
        import bench as B
        from femmd_old_gb300 import scene as SS
        from femmd_old_gb300.replicas import Group
        g = Group(backend="gloo")
        ens = SS.batched_ensemble()
        mine = B.ensemble_share(ens, g.world, g.rank)
        index = {id(sc): i for i, sc in enumerate(ens)}
        total = g.sum(sum(int(sc.meta["N"]) for sc in mine))
        got = g.gather(sorted(index[id(sc)] for sc in mine))
        if g.rank == 0:
            q.put(("ok", total, got, sum(int(sc.meta["N"]) for sc in ens)))
        g.close()
    except Exception as e:  # report instead of hanging the parent
        q.put(("error", repr(e)))


def test_two_gloo_ranks_split_the_ensemble():
    """Two ranks (gloo, CPU) each take their share of the batched ensemble:
    the shares are disjoint, cover all 512 replicas, and the ranks' summed
    atom count (the numerator of the whole-job throughput) is the
    ensemble's."""
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_share_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = q.get(timeout=180)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert res[0] == "ok", res
    _, total, got, want = res
    assert total == want
    assert sorted(got[0] + got[1]) == list(range(512))
    assert not set(got[0]) & set(got[1])


def test_single_process_stand_in_has_the_group_methods_the_bench_uses():
    from femmd_old_gb300.replicas import Group
    solo = bench._Solo()
    for name in ("barrier", "max", "sum"):
        assert callable(getattr(solo, name)) and callable(getattr(Group, name))
    assert solo.sum(3.5) == 3.5 and solo.max(2.0) == 2.0
    assert (solo.world, solo.rank, solo.local) == (1, 0, 0)


def test_small_run_path_follows_the_library_rule():
    # the cooperative small-system run: fast mode, one kind, no bonded
    # particles, walls, gravity or area springs, XY-periodic, <= 128 blocks
    lj = S.lj_fluid()
    lj.meta["types"] = 1
    assert bench.small_run_path(lj, 4096, False)
    assert not bench.small_run_path(lj, 4096, True)
    assert not bench.small_run_path(lj, bench.SMALL_RUN_MAX_ATOMS + 1, False)
    walled = S.lj_fluid()
    walled.meta["types"] = 1
    walled.add("set_gravity", 0.1)
    assert not bench.small_run_path(walled, 4096, False)
