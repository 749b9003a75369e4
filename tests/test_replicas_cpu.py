"""The multi-rank host logic on CPU: cost-balanced sharding of an ensemble's
runs and the replica group's barrier / max / sum / gather over two gloo
ranks (127.0.0.1), as bench.py --gpus N uses them with NCCL."""

import os
import socket

import pytest

from spectral2d_gb300.replicas import ReplicaGroup, run_cost, shard_runs


def test_shard_runs_partitions_and_balances():
    nxs = [128] * 32 + [256] * 32 + [512] * 32
    costs = [run_cost(n) for n in nxs]
    for world in (1, 2, 3, 4, 8):
        shards = shard_runs(costs, world)
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(nxs)))
        loads = [sum(costs[i] for i in s) for s in shards]
        # greedy LPT: no rank exceeds the mean by more than the largest run
        assert max(loads) - sum(loads) / world <= max(costs) + 1e-9
        assert shards == shard_runs(costs, world)   # deterministic
    assert shard_runs([], 2) == [[], []]
    with pytest.raises(ValueError):
        shard_runs(costs, 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    g = ReplicaGroup(backend="gloo")
    g.barrier()
    mx = g.reduce(10.0 + rank, "MAX")
    sm = g.reduce(1.0 + rank, "SUM")
    costs = [run_cost(n) for n in [64, 128, 256, 512, 128, 64]]
    mine = shard_runs(costs, world)[rank]
    everyone = g.gather(mine)
    g.close()
    q.put((rank, mx, sm, mine, everyone))


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, sm, mine, everyone in res:
        assert mx == 11.0 and sm == 3.0
        assert everyone[rank] == mine
        assert sorted(everyone[0] + everyone[1]) == list(range(6))


def test_single_rank_is_local(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    g = ReplicaGroup()
    assert g.world == 1 and g.reduce(3.5, "MAX") == 3.5 and g.gather(7) == [7]
    g.barrier()
    g.close()
