"""Independent runs across ranks: one process per GPU, no data-path collective.

A single Spectral2D run does not shard (every 2-D FFT would need a global
transpose, the all-to-all of the reference's slab decomposition,
src/Alloc.F90:90-100), so several GPUs run replicas or split an ensemble by
run.  This module holds the host-side pieces:

* :func:`run_cost` -- the relative cost of one run, M^2 log2 M with M = 3 nx/2;
* :func:`shard_runs` -- a deterministic cost-balanced split of an ensemble's
  runs over ranks (longest processing time first: each run, most expensive
  first, goes to the rank with the least work so far; ties go to the lower
  rank);
* :class:`ReplicaGroup` -- barrier and max / sum over ranks from the usual
  ``RANK`` / ``WORLD_SIZE`` / ``MASTER_ADDR`` / ``MASTER_PORT`` environment
  (NCCL on GPUs, gloo on CPUs), and a host-side gather of per-rank
  diagnostics.  With one rank every call is local.
"""

from __future__ import annotations

import math
import os


def run_cost(nx: int) -> float:
    """Relative cost of one RK3 step of an nx^2 run: M^2 log2 M, M = 3 nx / 2."""
    m = 3 * nx // 2
    return float(m * m * math.log2(m))


def shard_runs(costs, world: int):
    """Split run indices over ``world`` ranks, balancing the summed cost.
    Returns one sorted index list per rank; every index appears once."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    shards = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        shards[r].append(i)
        load[r] += costs[i]
    return [sorted(s) for s in shards]


class ReplicaGroup:
    """Barrier, max / sum and gather over the ranks of one node."""

    def __init__(self, backend: str | None = None, device: int | None = None):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", str(self.rank)))
        self.dist = None
        if self.world > 1:
            import torch
            import torch.distributed as dist
            if backend is None:
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local if device is None else device)
                self.dev = torch.device("cuda", torch.cuda.current_device())
            else:
                self.dev = torch.device("cpu")
            dist.init_process_group(backend)
            self.torch, self.dist = torch, dist

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def reduce(self, x: float, op: str = "MAX") -> float:
        """All-reduce one number (op = "MAX" or "SUM")."""
        if self.dist is None:
            return float(x)
        t = self.torch.tensor([float(x)], dtype=self.torch.float64, device=self.dev)
        self.dist.all_reduce(t, op=getattr(self.dist.ReduceOp, op))
        return float(t.item())

    def gather(self, obj):
        """Every rank's obj, in rank order (host-side diagnostics only)."""
        if self.dist is None:
            return [obj]
        out = [None] * self.world
        self.dist.all_gather_object(out, obj)
        return out

    def close(self) -> None:
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None
