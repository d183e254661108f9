"""Replicas across GPUs: one process per GPU, independent replicas on each,
no exchange on the data path.

The reference has no multi-GPU path.  Independent systems (replicas of an
ensemble, configurations of a parameter sweep) need none: each rank advances
its own share with the batched kernel and the ranks meet only to gather
observables and timings on the host.

``partition`` splits a list of replica costs over ranks (heaviest first, each
to the least-loaded rank; ties to the lower rank, so every rank computes the
same split without communicating).  ``Group`` wraps ``torch.distributed``
(NCCL on GPUs, gloo on CPU) for the barrier, the max of a timing and the
gather of per-rank results; with one process it does nothing.
"""
from __future__ import annotations

import heapq
import os


def partition(costs, world):
    """Indices of ``costs`` for each of ``world`` ranks: longest-processing-
    time first, deterministic.  Returns a list of ``world`` index lists, each
    in ascending cost order of assignment (heaviest first)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    out = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return out


class Group:
    """The ranks of a replicas-only run.  ``backend`` None picks NCCL when CUDA
    is available and gloo otherwise; the rendezvous comes from the usual
    torchrun environment (RANK, WORLD_SIZE, MASTER_ADDR, MASTER_PORT)."""

    def __init__(self, backend=None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        self.device = "cpu"
        if self.world > 1:
            import torch
            import torch.distributed as dist
            if backend is None:
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
                self.device = f"cuda:{self.local}"
            if not dist.is_initialized():
                dist.init_process_group(backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        """The largest of the ranks' values (timings: the slowest rank)."""
        if not self.pg:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.pg:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def gather(self, obj):
        """Every rank's ``obj`` on rank 0 (a list in rank order); None on the
        other ranks."""
        if not self.pg:
            return [obj]
        out = [None] * self.world if self.rank == 0 else None
        self.pg.gather_object(obj, out, dst=0)
        return out

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()
            self.pg = None
