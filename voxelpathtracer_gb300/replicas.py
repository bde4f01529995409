"""Replica bookkeeping for running the tracer on several GPUs of one node.

The traced path has no exchange step: every pixel and every world is
independent given the voxel volume and its distance field. So each GPU holds a
full replica of the volume and the distance field and works on its own share
of the units (screen rows of one frame, or whole worlds of a batch); the host
needs only a barrier and max/sum reductions of scalars to time the job, which
run over gloo (TCP) and never touch device memory. There is no data-path
collective and no NCCL.
"""
from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass(frozen=True)
class RankInfo:
    rank: int
    world: int
    local: int


def rank_info() -> RankInfo:
    """RANK / WORLD_SIZE / LOCAL_RANK as torch.distributed.run sets them (1 rank without)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    if not (0 <= rank < world):
        raise ValueError(f"RANK {rank} outside WORLD_SIZE {world}")
    return RankInfo(rank, world, local)


class Replicas:
    """Barrier and scalar reductions over the ranks of a replica job."""

    def __init__(self, world: int, backend: str = "gloo"):
        self.world = world
        self.td = None
        if world > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            if not td.is_initialized():
                td.init_process_group(backend)
            self.td = td

    def barrier(self) -> None:
        if self.td is not None:
            self.td.barrier()

    def _reduce(self, v: float, op) -> float:
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=op)
        return float(t.item())

    def max(self, v: float) -> float:
        return float(v) if self.td is None else self._reduce(v, self.td.ReduceOp.MAX)

    def sum(self, v: float) -> float:
        return float(v) if self.td is None else self._reduce(v, self.td.ReduceOp.SUM)

    def close(self) -> None:
        if self.td is not None:
            self.td.destroy_process_group()
            self.td = None


def shard_rows(height: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous band [r0, r1) of image rows for `rank`; bands differ by at most one row."""
    if height < 0 or world < 1 or not (0 <= rank < world):
        raise ValueError("bad shard request")
    base, extra = divmod(height, world)
    r0 = rank * base + min(rank, extra)
    return r0, r0 + base + (1 if rank < extra else 0)


def shard_worlds(costs, world: int) -> list[list[int]]:
    """Longest-processing-time split of batch worlds over `world` ranks.

    `costs` is one estimate per world (its ray count); worlds go, largest
    first, to the rank with the least assigned cost (ties to the lower rank),
    so the slowest rank carries at most 4/3 of the optimum. Each rank's list
    keeps the worlds in ascending index order.
    """
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0.0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += float(costs[i])
    return [sorted(o) for o in out]
