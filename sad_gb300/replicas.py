"""Replicas on several GPUs of one node: one process per GPU, each fitting its own images.

The fit-and-render path has no exchange between images (a fit's per-site gradients and
candidate fields are its own), so several GPUs run independent replicas: no collective on
the data path.  The only cross-rank operations are around the timing: a barrier before and
the maximum of the ranks' times after.  Launch with
`python -m torch.distributed.run --nproc-per-node N --master-addr 127.0.0.1 ...`.
"""
from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass(frozen=True)
class RankEnv:
    world_size: int
    rank: int
    local_rank: int


def rank_env() -> RankEnv:
    """WORLD_SIZE / RANK / LOCAL_RANK as torch.distributed.run sets them (1, 0, 0 alone)."""
    return RankEnv(int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
                   int(os.environ.get("LOCAL_RANK", "0")))


def init(env: RankEnv, backend: str = "nccl") -> None:
    """Join the process group when there is more than one rank."""
    if env.world_size > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend)


def finish(env: RankEnv) -> None:
    if env.world_size > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()


def barrier(env: RankEnv) -> None:
    if env.world_size > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(env: RankEnv, value: float, device=None) -> float:
    """The largest of the ranks' values (every rank gets it); `device` is where the
    backend reduces (a CUDA device for NCCL, None for gloo)."""
    if env.world_size == 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard(items: list, env: RankEnv) -> list:
    """This rank's share of independent work items: every world_size-th from its rank, so
    the shares partition the list and differ in length by at most one."""
    return items[env.rank::env.world_size]
