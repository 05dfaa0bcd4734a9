"""Replicas-only multi-GPU runs: one independent replicated IMC problem per
rank (its own GPU and seed), no collective on the data path.  Upstream the
only exchange in the replicated step is the tally allreduce
(replicated_driver.h:90-94), which replicas do not need: each rank's
problem is complete on its own GPU.  These helpers give each rank its seed
and combine the ranks' timing into the whole-job figure (histories summed
over ranks, time = the slowest rank)."""
from __future__ import annotations

from typing import Tuple


def replica_seed(seed: int, rank: int) -> int:
    """Seed of rank r's replica: distinct per rank, rank 0 keeps the deck's."""
    return (int(seed) + 7919 * int(rank)) & 0xFFFFFFFF


def combine(elapsed_s: float, histories: float, device=None) -> Tuple[float, float]:
    """(max elapsed over ranks, total histories over ranks) through
    torch.distributed when a process group is up (any backend: tensors live on
    `device`, CPU for gloo); the local values otherwise."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(elapsed_s), float(histories)
    t = torch.tensor([float(elapsed_s)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    h = torch.tensor([float(histories)], dtype=torch.float64, device=device)
    dist.all_reduce(h, op=dist.ReduceOp.SUM)
    return float(t.item()), float(h.item())
