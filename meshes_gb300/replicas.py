"""Several GPUs: independent replicas, or one batch split by columns.

Propagation needs no exchange between GPUs: the columns of a batch are independent and so are meshes.
Forward and forward-mode derivatives split with no collective at all.  A gradient over a batch split
across ranks needs one sum of dJ/dp (L x N/2 x n_p floats) over the ranks.  ``allreduce_grad`` does it
in a fixed order, so the result does not depend on which rank finishes first: every rank contributes
its partial gradient to an all-gather, and every rank adds the gathered partials in rank order.

These helpers take an initialised torch.distributed process group (NCCL on GPUs, gloo on CPU) and are
what ``bench.py`` uses under torchrun (one process per GPU, time = max over ranks).
"""
from __future__ import annotations

from typing import Optional, Tuple

import torch
import torch.distributed as dist


def shard_range(B: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous block of the B batch columns owned by `rank` (the first B % world ranks get one more)."""
    if world < 1 or not (0 <= rank < world) or B < 0:
        raise ValueError("bad shard request: B=%d rank=%d world=%d" % (B, rank, world))
    base, extra = divmod(B, world)
    b0 = rank * base + min(rank, extra)
    return b0, b0 + base + (1 if rank < extra else 0)


def max_over_ranks(t: float, group: Optional[dist.ProcessGroup] = None, device=None) -> float:
    """The slowest rank's time (the whole job finishes when its last replica does)."""
    if not dist.is_initialized() or dist.get_world_size(group) == 1:
        return float(t)
    x = torch.tensor([float(t)], dtype=torch.float64, device=device)
    dist.all_reduce(x, op=dist.ReduceOp.MAX, group=group)
    return float(x.item())


def allreduce_grad(dp: torch.Tensor, group: Optional[dist.ProcessGroup] = None) -> torch.Tensor:
    """Sum a per-rank partial gradient over the ranks, in rank order (deterministic); returns the sum.

    The partials are gathered and added rank 0 first, so the float32 result is bit-identical on every
    rank and from run to run, unlike a reduction whose order depends on the transport.
    """
    if not dist.is_initialized() or dist.get_world_size(group) == 1:
        return dp.clone()
    world = dist.get_world_size(group)
    parts = [torch.empty_like(dp) for _ in range(world)]
    dist.all_gather(parts, dp.contiguous(), group=group)
    out = parts[0].clone()
    for p in parts[1:]:
        out += p
    return out
