"""Sharding of Monte-Carlo realisations across ranks (one process per GPU).

Realisations are independent, so a job of `total` realisations is split
into contiguous index ranges, one per rank; each rank draws its spectra from
counter-based keys of its own range (numpy default_rng([seed, r]) or the
device Philox generator at counter r), so the union over ranks is the same
set of realisations whatever the world size.  The only exchange is one
gather of the per-realisation scalars at the end; there is no collective on
the propagation path.
"""
from __future__ import annotations

from typing import Tuple


def realisation_range(rank: int, world: int, total: int) -> Tuple[int, int]:
    """[first, last) of this rank's realisations; sizes differ by at most 1."""
    if world < 1 or not (0 <= rank < world) or total < 0:
        raise ValueError("bad shard arguments")
    base, extra = divmod(total, world)
    first = rank * base + min(rank, extra)
    return first, first + base + (1 if rank < extra else 0)


def gather_measures(local, group=None):
    """Concatenates every rank's [n_local, n_out] measures in rank order (all
    ranks receive the result).  Works with gloo (CPU tensors) and NCCL (CUDA
    tensors); ranks may hold different row counts."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    n = torch.tensor([local.shape[0]], dtype=torch.int64, device=local.device)
    counts = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(counts, n, group=group)
    m = int(max(c.item() for c in counts))
    pad = torch.zeros((m, local.shape[1]), dtype=local.dtype, device=local.device)
    pad[: local.shape[0]] = local
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    return torch.cat([p[: int(c.item())] for p, c in zip(parts, counts)], dim=0)


def max_over_ranks(seconds: float, group=None, device=None) -> float:
    """Wall time of the slowest rank (the job's time)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
