"""Sharding a query batch over ranks (one process per GPU).

The reference splits its task index space into contiguous chunks, one per
HTCondor job (src/GP/pipeline/partt.py:10-35, chunk boundaries at
int(k * n / parts)), and gathers the per-chunk outputs afterwards.  Here each
rank owns the same contiguous range of the batch and answers it on its GPU;
`gather` concatenates the per-rank results in rank order.  Queries are
independent, so there is no collective on the data path -- only this final
concatenation.
"""
from __future__ import annotations

import numpy as np


def shard_range(n: int, rank: int, world: int):
    """[lo, hi) of rank's chunk: boundaries int(k * n / world) as partt.chunk_it draws them."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    avg = n / float(world)
    lo = int(rank * avg)
    hi = n if rank == world - 1 else int((rank + 1) * avg)
    return lo, hi


def gather(local, world: int, group=None):
    """All-gather variable-length 1-D results (torch tensors or numpy arrays) in rank order."""
    import torch
    import torch.distributed as dist
    t = torch.as_tensor(np.asarray(local)) if not isinstance(local, torch.Tensor) else local
    dev = t.device
    size = torch.tensor([t.shape[0]], dtype=torch.int64, device=dev)
    sizes = [torch.zeros_like(size) for _ in range(world)]
    dist.all_gather(sizes, size, group=group)
    m = int(max(s.item() for s in sizes))
    padded = torch.zeros((m,) + tuple(t.shape[1:]), dtype=t.dtype, device=dev)
    padded[:t.shape[0]] = t
    parts = [torch.zeros_like(padded) for _ in range(world)]
    dist.all_gather(parts, padded, group=group)
    return torch.cat([p[:int(s.item())] for p, s in zip(parts, sizes)])
