"""Sharding a search batch across GPUs (one process per GPU).

leniax's ``run_scan_mem_optimized_pmap`` (runner.py:218-268) maps solutions
over devices with no collective; results come back as per-device shards.
Here each rank runs ``runner.run_scan_mem_optimized`` on a contiguous slice
of the solutions and the small per-world results (stop counts, optionally
stats) are gathered to one rank.  The data path has no collective.
"""
from typing import Dict, Tuple

import torch
import torch.distributed as dist


def shard_bounds(n: int, rank: int, world_size: int) -> Tuple[int, int]:
    """Contiguous slice [start, end) of n items owned by `rank`; the first
    n % world_size ranks get one extra item."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError('bad rank / world size')
    base, extra = divmod(n, world_size)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard_batch(tensors, rank: int, world_size: int):
    """Slice every tensor of a batch along its leading (solution) axis."""
    n = tensors[0].shape[0]
    a, b = shard_bounds(n, rank, world_size)
    return [t[a:b] for t in tensors]


def gather_leading(local: torch.Tensor, world_size: int, dst: int = 0):
    """Concatenate per-rank tensors (leading axes may differ) on rank `dst`;
    other ranks get None.  Works with gloo (CPU tensors) and nccl (CUDA)."""
    rank = dist.get_rank()
    n = torch.tensor([local.shape[0]], dtype=torch.int64, device=local.device)
    sizes = [torch.zeros_like(n) for _ in range(world_size)]
    dist.all_gather(sizes, n)
    sizes = [int(s.item()) for s in sizes]
    mx = max(sizes)
    pad = torch.zeros((mx, ) + tuple(local.shape[1:]), dtype=local.dtype, device=local.device)
    pad[:local.shape[0]] = local
    bufs = [torch.zeros_like(pad) for _ in range(world_size)]
    dist.all_gather(bufs, pad)
    if rank != dst:
        return None
    return torch.cat([b[:s] for b, s in zip(bufs, sizes)], dim=0)


def gather_results(local: Dict[str, torch.Tensor], world_size: int, dst: int = 0) -> Dict[str, torch.Tensor]:
    """gather_leading over every entry of a result dict (sorted keys, so all
    ranks issue the same collectives in the same order)."""
    out = {}
    for k in sorted(local):
        g = gather_leading(local[k].contiguous(), world_size, dst)
        if g is not None:
            out[k] = g
    return out
