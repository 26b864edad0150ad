"""Sharding a search batch across GPUs (one process per GPU).

leniax's ``run_scan_mem_optimized_pmap`` (runner.py:218-268) maps solutions
over devices with no collective; results come back as per-device shards.
Here each rank runs ``runner.run_scan_mem_optimized`` on a contiguous slice
of the solutions and the small per-world results (stop counts, optionally
stats) are gathered to one rank (:func:`run_scan_mem_optimized_sharded`).
The data path has no collective.
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


def run_scan_mem_optimized_sharded(rng_key, cells0, K, gf_params, kernels_weight_per_channel, T, max_run_iter: int,
                                   R: float, update_fn, compute_stats_fn, dst: int = 0, run_fn=None, **kw):
    """``run_scan_mem_optimized`` (runner.py:167-215) over the ranks of the
    default process group, one process per GPU: every rank passes the whole
    batch (``cells0`` ``[N_sols, N_init, C, *world]`` and the per-solution
    ``K``, ``gf_params``, weights and ``T``), runs its contiguous slice of
    the solutions (:func:`shard_bounds`) on its own device, and rank ``dst``
    receives ``(stats, final_cells)`` of the whole batch in solution order;
    the other ranks receive ``(None, None)``.  The rollouts exchange nothing;
    only the results are gathered (``N``, the stats and the final cells are
    per world).  Without an initialised process group it is one call of
    ``run_fn``.  ``run_fn`` defaults to ``runner.run_scan_mem_optimized``
    (same arguments; ``kw`` is passed on)."""
    if run_fn is None:
        from .runner import run_scan_mem_optimized as run_fn
    args = (max_run_iter, R, update_fn, compute_stats_fn)
    if not (dist.is_available() and dist.is_initialized()):
        return run_fn(rng_key, cells0, K, gf_params, kernels_weight_per_channel, T, *args, **kw)
    rank, world_size = dist.get_rank(), dist.get_world_size()
    n = int(cells0.shape[0])
    if n < world_size:
        raise ValueError(f'{n} solutions cannot be shared by {world_size} ranks (at least one each)')
    for name, t in (('K', K), ('gf_params', gf_params), ('kernels_weight_per_channel', kernels_weight_per_channel),
                    ('T', T)):
        if int(t.shape[0]) != n:
            raise ValueError(f'{name} has {int(t.shape[0])} solutions, cells0 has {n}')
    local = shard_batch([cells0, K, gf_params, kernels_weight_per_channel, T], rank, world_size)
    stats, final = run_fn(rng_key, *local, *args, **kw)
    flat = {'stats.' + k: v for k, v in stats.items()}
    flat['final'] = final
    if dist.get_backend() == 'gloo':  # gloo gathers host tensors
        flat = {k: v.cpu() for k, v in flat.items()}
    out = gather_results(flat, world_size, dst)
    if rank != dst:
        return None, None
    final = out.pop('final')
    return {k[len('stats.'):]: v for k, v in out.items()}, final
