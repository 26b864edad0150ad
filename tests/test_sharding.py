"""Multi-rank host logic of the sharded search batch, world_size 2 over gloo
(CPU processes; the per-rank engine call is replaced by a deterministic
function of the shard)."""
import os
import socket

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from leniax_gb300.sharding import gather_results, shard_batch, shard_bounds


def test_shard_bounds_cover_exactly():
    for n in (0, 1, 5, 1024, 4097):
        for ws in (1, 2, 3, 8):
            spans = [shard_bounds(n, r, ws) for r in range(ws)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _worker(rank, world_size, port, q):
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world_size)
    try:
        cells = torch.arange(5 * 3 * 4, dtype=torch.float32).reshape(5, 3, 4)  # 5 solutions
        T = torch.arange(5, dtype=torch.float32)
        lc, lT = shard_batch([cells, T], rank, world_size)
        # stand-in for the engine: per-(solution, init) stop counts and a per-step stat
        local = {'N': lc.sum(dim=2), 'mass': lc[:, None, :, 0].repeat(1, 2, 1) + lT[:, None, None]}
        out = gather_results(local, world_size)
        if rank == 0:
            q.put({k: v.tolist() for k, v in out.items()})
    finally:
        dist.destroy_process_group()


def test_gather_matches_single_process_world_size_2():
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = q.get(timeout=10)
    cells = torch.arange(5 * 3 * 4, dtype=torch.float32).reshape(5, 3, 4)
    T = torch.arange(5, dtype=torch.float32)
    assert got['N'] == cells.sum(dim=2).tolist()
    assert got['mass'] == (cells[:, None, :, 0].repeat(1, 2, 1) + T[:, None, None]).tolist()
