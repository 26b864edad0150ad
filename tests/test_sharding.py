"""Multi-rank host logic of the sharded search batch, world sizes 2 and 3
over gloo: ``sharding.run_scan_mem_optimized_sharded`` slices the batch,
runs each rank's shard and gathers the results on rank 0 in solution order.
CPU processes: the per-rank engine call (``run_fn``) is a deterministic
function of every batched argument of the shard, so a result on rank 0
equals one call over the whole batch only if every rank got its own slice
and the gather put it back in place."""
import os
import socket

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import pytest

from leniax_gb300.sharding import gather_results, run_scan_mem_optimized_sharded, shard_batch, shard_bounds


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


def _fake_run(rng_key, cells0, K, gf, w, T, steps, R, update_fn, compute_stats_fn):
    # run_scan_mem_optimized's outputs, each a function of every batched input of its solution
    key = (cells0.flatten(2).sum(-1) + K.flatten(1).sum(-1)[:, None] + gf.flatten(1).sum(-1)[:, None] +
           w.flatten(1).sum(-1)[:, None] + T[:, None])  # [Ns, Ni]
    mass = key[:, None, :].repeat(1, steps, 1) * R
    stats = {'N': key.round(), 'mass': mass, 'channel_mass': torch.stack([mass, -mass], dim=-1)}
    return stats, cells0 * 2 + T[:, None, None, None, None]


def _batch(n=5):
    g = torch.Generator().manual_seed(0)
    return (torch.rand((n, 3, 1, 4, 4), generator=g), torch.rand((n, 1, 1, 1, 4, 3), generator=g),
            torch.rand((n, 1, 2), generator=g), torch.rand((n, 1, 1), generator=g), torch.arange(n) + 10.)


def _sharded_worker(rank, world_size, port, q, n):
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world_size)
    try:
        try:
            stats, final = run_scan_mem_optimized_sharded(None, *_batch(n), 6, 2.0, None, None, run_fn=_fake_run)
        except ValueError as e:
            q.put((rank, 'ValueError', str(e)))
            return
        if rank == 0:
            q.put((rank, {k: v.tolist() for k, v in stats.items()}, final.tolist()))
        else:
            q.put((rank, stats, final))
    finally:
        dist.destroy_process_group()


def _run_ranks(world_size, n):
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_sharded_worker, args=(r, world_size, port, q, n)) for r in range(world_size)]
    for p in procs:
        p.start()
    got = dict((r, rest) for r, *rest in (q.get(timeout=120) for _ in range(world_size)))
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    return got


@pytest.mark.parametrize('world_size', [2, 3])
def test_sharded_driver_equals_one_call_over_the_batch(world_size):
    got = _run_ranks(world_size, 5)
    want_stats, want_final = _fake_run(None, *_batch(5), 6, 2.0, None, None)
    stats, final = got[0]
    assert set(stats) == set(want_stats)
    for k, v in want_stats.items():
        assert stats[k] == v.tolist(), k
    assert final == want_final.tolist()
    for r in range(1, world_size):
        assert got[r] == [None, None]  # only rank 0 receives the results


def test_sharded_driver_needs_a_solution_per_rank():
    got = _run_ranks(3, 2)
    assert all(got[r][0] == 'ValueError' for r in range(3))


def test_sharded_driver_without_a_process_group_is_one_call():
    stats, final = run_scan_mem_optimized_sharded(None, *_batch(4), 3, 1.0, None, None, run_fn=_fake_run)
    want_stats, want_final = _fake_run(None, *_batch(4), 3, 1.0, None, None)
    assert torch.equal(final, want_final) and all(torch.equal(stats[k], want_stats[k]) for k in want_stats)
