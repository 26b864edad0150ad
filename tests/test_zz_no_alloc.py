"""lgx_run_noalloc -- the rollout for callers that cannot allocate device memory
(e.g. a runtime that pre-reserves the GPU's memory for its own pool) -- must
give the same results as lgx_run with a caller workspace.

Called through the C ABI with ctypes, twice in a row (the second call reuses
the fixed scratch array the first one left behind).  This file is collected
last so a failure here comes after every other test has run; it also passes
when run alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

from leniax_gb300 import _lib, helpers, kernels
from tests.cases import bump_kernel_params, patch_init

pytestmark = pytest.mark.gpu


def _bind(lib):
    lib.lgx_run_noalloc.argtypes = [ctypes.c_void_p, ctypes.POINTER(_lib.Rollout), ctypes.c_void_p]
    lib.lgx_run_noalloc.restype = ctypes.c_int
    lib.lgx_noalloc_scratch_bytes.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.lgx_noalloc_scratch_bytes.restype = ctypes.c_size_t
    lib.lgx_noalloc_last_error.restype = ctypes.c_char_p


def _job(cells, kh, gf, w, T, steps, outs, R, per_sol=None):
    job = _lib.Rollout()
    if per_sol is not None:  # per-solution statistics R and T
        job.stats_R_sol, job.stats_T_sol = per_sol[0].data_ptr(), per_sol[1].data_ptr()
    job.n_sols, job.n_init, job.steps = cells.shape[0], cells.shape[1], steps
    job.cells0, job.k_half, job.gf_params, job.weights, job.T = (cells.data_ptr(), kh.data_ptr(), gf.data_ptr(),
                                                                  w.data_ptr(), T.data_ptr())
    job.stats_R, job.stats_T = R, 10.0
    job.final_cells = outs['final'].data_ptr()
    job.stats = outs['stats'].data_ptr()
    job.n_continue = outs['N'].data_ptr()
    job.n_box = outs['N_box'].data_ptr()
    job.centroid = outs['centroid'].data_ptr()
    if 'traj' in outs:
        job.traj_cells, job.traj_field, job.traj_potential = (t.data_ptr() for t in outs['traj'])
    job.engine = _lib.ENGINES['resident']
    return job


def _outs(cells, steps, dev, traj=False):
    Ns, Ni = cells.shape[:2]
    out = {
        'final': torch.empty_like(cells),
        'stats': torch.full((Ns, max(steps, 1), Ni, 1 + _lib.NSTAT_SCALAR), float('nan'), device=dev),
        'N': torch.full((Ns, Ni), -1.0, device=dev),
        'N_box': torch.full((Ns, Ni), -1.0, device=dev),
        'centroid': torch.full((Ns, max(steps, 1), Ni, 2), float('nan'), device=dev),
    }
    if traj:
        shape = (steps, Ns * Ni) + tuple(cells.shape[2:])
        out['traj'] = tuple(torch.full(shape, float('nan'), device=dev) for _ in range(3))
    return out


def _model(size, dev):
    R = {32: 6, 64: 10, 128: 13}[size]
    # two solutions with their own kernel radius, growth parameters and T
    specs = []
    for sol, (m, s, r) in enumerate(((0.15, 0.015, 1.0), (0.2, 0.03, 0.8))):
        kp = bump_kernel_params(m=m, s=s, r=r)
        K, mp = kernels.get_kernels_and_mapping(kp, [size, size], 1, R, True, dev)
        specs.append((K, mp))
    upd = helpers.build_update_fn(specs[0][0].shape, specs[0][1])
    kh = torch.stack([torch.view_as_real(K[..., :size // 2 + 1].contiguous()).reshape(1, 1, size, size // 2 + 1, 2)
                      for K, _ in specs]).contiguous()
    gf = torch.stack([mp.get_gf_params(dev) for _, mp in specs]).contiguous()
    w = torch.stack([mp.get_kernels_weight_per_channel(dev) for _, mp in specs]).contiguous()
    return upd, kh, gf, w, torch.tensor([10.0, 5.0], device=dev), R


@pytest.mark.parametrize('size,traj,per_sol', [(32, False, False), (64, False, False), (128, False, False),
                                               (64, True, False), (64, False, True)])
def test_noalloc_rollout_matches_workspace_rollout_twice(cuda, size, traj, per_sol):
    dev = cuda
    lib = _lib.load()
    _bind(lib)
    steps, n_sols, n_init = (24 if traj else 48), 2, 5
    upd, kh, gf, w, T, R = _model(size, dev)
    sol = (torch.tensor([R, 2.0 * R], device=dev), torch.tensor([10.0, 7.0], device=dev)) if per_sol else None
    plan = upd.model.plan.handle
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call, seed in enumerate((3, 4)):
        cells = torch.from_numpy(np.stack([patch_init(n_init, size, size // 3, seed=seed + 10 * s,
                                                      scale_range=(0.6, 1.0)) for s in range(n_sols)])).to(dev)
        assert 0 < lib.lgx_noalloc_scratch_bytes(plan, n_sols, n_init, steps) <= 16 * 1024 * 1024
        ref = _outs(cells, steps, dev, traj)
        ws = torch.empty(lib.lgx_run_workspace_bytes(plan, n_sols, n_init, steps, _lib.ENGINES['resident']),
                         dtype=torch.uint8, device=dev)
        _lib.check(lib.lgx_run(plan, _job(cells, kh, gf, w, T, steps, ref, R, sol), ws.data_ptr(), ws.numel(),
                               stream))
        got = _outs(cells, steps, dev, traj)
        rc = lib.lgx_run_noalloc(plan, _job(cells, kh, gf, w, T, steps, got, R, sol), stream)
        assert rc == _lib.LGX_OK, lib.lgx_noalloc_last_error()
        torch.cuda.synchronize()
        # same kernels on the same inputs: the state tolerance of the parity tests (1e-5) holds with margin
        assert (got['final'] - ref['final']).abs().max().item() <= 1e-5, call
        assert torch.allclose(got['stats'], ref['stats'], rtol=1e-5, atol=1e-6, equal_nan=False), call
        assert torch.allclose(got['centroid'], ref['centroid'], rtol=1e-5, atol=1e-5), call
        assert torch.equal(got['N'], ref['N']) and torch.equal(got['N_box'], ref['N_box']), call
        if traj:
            for a, b in zip(got['traj'], ref['traj']):
                assert (a - b).abs().max().item() <= 1e-5, call
        if per_sol:
            # the second solution's statistics R differs from the scalar one: its mass (/ R^2) does too
            scalar = _outs(cells, steps, dev)
            _lib.check(lib.lgx_run(plan, _job(cells, kh, gf, w, T, steps, scalar, R), ws.data_ptr(), ws.numel(),
                                   stream))
            torch.cuda.synchronize()
            assert torch.allclose(scalar['stats'][0], got['stats'][0], rtol=1e-6, atol=1e-7), call
            mass = 1  # stats columns: channel_mass, mass, ...
            assert torch.allclose(got['stats'][1, ..., mass] * 4, scalar['stats'][1, ..., mass], rtol=1e-5), call


def test_noalloc_zero_steps_returns_the_initial_cells(cuda):
    dev = cuda
    lib = _lib.load()
    _bind(lib)
    upd, kh, gf, w, T, R = _model(64, dev)
    cells = torch.from_numpy(np.stack([patch_init(3, 64, 20, seed=s) for s in range(2)])).to(dev)
    got = _outs(cells, 0, dev)
    rc = lib.lgx_run_noalloc(upd.model.plan.handle, _job(cells, kh, gf, w, T, 0, got, R),
                             torch.cuda.current_stream(dev).cuda_stream)
    assert rc == _lib.LGX_OK, lib.lgx_noalloc_last_error()
    torch.cuda.synchronize()
    assert torch.equal(got['final'], cells)
    assert float(got['N'].abs().sum()) == 0.0 and float(got['N_box'].abs().sum()) == 0.0


def test_noalloc_rejects_batches_beyond_the_fixed_scratch(cuda):
    dev = cuda
    lib = _lib.load()
    _bind(lib)
    K, mp = kernels.get_kernels_and_mapping(bump_kernel_params(), [128, 128], 1, 13, True, dev)
    upd = helpers.build_update_fn(K.shape, mp)  # keeps the plan alive while its handle is used
    plan = upd.model.plan.handle
    steps, n_init = 4096, 64  # 64 worlds x 4096 steps of moments: > 16 MiB
    assert lib.lgx_noalloc_scratch_bytes(plan, 1, n_init, steps) > 16 * 1024 * 1024
    cells = torch.zeros((1, n_init, 1, 128, 128), device=dev)
    kh = torch.zeros((1, 1, 1, 128, 65, 2), device=dev)
    gf = torch.tensor([[[0.15, 0.015]]], device=dev)
    w = torch.ones((1, 1, 1), device=dev)
    T = torch.tensor([10.0], device=dev)
    outs = {
        'final': torch.empty_like(cells),
        'stats': torch.empty(1, device=dev),
        'N': torch.empty(1, device=dev),
        'N_box': torch.empty(1, device=dev),
        'centroid': torch.empty(1, device=dev)
    }
    job = _job(cells, kh, gf, w, T, steps, outs, 13.0)
    rc = lib.lgx_run_noalloc(plan, job, torch.cuda.current_stream(dev).cuda_stream)
    assert rc == _lib.LGX_ERR_WORKSPACE
    assert b'scratch' in lib.lgx_noalloc_last_error()
