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


def _job(cells, kh, gf, w, T, steps, outs):
    job = _lib.Rollout()
    job.n_sols, job.n_init, job.steps = cells.shape[0], cells.shape[1], steps
    job.cells0, job.k_half, job.gf_params, job.weights, job.T = (cells.data_ptr(), kh.data_ptr(), gf.data_ptr(),
                                                                  w.data_ptr(), T.data_ptr())
    job.stats_R, job.stats_T = 13.0, 10.0
    job.final_cells = outs['final'].data_ptr()
    job.stats = outs['stats'].data_ptr()
    job.n_continue = outs['N'].data_ptr()
    job.n_box = outs['N_box'].data_ptr()
    job.centroid = outs['centroid'].data_ptr()
    job.engine = _lib.ENGINES['resident']
    return job


def _outs(cells, steps, dev):
    Ns, Ni = cells.shape[:2]
    return {
        'final': torch.empty_like(cells),
        'stats': torch.full((Ns, steps, Ni, 1 + _lib.NSTAT_SCALAR), float('nan'), device=dev),
        'N': torch.full((Ns, Ni), -1.0, device=dev),
        'N_box': torch.full((Ns, Ni), -1.0, device=dev),
        'centroid': torch.full((Ns, steps, Ni, 2), float('nan'), device=dev),
    }


def test_noalloc_rollout_matches_workspace_rollout_twice(cuda):
    dev = cuda
    lib = _lib.load()
    _bind(lib)
    size, steps = 128, 48
    K, mp = kernels.get_kernels_and_mapping(bump_kernel_params(), [size, size], 1, 13, True, dev)
    upd = helpers.build_update_fn(K.shape, mp)
    plan = upd.model.plan.handle
    kh = torch.view_as_real(K[..., :size // 2 + 1].contiguous()).reshape(1, 1, 1, size, size // 2 + 1, 2).contiguous()
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call, seed in enumerate((3, 4)):
        cells = torch.from_numpy(patch_init(6, size, 40, seed=seed, scale_range=(0.6, 1.0))[None]).to(dev)
        gf = torch.tensor([[[0.15, 0.015]]], device=dev)
        w = torch.ones((1, 1, 1), device=dev)
        T = torch.tensor([10.0], device=dev)
        assert 0 < lib.lgx_noalloc_scratch_bytes(plan, 1, 6, steps) <= 16 * 1024 * 1024
        ref = _outs(cells, steps, dev)
        ws = torch.empty(lib.lgx_run_workspace_bytes(plan, 1, 6, steps, _lib.ENGINES['resident']), dtype=torch.uint8,
                         device=dev)
        _lib.check(lib.lgx_run(plan, _job(cells, kh, gf, w, T, steps, ref), ws.data_ptr(), ws.numel(), stream))
        got = _outs(cells, steps, dev)
        rc = lib.lgx_run_noalloc(plan, _job(cells, kh, gf, w, T, steps, got), stream)
        assert rc == _lib.LGX_OK, lib.lgx_noalloc_last_error()
        torch.cuda.synchronize()
        # same kernels on the same inputs: the state tolerance of the parity tests (1e-5) holds with margin
        assert (got['final'] - ref['final']).abs().max().item() <= 1e-5, call
        assert torch.allclose(got['stats'], ref['stats'], rtol=1e-5, atol=1e-6, equal_nan=False), call
        assert torch.allclose(got['centroid'], ref['centroid'], rtol=1e-5, atol=1e-5), call
        assert torch.equal(got['N'], ref['N']) and torch.equal(got['N_box'], ref['N_box']), call


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
    job = _job(cells, kh, gf, w, T, steps, outs)
    rc = lib.lgx_run_noalloc(plan, job, torch.cuda.current_stream(dev).cuda_stream)
    assert rc == _lib.LGX_ERR_WORKSPACE
    assert b'scratch' in lib.lgx_noalloc_last_error()
