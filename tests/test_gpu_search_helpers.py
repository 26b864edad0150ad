"""The callers of the scan drivers in leniax ``helpers.py`` / ``runner.py``:
``multi_init_and_run`` (helpers.py:192-237), ``search_for_init``
(319-393), ``search_for_mutation`` (240-316) and
``run_scan_mem_optimized_pmap`` (runner.py:218-268), each checked against
the drivers it batches."""
import copy

import numpy as np
import pytest
import torch

from leniax_gb300 import helpers, kernels, runner, statistics
from tests.cases import golden_case, patch_init
from tests.test_gpu_pipeline import _config

pytestmark = pytest.mark.gpu


def _orbium_config(max_run_iter=48):
    cfg, init, _ = golden_case('orbium')
    c = _config(cfg, init)
    c['run_params']['max_run_iter'] = max_run_iter
    return c


def test_multi_init_and_run_equals_one_run_per_config(cuda):
    main = _orbium_config()
    configs = []
    for T, m in ((10., 0.15), (8., 0.15), (10., 0.16)):
        c = copy.deepcopy(main)
        c['world_params']['T'] = T
        c['kernels_params'][0]['gf_params'] = [m, 0.015]
        configs.append(c)
    cells, fields, pots, stats = helpers.multi_init_and_run(None, main, configs, device=cuda)
    assert tuple(cells.shape) == (3, 48, 1, 1, 128, 128)
    for i, c in enumerate(configs):
        ci, fi, pi, si = helpers.init_and_run(None, c, with_jit=True, device=cuda)
        assert torch.equal(cells[i], ci) and torch.equal(pots[i], pi) and torch.equal(fields[i], fi)
        assert int(stats['N'][i]) == int(si['N'])
        assert torch.equal(stats['mass'][i], si['mass'])


def test_search_for_init_picks_the_reference_choice(cuda):
    c = _orbium_config(64)
    c['run_params']['nb_init_search'] = 8
    c['algo'] = {'init_slug': 'perlin'}
    best, idx = helpers.search_for_init(1234, c, device=cuda)
    # the reference's loop over the same candidates, one run_scan each
    from leniax_gb300 import initializations as linit
    wp, ws = c['world_params'], c['render_params']['world_size']
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in c['kernels_params']], ws, 1, wp['R'], True, cuda)
    upd = helpers.build_update_fn(K.shape, mp)
    sfn = statistics.build_compute_stats_fn(wp, c['render_params'])
    _, noises = linit.register['perlin'](1234, 8, ws, wp['R'], c['kernels_params'][0]['gf_params'])
    T = torch.tensor(float(wp['T']), device=cuda)
    current, want_best, want_i = 0, None, 0
    runs = []
    for i in range(8):
        cells0 = noises[i:i + 1].reshape(1, 1, *ws).to(cuda)
        out = runner.run_scan(None, cells0, K, mp.get_gf_params(cuda), mp.get_kernels_weight_per_channel(cuda), T, 64,
                              wp['R'], upd, sfn)
        runs.append(out)
        n = int(out[3]['N'])
        want_i = i
        if current < n:
            current, want_best = n, i
        if n >= 64:
            break
    assert idx == want_i
    if want_best is None:
        assert best == {}
    else:
        assert int(best['N']) == int(runs[want_best][3]['N'])
        assert torch.equal(best['all_cells'], runs[want_best][0])


def test_search_for_mutation_runs_and_keeps_the_best(cuda):
    c = _orbium_config(32)
    c['run_params']['nb_mut_search'] = 3
    c['genotype'] = [{'key': 'kernels_params.0.gf_params.0', 'domain': [0., 1.], 'type': 'float'}]
    best, idx = helpers.search_for_mutation(7, c, nb_scale_for_stability=1, device=cuda, mutation_rate=1e-4)
    assert 0 <= idx < 3
    assert best and int(best['N']) <= 32
    m = best['config']['kernels_params'][0]['gf_params'][0]
    assert m != 0.15 and abs(m - 0.15) < 1e-2  # a mutated gene, a small step
    assert tuple(best['all_cells'].shape) == (32, 1, 128, 128)


def test_pmap_form_equals_one_call_per_slice(cuda):
    dev = cuda
    size, R, steps = 64, 10.0, 24
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in golden_case('orbium')[0]['kernels_params']],
                                            [size, size], 1, R, True, dev)
    upd = helpers.build_update_fn(K.shape, mp)
    sfn = statistics.ComputeStatsFn([size, size], R, 10)
    cells = torch.from_numpy(np.stack([np.stack([patch_init(2, size, 24, seed=10 * d + s) for s in range(2)])
                                       for d in range(2)])).to(dev)  # [N_device, N_sols, N_init, C, H, W]
    Kb = torch.stack([torch.stack([K, K])] * 2)
    gf = torch.stack([torch.stack([mp.get_gf_params(dev)] * 2)] * 2)
    w = torch.stack([torch.stack([mp.get_kernels_weight_per_channel(dev)] * 2)] * 2)
    T = torch.tensor([[10., 9.], [8., 10.]])
    stats, final = runner.run_scan_mem_optimized_pmap(None, cells, Kb, gf, w, T, steps, R, upd, sfn)
    assert tuple(final.shape) == tuple(cells.shape)
    for d in range(2):
        sd, fd = runner.run_scan_mem_optimized(None, cells[d], Kb[d], gf[d], w[d], T[d], steps, R, upd, sfn)
        assert torch.equal(final[d], fd)
        assert torch.equal(stats['N'][d], sd['N'])
