"""Square 2D worlds whose side is not a power of two (even, factors 2, 3, 5,
7): the mixed-radix streamed step against the oracle — single steps
(potential, field, state), multi-channel topologies and short rollouts with
statistics and stop counts."""
import numpy as np
import pytest
import torch

from leniax_gb300 import runner, statistics, workloads
from oracle import lenia_oracle as O
from tests.cases import bump_kernel_params, patch_init
from tests.test_gpu_parity import STEP_TOL, engine_model, oracle_model, single_step_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('size', [48, 72, 100, 112])
def test_single_step_bump_gaussian(cuda, size):
    R = 9 if size < 72 else 13
    cells = patch_init(3, size, size // 2, seed=size)
    (s, f, p), (so, fo, po) = single_step_case(bump_kernel_params(), [size, size], 1, R, cells, 10)
    assert np.abs(p - po).max() < 5e-6
    assert np.abs(s - so).max() <= STEP_TOL
    assert np.abs(f - fo).max() < 2e-4


@pytest.mark.parametrize('average', [True, False])
def test_single_step_multichannel(cuda, average):
    size, C = 72, 3
    kp = workloads.multichannel_params(C, 3, seed=4, R_range=(6, 12), world_R=12.0)
    rng = np.random.Generator(np.random.PCG64(9))
    cells = np.zeros((2, C, size, size), np.float32)
    cells[:, :, 18:54, 18:54] = rng.random((2, C, 36, 36), dtype=np.float32)
    (s, f, p), (so, fo, po) = single_step_case(kp, [size, size], C, 12.0, cells, 5, average=average)
    assert np.abs(p - po).max() < 5e-6
    assert np.abs(s - so).max() <= STEP_TOL
    assert np.abs(f - fo).max() < 5e-4


@pytest.mark.parametrize('engine', ['auto', 'streamed'])
def test_rollout_statistics_and_stop_counts(cuda, engine):
    # 'auto' takes the N-D engine for these sides, 'streamed' the mixed-radix
    # streamed step
    dev = torch.device('cuda')
    size, R, steps = 72, 11.0, 24
    K, mp, upd = engine_model(bump_kernel_params(s=0.02), [size, size], 1, R, dev=dev)
    Ko, mpo, model = oracle_model(bump_kernel_params(s=0.02), [size, size], 1, R)
    cells = patch_init(3, size, 30, seed=17, scale_range=(0.6, 1.0))
    cs, fs, ps, st = runner.run_scan(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev),
                                     mp.get_kernels_weight_per_channel(dev), torch.tensor(10.), steps, R, upd,
                                     statistics.ComputeStatsFn([size, size], R, 10), engine=engine)
    cs_o, fs_o, ps_o, st_o = O.run_scan(cells, Ko, mpo['gf_params'], mpo['weights'], 10, steps, R, model)
    assert np.abs(cs[:4].cpu().numpy() - cs_o[:4]).max() < 4 * STEP_TOL
    assert np.abs(ps[:4].cpu().numpy() - ps_o[:4]).max() < 2e-5
    np.testing.assert_array_equal(st['N'].cpu().numpy(), st_o['N'])
    for k in ('mass', 'growth', 'mass_speed'):
        a, b = st[k][:4].cpu().numpy(), st_o[k][:4]
        assert np.allclose(a, b, rtol=1e-4, atol=1e-4), (k, np.abs(a - b).max())
