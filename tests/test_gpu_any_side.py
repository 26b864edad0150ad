"""Worlds whose sides have a prime factor above 7 (66 = 2 * 3 * 11, 127,
26 = 2 * 13, 1031, 3D 11 x 13 x 17): the N-D engine's Bluestein lines
against the oracle (numpy's FFT takes any length, as jnp.fft.fftn does,
core.py:74-87), single steps, a rollout with statistics and stop counts, and
the adjoint against float64 autograd.  The chirp-z transform rounds a little
more than a direct mixed-radix one: potentials within 1e-5, states within
2e-5 after one step."""
import numpy as np
import pytest
import torch

from leniax_gb300 import _lib, helpers, kernels, runner, statistics
from oracle import lenia_oracle as O
from tests.cases import bump_kernel_params, random_multichannel_params
from tests.test_gpu_nd import REL, _cells, _engine_vs_autograd, relerr

pytestmark = pytest.mark.gpu

# (world, C, R, mean)
CASES = [
    ([66, 66], 1, 12.0, True),
    ([127, 127], 1, 20.0, True),
    ([26, 100], 2, 6.0, False),
    ([1031, 64], 1, 10.0, True),
    ([11, 13, 17], 1, 3.0, True),
    ([22, 26, 32], 2, 4.0, False),
]


def _kp(C, R):
    if C == 1:
        return bump_kernel_params(s=0.03)
    return random_multichannel_params(C, 1, seed=C + 1, R_range=(0.5 * R, R), world_R=R)


@pytest.mark.parametrize('world,C,R,mean', CASES)
def test_any_side_single_step_matches_oracle(cuda, world, C, R, mean):
    dev = cuda
    kp = _kp(C, R)
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], list(world), C, R, True, dev)
    upd = helpers.build_update_fn(K.shape, mp, 'v1', mean)
    assert _lib.load().lgx_select_engine(upd.model.plan.handle, 1, 2, 0) == _lib.ENGINES['nd']
    Ko, mpo = O.get_kernels_and_mapping([dict(p) for p in kp], list(world), C, R, True, np.float32)
    cells = _cells(2, C, world, seed=sum(world), frac=2)
    dt = np.float32(0.2)
    so, fo, po = O.update(cells, Ko, mpo['gf_params'], mpo['weights'], dt, O.Model(mpo, 'v1', mean))
    s, f, p = upd(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev),
                  mp.get_kernels_weight_per_channel(dev), torch.tensor(dt, device=dev))
    assert np.abs(p.cpu().numpy() - po).max() < 1e-5
    assert np.abs(f.cpu().numpy() - fo).max() < 5e-4
    assert np.abs(s.cpu().numpy() - so).max() <= 2e-5


def test_any_side_rollout_statistics_and_stop_counts(cuda):
    dev = cuda
    world, R, steps = [66, 66], 11.0, 24
    kp = bump_kernel_params(s=0.02)
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], world, 1, R, True, dev)
    upd = helpers.build_update_fn(K.shape, mp)
    Ko, mpo = O.get_kernels_and_mapping([dict(p) for p in kp], world, 1, R, True, np.float32)
    cells = _cells(3, 1, world, seed=17, frac=2)
    cs, fs, ps, st = runner.run_scan(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev),
                                     mp.get_kernels_weight_per_channel(dev), torch.tensor(10.), steps, R, upd,
                                     statistics.ComputeStatsFn(world, R, 10))
    cs_o, fs_o, ps_o, st_o = O.run_scan(cells, Ko, mpo['gf_params'], mpo['weights'], 10, steps, R, O.Model(mpo))
    assert np.abs(cs[:4].cpu().numpy() - cs_o[:4]).max() < 1e-4
    np.testing.assert_array_equal(st['N'].cpu().numpy(), st_o['N'])
    for k in ('mass', 'growth', 'mass_speed'):
        a, b = st[k][:4].cpu().numpy(), st_o[k][:4]
        assert np.allclose(a, b, rtol=1e-4, atol=1e-4), (k, np.abs(a - b).max())


@pytest.mark.parametrize('world,C,R,mean', [([66, 66], 1, 12.0, True), ([26, 100], 2, 6.0, False),
                                            ([11, 13, 17], 1, 3.0, True)])
def test_any_side_adjoint_matches_float64_autograd(cuda, world, C, R, mean):
    kp = _kp(C, R)
    cells = _cells(1, C, world, seed=5, frac=2)
    res = _engine_vs_autograd(cuda, kp, world, C, R, mean, cells, 4, 2, 0.2)
    for name, (g, r) in zip(('cells', 'kernel', 'gf'), res[0][:3]):
        assert relerr(g, r) <= REL, (world, name, relerr(g, r))
