"""leniax's direct-convolution path (``fft=False``: ``core.get_potential``,
core.py:105-146, with the wrap padding of helpers.py:465-481) through the
engine: the conv-potential KAT of leniax's ``tests/test_core.py:55-103``,
single steps against the oracle's direct convolution (2D golden models, a 3D
world), rollouts against the FFT path, the batched runner, and the orbium
pipeline golden with ``fft=False``."""
import numpy as np
import pytest
import torch

from leniax_gb300 import helpers, kernels, runner, statistics
from leniax_gb300.kernels import KernelMapping
from oracle import lenia_oracle as O
from tests.cases import bump_kernel_params, golden_case, golden_world, patch_init
from tests.test_gpu_pipeline import _config

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-5


def test_conv_potential_kat_through_the_engine(cuda):
    # tests/test_core.py:55-103: a 2x2 torus, 2 channels, 3 true kernels in 4
    # slots of 3x3 kernels (larger than the world: taps wrap and add up)
    dev = cuda
    cells = np.ones([1, 2, 2, 2], np.float32)
    cells[0, 0] = 0.1
    cells[0, 1] = 0.2
    K = np.ones([4, 1, 3, 3], np.float32)
    K[0], K[1], K[2], K[3] = 0.1, 0.2, 0.3, 0
    mp = KernelMapping(2, 3)
    mp.cin_kernels = [[0, 1], [2]]
    mp.cin_gfs = [['gaussian', 'gaussian'], ['gaussian']]
    mp.cin_gf_params = [[[0.15, 0.015], [0.15, 0.015]], [[0.15, 0.015]]]
    mp.kernels_weight_per_channel = [[1., 1., 0.], [0., 0., 1.]]
    mp.true_channels = [True, True, True, False]
    upd = helpers.build_update_fn(K.shape, mp, fft=False)
    s, f, p = upd(None, torch.from_numpy(cells).to(dev), torch.from_numpy(K).to(dev), mp.get_gf_params(dev),
                  mp.get_kernels_weight_per_channel(dev), torch.tensor(0.1, device=dev))
    true = np.ones([1, 3, 2, 2], np.float32)
    true[0, 0], true[0, 1], true[0, 2] = 0.09, 0.18, 0.54
    np.testing.assert_allclose(p.cpu().numpy(), true, rtol=1e-6)


def _direct_step(dev, kp, world, C, R, cells, T, average=True):
    Kd, mp = kernels.get_kernels_and_mapping([dict(x) for x in kp], list(world), C, R, False, dev)
    upd = helpers.build_update_fn(Kd.shape, mp, 'v1', average, fft=False)
    Ko, mpo = O.get_kernels_and_mapping([dict(x) for x in kp], list(world), C, R, False, np.float32)
    dt = np.float32(1) / np.float32(T)
    so, fo, po = O.update_conv(cells, Ko, mpo['gf_params'], mpo['weights'], dt, O.Model(mpo, 'v1', average))
    s, f, p = upd(None, torch.from_numpy(cells).to(dev), Kd, mp.get_gf_params(dev),
                  mp.get_kernels_weight_per_channel(dev), torch.tensor(dt, device=dev))
    return (s.cpu().numpy(), f.cpu().numpy(), p.cpu().numpy()), (so, fo, po)


@pytest.mark.parametrize('name', ['orbium', 'orbium_scutium', 'aquarium'])
def test_direct_step_matches_the_oracle_convolution(cuda, name):
    cfg, init, _ = golden_case(name)
    cells, _, _ = golden_world(cfg, init)
    (s, f, p), (so, fo, po) = _direct_step(cuda, cfg['kernels_params'], cfg['world_size'], cfg['nb_channels'],
                                           cfg['R'], cells, cfg['T'], cfg['weighted_average'])
    assert np.abs(p - po).max() < 1e-5
    assert np.abs(f - fo).max() < 5e-4
    assert np.abs(s - so).max() <= STEP_TOL


def test_direct_step_3d_matches_the_oracle_convolution(cuda):
    world, R = [16, 12, 10], 4.0
    rng = np.random.Generator(np.random.PCG64(3))
    cells = rng.random((2, 1) + tuple(world), dtype=np.float32) * 0.6
    (s, f, p), (so, fo, po) = _direct_step(cuda, bump_kernel_params(s=0.05), world, 1, R, cells, 10)
    assert np.abs(p - po).max() < 1e-5
    assert np.abs(s - so).max() <= STEP_TOL


def test_direct_rollout_follows_the_fft_path(cuda):
    # run_scan with fft=False and fft=True: the same potentials up to the
    # rounding of the two spectra, the same stop count
    dev = cuda
    size, R, steps = 64, 10.0, 32
    kp = bump_kernel_params()
    cells = torch.from_numpy(patch_init(2, size, 24, seed=6)).to(dev)
    out = {}
    for fft in (True, False):
        K, mp = kernels.get_kernels_and_mapping([dict(x) for x in kp], [size, size], 1, R, fft, dev)
        upd = helpers.build_update_fn(K.shape, mp, fft=fft)
        out[fft] = runner.run_scan(None, cells, K, mp.get_gf_params(dev), mp.get_kernels_weight_per_channel(dev),
                                   torch.tensor(10.), steps, R, upd, statistics.ComputeStatsFn([size, size], R, 10))
    (ca, fa, pa, sa), (cb, fb, pb, sb) = out[True], out[False]
    assert np.abs(pa[:4].cpu().numpy() - pb[:4].cpu().numpy()).max() < 1e-5
    assert np.abs(ca[:8].cpu().numpy() - cb[:8].cpu().numpy()).max() < 1e-4
    np.testing.assert_array_equal(sa['N'].cpu().numpy(), sb['N'].cpu().numpy())


def test_direct_batched_runner(cuda):
    # run_scan_mem_optimized with per-solution direct kernels [Ns, C*max_k, 1, kh, kw]
    dev = cuda
    size, R, steps = 64, 10.0, 16
    kp = bump_kernel_params()
    Kd, mp = kernels.get_kernels_and_mapping([dict(x) for x in kp], [size, size], 1, R, False, dev)
    Kf, _ = kernels.get_kernels_and_mapping([dict(x) for x in kp], [size, size], 1, R, True, dev)
    updd = helpers.build_update_fn(Kd.shape, mp, fft=False)
    updf = helpers.build_update_fn(Kf.shape, mp)
    cells = torch.from_numpy(np.stack([patch_init(3, size, 24, seed=s) for s in (1, 2)])).to(dev)
    gf = torch.stack([mp.get_gf_params(dev), mp.get_gf_params(dev) * torch.tensor([1.05, 1.1], device=dev)])
    w = torch.stack([mp.get_kernels_weight_per_channel(dev)] * 2)
    T = torch.tensor([10., 8.])
    stats_fn = statistics.ComputeStatsFn([size, size], R, 10)
    sd, fin = runner.run_scan_mem_optimized(None, cells, torch.stack([Kd, Kd]), gf, w, T, steps, R, updd, stats_fn)
    sf, finf = runner.run_scan_mem_optimized(None, cells, torch.stack([Kf, Kf]), gf, w, T, steps, R, updf, stats_fn)
    assert tuple(fin.shape) == tuple(cells.shape)
    assert np.abs(fin.cpu().numpy() - finf.cpu().numpy()).max() < 1e-4
    np.testing.assert_array_equal(sd['N'].cpu().numpy(), sf['N'].cpu().numpy())


@pytest.mark.parametrize('with_jit', [False, True])
def test_init_and_run_direct_path_reproduces_orbium(cuda, with_jit):
    cfg, init, last = golden_case('orbium')
    all_cells, _, _, _ = helpers.init_and_run(None, _config(cfg, init), with_jit=with_jit, fft=False, device=cuda)
    assert len(all_cells) == cfg['max_run_iter']
    np.testing.assert_array_almost_equal(last, all_cells[-1, 0].cpu().numpy(), decimal=cfg['decimal'])
