"""Edge cases against the oracle: the largest channel / kernel counts a model
may have (16 channels, 64 kernels), tiny and prime-sided worlds on the
general N-D engine, a single-world single-step rollout, and an uneven batch
with an empty class (core.py:13-49, runner.py:119-215)."""
import numpy as np
import pytest
import torch

from leniax_gb300 import _lib
from leniax_gb300 import batch as lbatch
from leniax_gb300 import helpers, kernels, runner, statistics
from oracle import lenia_oracle as O
from tests.cases import bump_kernel_params, random_multichannel_params

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-5


def _step_case(dev, kp, world, C, R, cells, mean=True, T=5.0):
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], list(world), C, R, True, dev)
    upd = helpers.build_update_fn(K.shape, mp, 'v1', mean)
    Ko, mpo = O.get_kernels_and_mapping([dict(p) for p in kp], list(world), C, R, True, np.float32)
    dt = np.float32(1) / np.float32(T)
    so, fo, po = O.update(cells, Ko, mpo['gf_params'], mpo['weights'], dt, O.Model(mpo, 'v1', mean))
    s, f, p = upd(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev),
                  mp.get_kernels_weight_per_channel(dev), torch.tensor(dt, device=dev))
    return upd, (s.cpu().numpy(), f.cpu().numpy(), p.cpu().numpy()), (so, fo, po)


def _cells(n, C, world, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.random((n, C) + tuple(world), dtype=np.float32) * 0.6


@pytest.mark.parametrize('world', [[32, 32], [12, 10, 8]])
def test_largest_channel_and_kernel_counts(cuda, world):
    # C = 16 channels, K = 64 kernels (4 per channel): the largest model the
    # plan accepts; the streamed engine (2D) and the N-D engine (3D)
    C, per, R = 16, 4, 4.0
    kp = random_multichannel_params(C, per, seed=99, R_range=(1.5, 4.0), world_R=R)
    cells = _cells(2, C, world, seed=1)
    for mean in (True, False):
        upd, (s, f, p), (so, fo, po) = _step_case(cuda, kp, world, C, R, cells, mean)
        assert upd.model.K == 64 and upd.model.C == 16
        assert np.abs(p - po).max() < 5e-6
        assert np.abs(s - so).max() <= STEP_TOL
        assert np.abs(f - fo).max() < 2e-4
    with pytest.raises(_lib.LgxError):  # one kernel more is rejected
        kernels_more = kp + [dict(kp[0])]
        K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kernels_more], list(world), C, R, True, cuda)
        helpers.build_update_fn(K.shape, mp)


@pytest.mark.parametrize('world', [[4, 4], [5, 7], [7, 7], [6, 10], [5, 7, 9], [6, 6, 6]])
def test_tiny_and_prime_sided_worlds(cuda, world):
    # tiny worlds with sides of factors 2, 3, 5 and 7 (odd and prime
    # included); R = floor(min side / 2) keeps the kernel box (2 ceil(R)
    # cells) inside the smallest side with a kernel that has mass
    R = float(min(world) // 2)
    kp = bump_kernel_params(s=0.05)
    cells = _cells(3, 1, world, seed=sum(world))
    upd, (s, f, p), (so, fo, po) = _step_case(cuda, kp, world, 1, R, cells)
    assert _lib.load().lgx_select_engine(upd.model.plan.handle, 1, 3, 0) == _lib.ENGINES['nd']
    assert np.abs(p - po).max() < 2e-6
    assert np.abs(s - so).max() <= STEP_TOL
    # a short rollout with statistics and stop counts
    K, mp = kernels.get_kernels_and_mapping([dict(x) for x in kp], list(world), 1, R, True, cuda)
    Ko, mpo = O.get_kernels_and_mapping([dict(x) for x in kp], list(world), 1, R, True, np.float32)
    st_o, fin_o = O.run_scan(cells, Ko, mpo['gf_params'], mpo['weights'], 5, 4, R, O.Model(mpo),
                             keep_intermediary=False, with_box=True)
    sd, fin = runner.run_scan_mem_optimized(None, torch.from_numpy(cells[None]).to(cuda), K[None],
                                            mp.get_gf_params(cuda)[None], mp.get_kernels_weight_per_channel(cuda)[None],
                                            torch.tensor([5.]), 4, R, upd, statistics.ComputeStatsFn(list(world), R, 5),
                                            with_box=True)
    assert np.abs(fin[0].cpu().numpy() - fin_o).max() <= 4 * STEP_TOL
    np.testing.assert_array_equal(sd['N'][0].cpu().numpy(), st_o['N'])
    np.testing.assert_array_equal(sd['N_box'][0].cpu().numpy(), st_o['N_box'])


@pytest.mark.parametrize('engine', ['resident', 'streamed', 'plain'])
def test_single_world_single_step_rollout(cuda, engine):
    # the smallest rollout: one solution, one init, one step -- statistics of
    # the initial state, N of one step
    size, R = 64, 10
    kp = bump_kernel_params()
    cells = np.zeros((1, 1, 1, size, size), np.float32)
    cells[..., 20:44, 20:44] = _cells(1, 1, [24, 24], seed=4)
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], [size, size], 1, R, True, cuda)
    upd = helpers.build_update_fn(K.shape, mp)
    sd, fin = runner.run_scan_mem_optimized(None, torch.from_numpy(cells).to(cuda), K[None],
                                            mp.get_gf_params(cuda)[None], mp.get_kernels_weight_per_channel(cuda)[None],
                                            torch.tensor([10.]), 1, R, upd,
                                            statistics.ComputeStatsFn([size, size], R, 10), engine=engine,
                                            with_box=True)
    Ko, mpo = O.get_kernels_and_mapping([dict(p) for p in kp], [size, size], 1, R, True, np.float32)
    st, fo = O.run_scan(cells[0], Ko, mpo['gf_params'], mpo['weights'], 10, 1, R, O.Model(mpo),
                        keep_intermediary=False, with_box=True)
    assert np.abs(fin[0].cpu().numpy() - fo).max() <= STEP_TOL
    for k in statistics.STAT_KEYS:
        a, b = sd[k][0].cpu().numpy(), st[k]
        atol = 8 / R**2 if k.endswith('volume') or k.endswith('density') else 1e-4
        assert np.allclose(a, b, rtol=1e-4, atol=atol), k
    assert int(sd['N'][0, 0]) == int(st['N'][0]) and int(sd['N_box'][0, 0]) == int(st['N_box'][0])


def test_uneven_batch_with_an_empty_class(cuda):
    # a class without worlds is skipped: the other classes' results equal a
    # batch built without it, bit for bit
    dev = cuda
    rng = np.random.Generator(np.random.PCG64(8))
    cells = np.zeros((3, 64, 64), np.float32)
    cells[:, 22:42, 22:42] = rng.random((3, 20, 20), dtype=np.float32)
    R = torch.tensor([8., 9., 10.], device=dev)
    K = lbatch.world_spectra([64, 64], R.tolist(), bump_kernel_params()[0], dev)
    full = lbatch.WorldClass(cells0=torch.from_numpy(cells).to(dev), K=K,
                             gf_params=torch.tensor([[0.15, 0.02]] * 3, device=dev), weights=torch.ones(3, device=dev),
                             T=torch.tensor([10., 5., 10.], device=dev), R=R)
    empty = lbatch.WorldClass(cells0=torch.zeros((0, 32, 32), device=dev),
                              K=torch.zeros((0, 32, 17), dtype=torch.complex64, device=dev),
                              gf_params=torch.zeros((0, 2), device=dev), weights=torch.zeros(0, device=dev),
                              T=torch.zeros(0, device=dev), R=torch.zeros(0, device=dev))
    a = lbatch.UnevenBatch([full, empty], 8)
    a.run()
    b = lbatch.UnevenBatch([full], 8)
    b.run()
    torch.cuda.synchronize()
    assert a.status() == 0
    ra, rb = a.results()[0], b.results()[0]
    assert torch.equal(ra['final'], rb['final'])
    for k in rb['stats']:
        assert torch.equal(ra['stats'][k], rb['stats'][k]), k
    assert tuple(a.results()[1]['final'].shape) == (0, 32, 32)


def test_inputs_that_do_not_fit_the_model_are_refused_before_any_launch(cuda):
    # the engine reads spectra, parameters and T through bare pointers: a
    # tensor of another shape must be refused on the host
    from leniax_gb300 import core
    from leniax_gb300 import grad as lgrad
    from leniax_gb300 import workloads
    dev = cuda
    K, mp = kernels.get_kernels_and_mapping(bump_kernel_params(), [64, 64], 1, 10.0, True, dev)
    upd = helpers.build_update_fn(K.shape, mp)
    gf, w = mp.get_gf_params(dev), mp.get_kernels_weight_per_channel(dev)
    state = torch.zeros((2, 1, 64, 64), device=dev)
    short = K[..., :32, :]  # the spectrum of a 32 x 64 world
    with pytest.raises(ValueError):
        upd(None, state, short, gf, w, torch.tensor(0.1, device=dev))
    with pytest.raises(ValueError):
        core.get_potential_fft(state, short)
    stats_fn = statistics.ComputeStatsFn([64, 64], 10.0, 10.0)
    cells = torch.zeros((1, 2, 1, 64, 64), device=dev)
    two_channels = torch.cat([K, K], dim=1)[None]  # [Ns = 1, 1, C = 2, max_k, 64, 64] for a one-channel model
    with pytest.raises(ValueError):
        runner.run_scan_mem_optimized(None, cells, two_channels, gf[None], w[None], torch.tensor([10.]), 4, 10.0, upd,
                                      stats_fn)
    cells2 = torch.zeros((2, 2, 1, 64, 64), device=dev)
    with pytest.raises(ValueError):  # three T for two solutions
        runner.run_scan_mem_optimized(None, cells2, torch.stack([K, K]), torch.stack([gf, gf]), torch.stack([w, w]),
                                      torch.tensor([10., 10., 10.]), 4, 10.0, upd, stats_fn)
    with pytest.raises(ValueError):  # growth parameters left on the host
        lgrad.rollout(cells, torch.zeros((1, 1, 64, 64), device=dev), gf[None].cpu(), w[None], torch.tensor([10.]),
                      upd, 2)
    with pytest.raises(ValueError):  # one spectrum for two worlds
        lbatch.UnevenBatch([lbatch.WorldClass(cells0=torch.zeros((2, 32, 32), device=dev),
                                              K=lbatch.world_spectra((32, 32), [6.0], workloads.RING, dev),
                                              gf_params=torch.tensor([[0.15, 0.015]] * 2, device=dev),
                                              weights=torch.ones(2, device=dev), T=torch.full((2, ), 10., device=dev),
                                              R=torch.full((2, ), 6., device=dev))], 4)
