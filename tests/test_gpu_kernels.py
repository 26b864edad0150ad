"""On-device ring-kernel construction vs leniax's host construction
(get_kernels_and_mapping + circle_2d, kernels.py:66-212) as the oracle
restates it in numpy."""
import numpy as np
import pytest
import torch

from leniax_gb300 import kernels
from oracle import lenia_oracle as O

pytestmark = pytest.mark.gpu


CASES = [
    ('gauss_bump', [1.0], [1.0]),
    ('gauss_bump', [4.0], [0.5, 1.0, 0.25]),
    ('poly_quad', [4.0], [1.0, 0.3]),
    ('step', [0.2], [1.0]),
    ('gauss', [0.5], [0.7, 1.0]),
    ('threshold', [0.3], [1.0]),
    ('staircase', [0.5, 0.2], [1.0]),
    ('triangle', [0.5, 0.3], [0.4, 1.0]),
]


@pytest.mark.parametrize('world', [[32, 32], [64, 64], [128, 128], [256, 256], [32, 32, 32], [64, 64, 64],
                                   [48, 48], [45, 45], [100, 100], [66, 66], [24, 24, 24], [27, 27, 27]])
@pytest.mark.parametrize('kf_slug,kf_params,b', CASES)
def test_ring_kernels_match_host_construction(cuda, world, kf_slug, kf_params, b):
    size = world[0]
    R = [size / 8.0, size / 5.0, 3.0]
    r = [1.0, 0.8, 1.0]
    kr, kh = kernels.ring_kernels(world, R, r, [b] * 3, kf_slug, kf_params)
    kr, kh = kr.cpu().numpy(), kh.cpu().numpy()
    for i in range(3):
        ref = _spectrum_ref(world, R[i], r[i], b, kf_slug, kf_params)
        real_ref = _real_ref(world, R[i], r[i], b, kf_slug, kf_params)
        # two FP32 evaluations (CUDA expf / powf vs numpy, sum orders): a few ulp per value
        assert np.abs(kr[i] - real_ref).max() <= 1e-5 * max(np.abs(real_ref).max(), 1e-30), (world, kf_slug, i)
        assert np.abs(kh[i] - ref).max() <= 2e-5 * max(np.abs(ref).max(), 1e-30), (world, kf_slug, i)


def _real_ref(world, R, r, b, kf_slug, kf_params):
    """fftshifted world-size real kernel, float32, as leniax places it before
    its fftn: the oracle's circle_kernel, _pad_kernel and fftshift
    (kernels.py:93-101,148,176-212)."""
    return O.world_kernel(R, [r, list(b)], kf_slug, kf_params, world, dtype=np.float32)


def _spectrum_ref(world, R, r, b, kf_slug, kf_params):
    return np.fft.rfftn(_real_ref(world, R, r, b, kf_slug, kf_params).astype(np.float64))


def test_ring_kernels_reject_boxes_larger_than_the_world(cuda):
    with pytest.raises(ValueError):
        kernels.ring_kernels([32, 32], [20.0], [1.0], [[1.0]], 'gauss_bump', [1.0])


def test_device_spectra_drive_the_same_rollout_as_host_spectra(cuda):
    # the engine fed with device-built spectra reproduces the host-built ones
    from leniax_gb300 import helpers, runner, statistics
    from tests.cases import bump_kernel_params, patch_init
    dev = torch.device('cuda')
    kp = bump_kernel_params()
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], [128, 128], 1, 13, True, dev)
    _, kh = kernels.ring_kernels([128, 128], [13.0], [1.0], [[1.0]], 'gauss_bump', [1.0])
    upd = helpers.build_update_fn(K.shape, mp)
    stats_fn = statistics.ComputeStatsFn([128, 128], 13, 10)
    cells = torch.from_numpy(patch_init(4, 128, 40, seed=3)[None]).to(dev)
    # noise worlds amplify the few-ulp kernel differences step by step: a short
    # horizon keeps the comparison about the spectra, not the chaos
    args = (mp.get_gf_params(dev)[None], mp.get_kernels_weight_per_channel(dev)[None], torch.tensor([10.]), 4, 13, upd,
            stats_fn)
    _, f_host = runner.run_scan_mem_optimized(None, cells, K[None], *args)
    _, f_dev = runner.run_scan_mem_optimized(None, cells, kh.reshape(1, 1, 1, 1, 128, 65), *args)
    assert (f_host - f_dev).abs().max().item() <= 2e-5
