"""Large and long-axis worlds on the general N-D engine (sides up to 4096
whose prime factors are 2, 3, 5, 7; jnp.fft.fftn takes any shape,
core.py:74-87) against the oracle, forward and adjoint.  Worlds whose fused
last-axis tile set does not fit shared memory (a 4096-point last axis with
several channels) take the separate last-axis passes; those cases are here
too.  The longer transforms round more: potentials within 1e-5, states
within 2e-5 after one step (the bump growth's slope is about 2 / s = 70)."""
import numpy as np
import pytest
import torch

from leniax_gb300 import _lib, helpers, kernels
from oracle import lenia_oracle as O
from tests.cases import bump_kernel_params, random_multichannel_params
from tests.test_gpu_nd import REL, _cells, _engine_vs_autograd, relerr

pytestmark = pytest.mark.gpu

# (world, C, R, mean); the multi-channel models sum their kernels (a channel
# that no kernel feeds has no weighted mean)
CASES = [
    ([1024, 1024], 1, 40.0, True),  # large square world
    ([600, 600], 1, 30.0, True),  # 600 = 2^3 * 3 * 5^2
    ([2048, 1024], 2, 24.0, False),  # large, non-square, two channels: fused last-axis pass
    ([4096, 16], 4, 4.0, False),  # 4096-point last axis, four channels: separate last-axis passes
    ([1024, 8, 8], 3, 3.0, False),  # 3D, long z: plane passes and the fused z pass
    ([4096, 4, 4], 4, 2.0, False),  # 3D, 4096-point z with four channels: separate z passes
]


def _kp(C, R):
    if C == 1:
        return bump_kernel_params(s=0.03)
    return random_multichannel_params(C, 1, seed=C, R_range=(0.5 * R, R), world_R=R)


@pytest.mark.parametrize('world,C,R,mean', CASES)
def test_large_world_single_step_matches_oracle(cuda, world, C, R, mean):
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


def test_large_world_rejects_sides_past_4096(cuda):
    with pytest.raises(_lib.LgxError):
        K, mp = kernels.get_kernels_and_mapping(bump_kernel_params(), [8192, 16], 1, 4.0, True, cuda)
        helpers.build_update_fn(K.shape, mp)


@pytest.mark.parametrize('world,C,R,mean', [([1024, 1024], 1, 40.0, True), ([4096, 16], 2, 4.0, False)])
def test_large_world_adjoint_matches_float64_autograd(cuda, world, C, R, mean):
    # 1024^2 takes the fused last-axis passes; 4096 x 16 with two channels
    # takes the fused forward pass but the separate adjoint passes
    kp = _kp(C, R)
    cells = _cells(1, C, world, seed=3, frac=2)
    res = _engine_vs_autograd(cuda, kp, world, C, R, mean, cells, 4, 2, 0.2)
    for name, (g, r) in zip(('cells', 'kernel', 'gf'), res[0][:3]):
        assert relerr(g, r) <= REL, (world, name, relerr(g, r))
