"""leniax's differentiable pipeline API on the engine (runner.py:363-448,
the kernel-learning pattern of the reference's optimization example): the
direct-path kernels ``K`` ``[C*max_k, 1, kh, kw]`` and growth parameters as
``params``, ``grad.LeniaApply`` as the step.  The pipeline's loss and
gradients equal the same rollout written with ``grad.rollout`` (whose
gradients are checked against float64 autograd elsewhere)."""
import pytest
import torch

from leniax_gb300 import grad as lgrad
from leniax_gb300 import helpers, kernels, runner
from tests.cases import bump_kernel_params, patch_init

pytestmark = pytest.mark.gpu


def _loss(rng_key, preds, targets):
    return ((preds['cells'] - targets['cells'])**2).mean(), 'aux'


def test_pipeline_gradients_equal_the_rollout_gradients(cuda):
    dev = cuda
    Kd, mp = kernels.get_kernels_and_mapping([dict(p) for p in bump_kernel_params()], [64, 64], 1, 10.0, False, dev)
    upd = helpers.build_update_fn(Kd.shape, mp, 'v1', True, fft=False)
    gf, w = mp.get_gf_params(dev), mp.get_kernels_weight_per_channel(dev)
    cells = torch.from_numpy(patch_init(2, 64, 24, seed=5)).to(dev)  # [N = 2, C = 1, 64, 64]
    target = cells * 0.5
    pipe = runner.make_pipeline_fn(6, 0.1, lgrad.LeniaApply(upd, checkpoint_every=3), _loss,
                                   keep_all_timesteps=False)
    (loss, aux), grads = runner.make_gradient_fn(pipe, normalize=False)(None, {'K': Kd, 'gf_params': gf},
                                                                        {'kernels_weight_per_channel': w}, cells,
                                                                        {'cells': target})
    assert aux == ['aux']
    K1, gf1 = Kd.clone().requires_grad_(True), gf.clone().requires_grad_(True)
    kr = lgrad.direct_world_kernels(K1, (64, 64), 1, 1, [0], [0])
    fin = lgrad.rollout(cells[None], kr[None], gf1[None], w[None], torch.full((1, ), 1 / 0.1), upd, 6, 3)
    ref = ((fin[0] - target)**2).mean()
    gK, ggf = torch.autograd.grad(ref, [K1, gf1])
    assert torch.allclose(loss, ref.detach())
    assert torch.allclose(grads['K'], gK) and torch.allclose(grads['gf_params'], ggf)
    assert torch.isfinite(grads['K']).all() and float(grads['K'].abs().sum()) > 0
    # every pre-update state in the loss: one engine step per state, normalised gradients
    pipe_all = runner.make_pipeline_fn(3, 0.1, lgrad.LeniaApply(upd), _loss, keep_all_timesteps=True)
    (_, _), g_all = runner.make_gradient_fn(pipe_all, normalize=True)(
        None, {'K': Kd}, {'gf_params': gf, 'kernels_weight_per_channel': w}, cells,
        {'cells': target[None].expand((3, ) + tuple(target.shape))})
    assert abs(float(torch.linalg.vector_norm(g_all['K'])) - 1.0) < 1e-4
