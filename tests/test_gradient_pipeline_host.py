"""Host side of the differentiable pipelines (leniax runner.py:363-448):
``grad.direct_world_kernels`` against the oracle's direct convolution
(core.py:105-146), and ``runner.make_pipeline_fn`` / ``make_gradient_fn`` /
``normalize_fn`` driven by a differentiable torch step on the CPU (the
engine step needs a GPU; its own gradients are checked there)."""
import numpy as np
import pytest
import torch

from leniax_gb300 import grad as lgrad
from leniax_gb300 import runner
from oracle import lenia_oracle as O


def _circular_potentials(state, kw, cin):
    # potential[k] = circular convolution of state[cin[k]] with the world kernel kw[k]
    axes = tuple(range(-kw.ndim + 1, 0))
    S = np.fft.fftn(state, axes=axes)
    return np.stack([np.real(np.fft.ifftn(S[:, c] * np.fft.fftn(kw[k], axes=axes), axes=axes))
                     for k, c in enumerate(cin)], axis=1)


@pytest.mark.parametrize('world,kd,C,max_k,table', [
    ((12, 10), (5, 4), 1, 1, [(0, 0)]),
    ((16, 16), (7, 7), 2, 2, [(0, 0), (1, 0), (1, 1)]),
    ((6, 5), (9, 8), 1, 2, [(0, 0), (0, 1)]),  # kernels longer than the world: taps wrap and add up
    ((6, 8, 5), (3, 4, 5), 2, 1, [(0, 0), (1, 0)]),
])
def test_direct_world_kernels_equal_the_direct_convolution(world, kd, C, max_k, table):
    rng = np.random.Generator(np.random.PCG64(sum(world) + sum(kd)))
    Kd = rng.random((C * max_k, 1) + kd)
    state = rng.random((2, C) + world)
    cin, slot = [c for c, _ in table], [s for _, s in table]
    tc = tuple(c * max_k + s for c, s in table)
    want = O.get_potential_conv(state, Kd, O.conv_padding(Kd.shape), tc)
    kw = lgrad.direct_world_kernels(torch.from_numpy(Kd), world, C, max_k, cin, slot)
    assert tuple(kw.shape) == (len(table), ) + world
    got = _circular_potentials(state, kw.numpy(), cin)
    np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-12)
    # a leading batch axis, and the gradient is the gather of the placement
    Kb = torch.from_numpy(np.stack([Kd, 2 * Kd])).requires_grad_(True)
    kwb = lgrad.direct_world_kernels(Kb, world, C, max_k, cin, slot)
    assert torch.allclose(kwb[1], 2 * kw)
    kwb.sum().backward()
    used = np.zeros(C * max_k)
    used[list(tc)] = 1
    want_grad = np.broadcast_to(used.reshape((1, -1) + (1, ) * (len(kd) + 1)), Kb.shape)
    np.testing.assert_array_equal(Kb.grad.numpy(), want_grad)  # every tap of a true kernel once, the rest 0


def test_normalize_fn():
    g = torch.tensor([[3.0, 0.0], [0.0, 4.0]])
    np.testing.assert_allclose(runner.normalize_fn(g).numpy(), g.numpy() / (5.0 + 1e-8))
    assert torch.equal(runner.normalize_fn(torch.zeros(3)), torch.zeros(3))


def _step(variables, rng_key, state, dt):
    # a differentiable stand-in for an update: s' = clamp(s + dt * (a * s + b), 0, 1)
    p = variables['params']
    return torch.clamp(state + dt * (p['a'] * state + p['inner']['b']), 0, 1), None, None


def _loss(rng_key, preds, targets):
    err = ((preds['cells'] - targets['cells'])**2).mean()
    return err, {'rng': rng_key}


def test_pipeline_keeps_every_pre_update_state_and_the_gradients_match_autograd():
    torch.manual_seed(0)
    state0 = torch.rand(3, 1, 6, 6) * 0.5
    params = {'a': torch.tensor(0.3), 'inner': {'b': torch.tensor([0.05])}}
    targets = {'cells': torch.rand(4, 3, 1, 6, 6)}
    pipe = runner.make_pipeline_fn(4, 0.1, _step, _loss, keep_all_timesteps=True)
    (loss, aux), grads = runner.make_gradient_fn(pipe, normalize=False)(7, params, {}, state0, targets)
    assert aux == [{'rng': 7}]
    # the same computation written out
    a = params['a'].clone().requires_grad_(True)
    b = params['inner']['b'].clone().requires_grad_(True)
    cur, states = state0, []
    for _ in range(4):
        states.append(cur)
        cur = torch.clamp(cur + 0.1 * (a * cur + b), 0, 1)
    ref = ((torch.stack(states) - targets['cells'])**2).mean()
    ga, gb = torch.autograd.grad(ref, [a, b])
    assert torch.allclose(loss, ref.detach())
    assert torch.allclose(grads['a'], ga) and torch.allclose(grads['inner']['b'], gb)
    # normalised: each gradient divided by its own norm
    _, ngrads = runner.make_gradient_fn(pipe, normalize=True)(7, params, {}, state0, targets)
    assert torch.allclose(ngrads['a'], ga / (ga.abs() + 1e-8))
    assert abs(float(torch.linalg.vector_norm(ngrads['inner']['b'])) - 1.0) < 1e-6


def test_pipeline_last_state_uses_the_rollout_of_the_apply_fn():
    calls = []

    class Apply:
        def __call__(self, variables, rng_key, state, dt):
            raise AssertionError('the last-state pipeline runs the whole horizon in one rollout')

        def rollout(self, variables, state, steps, dt):
            calls.append((steps, dt))
            return state * (1 + dt * variables['params']['a'])**steps

    state0 = torch.full((2, 1, 4, 4), 0.5)
    pipe = runner.make_pipeline_fn(5, 0.2, Apply(), _loss, keep_all_timesteps=False)
    loss, rest = pipe(0, {'a': torch.tensor(1.0)}, {}, state0, {'cells': torch.zeros(2, 1, 4, 4)})
    assert calls == [(5, 0.2)]
    assert torch.allclose(loss, torch.tensor((0.5 * 1.2**5)**2))
    with pytest.raises(NotImplementedError):
        runner.make_pipeline_fn(5, 0.2, Apply(), _loss, keep_intermediary_data=True)


def test_lenia_apply_reads_params_before_variables():
    class Model:
        world, C, K, max_k, cin, slot = (8, 8), 1, 1, 1, [0], [0]

    class Upd:
        def model_for(self, world):
            return Model()

    app = lgrad.LeniaApply(Upd())
    Kd = torch.rand(1, 1, 3, 3)
    Kw = torch.rand(1, 8, 8)
    gf, w = torch.rand(1, 2), torch.ones(1, 1)
    k, g, ww = app.kernels({'params': {'K': Kd}, 'K': Kw, 'gf_params': gf, 'kernels_weight_per_channel': w}, (8, 8))
    assert torch.equal(k, lgrad.direct_world_kernels(Kd, (8, 8), 1, 1, [0], [0])) and g is gf and ww is w
    k, _, _ = app.kernels({'params': {}, 'K': Kw, 'gf_params': gf, 'kernels_weight_per_channel': w}, (8, 8))
    assert k is Kw
    with pytest.raises(ValueError):
        app.kernels({'K': torch.rand(2, 8, 8), 'gf_params': gf, 'kernels_weight_per_channel': w}, (8, 8))
    with pytest.raises(KeyError):
        app.kernels({'K': Kw}, (8, 8))
