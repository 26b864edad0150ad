"""Hand-written adjoint vs float64 autograd (the jax.grad stand-in) and FP64
central finite differences; device kernel spectrum vs numpy's FFT."""
import numpy as np
import pytest
import torch

from leniax_gb300 import grad as lgrad
from leniax_gb300 import helpers, kernels
from oracle import lenia_grad_oracle as GO
from oracle import lenia_oracle as O
from tests.cases import bump_kernel_params, patch_init

pytestmark = pytest.mark.gpu

REL = 1e-3  # gradient relative error bound vs finite differences / float64 autograd


def relerr(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-30))


@pytest.mark.parametrize('size', [32, 64, 128, 256])
def test_kernel_spectrum_matches_numpy(cuda, size):
    rng = np.random.Generator(np.random.PCG64(size))
    k = rng.random((3, size, size), dtype=np.float32)
    got = lgrad.kernel_spectrum(torch.from_numpy(k).to(cuda)).cpu().numpy()
    ref = np.fft.rfft2(k.astype(np.float64))
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()


def _setup(cuda, size=64, R=10, steps=12, n_init=2, seed=5, slug='gaussian', m=0.15, s=0.02):
    kp = bump_kernel_params(m=m, s=s)
    kp[0]['gf_slug'] = slug
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], [size, size], 1, R, True, cuda)
    upd = helpers.build_update_fn(K.shape, mp)
    b = torch.tensor([1.0], device=cuda)
    k_real = lgrad.ring_kernel(R, 1.0, b, 'gauss_bump', [1.0], [size, size])
    cells = patch_init(n_init, size, size // 2, seed=seed, scale_range=(0.6, 1.0))
    target = patch_init(n_init, size, size // 2, seed=seed + 100) * 0.5
    return upd, k_real, cells, target


def _engine_grads(cuda, upd, k_real, cells, target, m, s, w, T, steps, clip, ckpt=4):
    c0 = torch.from_numpy(cells[None]).to(cuda).requires_grad_(True)
    kr = k_real[None].detach().clone().requires_grad_(True)
    gf = torch.tensor([[[m, s]]], device=cuda, requires_grad=True)
    ww = torch.tensor([[[w]]], device=cuda, requires_grad=True)
    fin = lgrad.rollout(c0, kr, gf, ww, torch.tensor([T]), upd, steps, ckpt, clip)
    loss = ((fin - torch.from_numpy(target[None]).to(cuda))**2).mean()
    loss.backward()
    return (float(loss.detach()), c0.grad[0].cpu().numpy(), kr.grad[0].cpu().numpy(), gf.grad[0, 0, 0].item(),
            gf.grad[0, 0, 1].item(), ww.grad.item())


@pytest.mark.parametrize('slug', ['gaussian', 'poly_quad4'])
def test_adjoint_matches_float64_autograd_ste(cuda, slug):
    steps, T, w = 12, 10.0, 1.0
    m, s = (0.15, 0.02) if slug == 'gaussian' else (0.15, 0.03)
    upd, k_real, cells, target = _setup(cuda, slug=slug, steps=steps, m=m, s=s)
    L, gc, gk, gm, gs, gw = _engine_grads(cuda, upd, k_real, cells, target, m, s, w, T, steps, 'ste')
    kref = k_real.detach().cpu().double().numpy()
    Lr, (rc, rk, rm, rs, rw) = GO.loss_and_grads(cells.astype(np.float64), kref, m, s, w, 1 / T, steps, target,
                                                 slug=slug, clip='ste')
    assert abs(L - Lr) <= 1e-5 * abs(Lr) + 1e-9
    assert relerr(gc, rc) <= REL
    assert relerr(gk, rk) <= REL
    assert abs(gm - rm) <= REL * abs(rm) + 1e-9
    assert abs(gs - rs) <= REL * abs(rs) + 1e-9
    assert abs(gw) <= 1e-6 and abs(rw) <= 1e-9  # weighted_mean with one kernel: f = g, no w dependence


def test_adjoint_streamed_size_matches_float64_autograd(cuda):
    # 256x256 worlds take the streamed adjoint (spectra through global memory,
    # column-major kernel spectrum planes), not the resident one
    size, R, steps, T, w, m, s = 256, 20, 8, 10.0, 1.0, 0.15, 0.02
    upd, k_real, cells, target = _setup(cuda, size=size, R=R, steps=steps, n_init=1, seed=13, m=m, s=s)
    L, gc, gk, gm, gs, gw = _engine_grads(cuda, upd, k_real, cells, target, m, s, w, T, steps, 'ste', ckpt=3)
    kref = k_real.detach().cpu().double().numpy()
    Lr, (rc, rk, rm, rs, rw) = GO.loss_and_grads(cells.astype(np.float64), kref, m, s, w, 1 / T, steps, target,
                                                 clip='ste')
    assert abs(L - Lr) <= 1e-5 * abs(Lr) + 1e-9
    assert relerr(gc, rc) <= REL
    assert relerr(gk, rk) <= REL
    assert abs(gm - rm) <= REL * abs(rm) + 1e-9
    assert abs(gs - rs) <= REL * abs(rs) + 1e-9


def test_adjoint_mask_clip_matches_float64_autograd(cuda):
    # mask clip = the exact derivative of the clipped map.  The clipped map has
    # kinks wherever a cell's s + dt f crosses 0 or 1, so central differences
    # of it are unstable (they move by ~0.3 % between h = 1e-5, 1e-6, 1e-7 on
    # this case); the float64 autograd of the same piecewise map is the check.
    steps, T, w, m, s = 10, 10.0, 1.0, 0.15, 0.02
    upd, k_real, cells, target = _setup(cuda, steps=steps, n_init=1, seed=9)
    L, gc, gk, gm, gs, gw = _engine_grads(cuda, upd, k_real, cells, target, m, s, w, T, steps, 'mask', ckpt=3)
    kref = k_real.detach().cpu().double().numpy()
    Lr, (rc, rk, rm, rs, rw) = GO.loss_and_grads(cells.astype(np.float64), kref, m, s, w, 1 / T, steps, target,
                                                 clip='mask')
    assert relerr(gc, rc) <= REL
    assert relerr(gk, rk) <= REL
    assert abs(gm - rm) <= REL * abs(rm)
    assert abs(gs - rs) <= REL * abs(rs)


@pytest.mark.parametrize('state_slug', ['v2', 'simple'])
def test_adjoint_matches_central_differences_on_smooth_updates(cuda, state_slug):
    # unclipped state updates (get_state_v2 / get_state_simple, core.py:275-319)
    # are smooth: FP64 central differences with h = 1e-6 are a stable check of
    # the adjoint (correlation, growth derivatives, parameter gradients)
    size, R, steps, T, w, m, s = 64, 10, 8, 10.0, 1.0, 0.15, 0.03
    kp = bump_kernel_params(m=m, s=s)
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], [size, size], 1, R, True, cuda)
    upd = helpers.build_update_fn(K.shape, mp, state_slug)
    k_real = lgrad.ring_kernel(R, 1.0, torch.tensor([1.0], device=cuda), 'gauss_bump', [1.0], [size, size])
    cells = patch_init(1, size, size // 2, seed=21, scale_range=(0.6, 1.0))
    target = patch_init(1, size, size // 2, seed=121) * 0.5
    L, gc, gk, gm, gs, gw = _engine_grads(cuda, upd, k_real, cells, target, m, s, w, T, steps, 'ste', ckpt=3)
    kref = k_real.detach().cpu().double().numpy()
    c64 = cells.astype(np.float64)

    def loss_of(cm=c64, km=kref, mm=m, sm=s):
        with torch.no_grad():
            fin = GO.rollout(torch.from_numpy(cm), torch.from_numpy(km), mm, sm, w, 1 / T, steps,
                             state_slug=state_slug)
            return float(((fin - torch.from_numpy(target.astype(np.float64)))**2).mean())

    fd_m = GO.fd_grad(lambda x: loss_of(mm=float(x[0])), np.array([m]), [0])[0]
    fd_s = GO.fd_grad(lambda x: loss_of(sm=float(x[0])), np.array([s]), [0])[0]
    assert abs(gm - fd_m) <= REL * abs(fd_m), (gm, fd_m)
    assert abs(gs - fd_s) <= REL * abs(fd_s), (gs, fd_s)
    flat = np.argsort(-np.abs(gc.ravel()))[:4]
    fd_c = GO.fd_grad(lambda x: loss_of(cm=x), c64, flat)
    assert np.abs(gc.ravel()[flat] - fd_c).max() <= REL * np.abs(fd_c).max()
    kflat = np.argsort(-np.abs(gk.ravel()))[:3]
    fd_k = GO.fd_grad(lambda x: loss_of(km=x), kref, kflat)
    assert np.abs(gk.ravel()[kflat] - fd_k).max() <= REL * np.abs(fd_k).max()


def test_ring_weight_gradient_through_kernel_builder(cuda):
    # two rings so dL/db is not identically zero (one ring cancels in the normalisation)
    size, R, steps, T, m, s = 64, 10, 8, 10.0, 0.15, 0.02
    upd, _, cells, target = _setup(cuda, size=size, R=R, steps=steps, n_init=1)
    b = torch.tensor([0.5, 1.0], device=cuda, requires_grad=True)
    kr = lgrad.ring_kernel(R, 1.0, b, 'gauss_bump', [1.0], [size, size])
    c0 = torch.from_numpy(cells[None]).to(cuda)
    fin = lgrad.rollout(c0, kr[None], torch.tensor([[[m, s]]], device=cuda), torch.ones((1, 1, 1), device=cuda),
                        torch.tensor([T]), upd, steps, 4, 'ste')
    loss = ((fin - torch.from_numpy(target[None]).to(cuda))**2).mean()
    (gb, ) = torch.autograd.grad(loss, [b])
    # float64 reference built from the oracle: each ring of circle_2d
    # (kernels.py:176-212) unnormalised and placed on the world (pad +
    # fftshift); the kernel is sum_j b_j ring_j / sum_j b_j sum(ring_j), so
    # autograd differentiates the normalisation too
    rings = np.stack([O.world_kernel(R, [1.0, list(onehot)], 'gauss_bump', [1.0], [size, size], normalize=False)
                      for onehot in ([1.0, 0.0], [0.0, 1.0])])
    rings = torch.from_numpy(rings)
    b64 = torch.tensor([0.5, 1.0], dtype=torch.float64, requires_grad=True)
    kr64 = (b64[:, None, None] * rings).sum(0) / (b64 * rings.sum(dim=(1, 2))).sum()
    fin64 = GO.rollout(torch.from_numpy(cells.astype(np.float64)), kr64, m, s, 1.0, 1 / T, steps, clip='ste')
    l64 = ((fin64 - torch.from_numpy(target.astype(np.float64)))**2).mean()
    (gb64, ) = torch.autograd.grad(l64, [b64])
    assert relerr(gb.cpu().numpy(), gb64.numpy()) <= REL
