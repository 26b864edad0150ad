"""The float64 gradient oracle is pinned to central finite differences (CPU)."""
import numpy as np
import torch

from oracle import lenia_grad_oracle as GO
from tests.cases import patch_init


def _kernel(size=32, R=6):
    from oracle import lenia_oracle as O
    k = O.circle_kernel(R, [1.0, [0.5, 1.0]], 'gauss_bump', [1.0], 2, np.float64)[0]
    pad = [((size - k.shape[0]) // 2, size - k.shape[0] - (size - k.shape[0]) // 2)] * 2
    return np.fft.fftshift(np.pad(k, pad))


def test_mask_clip_autograd_matches_central_differences():
    size, steps, dt, m, s, w = 32, 6, 0.1, 0.15, 0.02, 1.0
    cells = patch_init(1, size, 14, seed=3).astype(np.float64)
    target = patch_init(1, size, 14, seed=4).astype(np.float64) * 0.5
    k = _kernel(size)
    L, (gc, gk, gm, gs, gw) = GO.loss_and_grads(cells, k, m, s, w, dt, steps, target, clip='mask')

    def loss_of(cm=cells, km=k, mm=m, sm=s):
        with torch.no_grad():
            fin = GO.rollout(torch.from_numpy(cm), torch.from_numpy(km), mm, sm, w, dt, steps, clip='mask')
        return float(((fin - torch.from_numpy(target))**2).mean())

    assert abs(GO.fd_grad(lambda x: loss_of(mm=float(x[0])), np.array([m]), [0])[0] - gm) <= 1e-5 * abs(gm)
    assert abs(GO.fd_grad(lambda x: loss_of(sm=float(x[0])), np.array([s]), [0])[0] - gs) <= 1e-5 * abs(gs)
    idx = np.argsort(-np.abs(gc.ravel()))[:3]
    fd = GO.fd_grad(lambda x: loss_of(cm=x), cells, idx)
    assert np.abs(fd - gc.ravel()[idx]).max() <= 1e-5 * np.abs(fd).max()
    kidx = np.argsort(-np.abs(gk.ravel()))[:3]
    fdk = GO.fd_grad(lambda x: loss_of(km=x), k, kidx)
    assert np.abs(fdk - gk.ravel()[kidx]).max() <= 1e-5 * np.abs(fdk).max()


def test_ste_and_mask_agree_without_clipping():
    # state v2 has no clip: both clip modes are the same function
    size, steps = 32, 5
    cells = patch_init(1, size, 14, seed=6).astype(np.float64) * 0.5
    k = _kernel(size)
    a = GO.loss_and_grads(cells, k, 0.15, 0.03, 1.0, 0.1, steps, cells, clip='ste', state_slug='v2')
    b = GO.loss_and_grads(cells, k, 0.15, 0.03, 1.0, 0.1, steps, cells, clip='mask', state_slug='v2')
    assert abs(a[0] - b[0]) < 1e-15
    for x, y in zip(a[1], b[1]):
        np.testing.assert_allclose(x, y, rtol=1e-12, atol=1e-15)
