"""Host kernel builders beyond circle_2d (leniax kernels.py:214-317) and the
kernel-function registry (kernel_functions.py:253-261), on the CPU.  The
ellipse builders are tied to ``circle_2d`` (pinned by the reference's
``test_circle_2d`` known answer): with semi-axes a = b = 1 and no rotation
their distances are the circle's, and a quarter turn transposes them."""
import math

import numpy as np
import pytest
import torch

from leniax_gb300 import kernel_functions, kernels

R = 12.0


def _first_coordinate(r):
    k = math.ceil(r * R)
    return (np.indices([2 * k, 2 * k])[0].astype(np.float32) - np.float32(k)) / np.float32(r * R)


@pytest.mark.parametrize('bs,kf,kfp', [([1.0], 'gauss_bump', [4.0]), ([0.3, 1.0, 0.6], 'poly_quad', [4.0]),
                                       ([1.0, 0.5], 'step', [0.5, 0.3])])
def test_ellipse_of_unit_axes_is_the_signed_circle(bs, kf, kfp):
    circle = kernels.circle_2d(R, [1.0, bs], kf, kfp)[0]
    x = _first_coordinate(1.0)
    sign = np.where(x < -0.01, -1.0, np.where(x > 0.01, 1.0, x)).astype(np.float32)
    got = kernels.ellipse_2d(R, [1.0, bs, 1.0, 1.0, 0.0], kf, kfp)
    assert got.shape == (1, ) + circle.shape and got.dtype == np.float32
    np.testing.assert_allclose(got[0], circle * sign, rtol=1e-6, atol=1e-9)
    oriented = kernels.oriented_ellipse_2d(R, [1.0, bs, 1.0, 1.0, 0.0], kf, kfp)
    want = circle * x
    np.testing.assert_allclose(oriented[0], want / np.abs(want).sum(), rtol=1e-5, atol=1e-9)
    assert abs(float(np.abs(oriented).sum()) - 1.0) < 1e-5


@pytest.mark.parametrize('builder', [kernels.ellipse_2d, kernels.oriented_ellipse_2d])
def test_a_quarter_turn_transposes_the_ellipse(builder):
    kp = [0.8, [0.5, 1.0], 0.9, 0.55]
    flat = builder(R, kp + [0.0], 'gauss_bump', [4.0])[0]
    turned = builder(R, kp + [0.5], 'gauss_bump', [4.0])[0]
    np.testing.assert_allclose(turned, flat.T, atol=2e-6)
    assert np.abs(flat - flat.T).max() > 1e-3  # a != b: the turn is not the identity


def test_registers_and_the_builder_use_them():
    assert set(kernels.register) == {'raw', 'circle_2d', 'ellipse_2d', 'oriented_ellipse_2d'}
    assert kernel_functions.register is kernels.kf_register
    assert set(kernel_functions.register) == {'poly_quad', 'gauss_bump', 'gauss', 'step', 'threshold', 'staircase',
                                              'triangle'}
    world = [48, 40]
    kp = [{'k_slug': 'ellipse_2d', 'k_params': [1.0, [1.0], 1.0, 0.7, 0.25], 'kf_slug': 'gauss_bump',
           'kf_params': [4.0], 'gf_slug': 'gaussian', 'gf_params': [0.15, 0.015], 'h': 1.0, 'c_in': 0, 'c_out': 0}]
    K, _ = kernels.get_kernels_and_mapping([dict(p) for p in kp], world, 1, R, True, torch.device('cpu'))
    # the spectrum is the fftn of the fftshifted world-centred kernel (kernels.py:145-152)
    k = kernels.ellipse_2d(R, kp[0]['k_params'], 'gauss_bump', [4.0])[0]
    pads = [((w - s) // 2, (w - s) // 2 + (w - s) % 2) for w, s in zip(world, k.shape)]
    spatial = np.fft.ifftshift(np.real(np.fft.ifftn(K[0, 0, 0].numpy())))
    np.testing.assert_allclose(spatial, np.pad(k, pads), atol=1e-7)
    # a kernel function registered by the user reaches the builder
    kernel_functions.register['flat'] = lambda params, X: np.ones_like(X)
    try:
        kp2 = [dict(kp[0], k_slug='circle_2d', k_params=[1.0, [1.0]], kf_slug='flat', kf_params=[])]
        K2, _ = kernels.get_kernels_and_mapping(kp2, world, 1, R, True, torch.device('cpu'))
        disc = np.fft.ifftshift(np.real(np.fft.ifftn(K2[0, 0, 0].numpy())))
        inside = disc > 1e-6
        assert np.allclose(disc[inside], disc[inside].max(), rtol=1e-4)  # a flat disc
    finally:
        del kernel_functions.register['flat']
