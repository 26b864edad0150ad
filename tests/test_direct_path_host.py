"""The direct-convolution path's kernels (leniax ``fft=False``,
kernels.py:66-158 with utils.crop_zero): the product's cropped real kernels
``[C*max_k, 1, *kernel_dims]`` equal the oracle's, value for value, for the
golden models and a 3D world.  Host-only."""
import numpy as np
import pytest

from leniax_gb300 import kernels
from oracle import lenia_oracle as O
from tests.cases import bump_kernel_params, golden_case


def _both(kp, world, C, R):
    Kp, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], list(world), C, R, False, 'cpu')
    Ko, mpo = O.get_kernels_and_mapping([dict(p) for p in kp], list(world), C, R, False, np.float32)
    return Kp.numpy(), mp, Ko, mpo


@pytest.mark.parametrize('name', ['orbium', 'orbium_scutium', 'aquarium'])
def test_direct_kernels_match_the_oracle(name):
    cfg, _, _ = golden_case(name)
    Kp, mp, Ko, mpo = _both(cfg['kernels_params'], cfg['world_size'], cfg['nb_channels'], cfg['R'])
    assert Kp.shape == Ko.shape and Kp.shape[1] == 1
    assert Kp.shape[0] == cfg['nb_channels'] * max(map(len, mp.cin_kernels))
    assert (mp.true_channels is None) == (mpo['true_channels'] is None)
    np.testing.assert_allclose(Kp, Ko, rtol=1e-6, atol=1e-9)


def test_direct_kernels_3d_and_crop():
    Kp, mp, Ko, _ = _both(bump_kernel_params(), [24, 20, 16], 1, 5.0)
    # a ring of radius 5 cropped to its support (the bump is zero on the rim)
    assert Kp.shape == Ko.shape and Kp.shape[:2] == (1, 1) and len(set(Kp.shape[2:])) == 1
    assert Kp.shape[2] % 2 == 1 and Kp.shape[2] < 11
    np.testing.assert_allclose(Kp, Ko, rtol=1e-6, atol=1e-9)


def test_crop_zero_removes_every_all_zero_index():
    # utils.py:296-317 drops interior all-zero rows too, not only the border
    k = np.zeros((2, 5, 6), np.float32)
    k[0, 0, 1] = 1
    k[1, 4, 4] = 2
    k[0, 2, 5] = 3
    got = kernels.crop_zero(k)
    want = O.crop_zero(k)
    assert got.shape == want.shape == (2, 3, 3)  # rows 0, 2, 4; columns 1, 4, 5
    np.testing.assert_array_equal(got, want)


def test_crop_zero_kat():
    # tests/test_utils.py:20-43: two 4 x 4 kernels cropped to their common 2 x 3 support
    k = np.zeros((2, 4, 4), np.float32)
    k[0, 1, 1] = k[0, 2, 1] = k[0, 2, 2] = 1
    k[1, 1, 2] = k[1, 1, 3] = k[1, 2, 1] = 1
    want = np.array([[[1, 0, 0], [1, 1, 0]], [[0, 1, 1], [1, 0, 0]]], np.float32)
    np.testing.assert_array_equal(O.crop_zero(k), want)
    np.testing.assert_array_equal(kernels.crop_zero(k), want)


@pytest.mark.parametrize('shape', [(4, 1, 3, 3), (2, 1, 8, 6), (1, 1, 5, 4, 7)])
def test_potential_builder_pads_like_the_reference(shape):
    # helpers.py:465-481: (d // 2, d // 2 - 1) for even kernel sides,
    # (d // 2, d // 2) for odd ones, after the batch and channel axes
    from leniax_gb300 import helpers
    fn = helpers.build_get_potential_fn(shape, [True] * shape[0], fft=False)
    want = [(0, 0), (0, 0)] + [(d // 2, d // 2 - 1) if d % 2 == 0 else (d // 2, d // 2) for d in shape[2:]]
    assert list(fn.keywords['padding']) == want
    assert fn.keywords['tc_indices'] == tuple(range(shape[0]))
    assert list(fn.keywords['padding']) == list(O.conv_padding(shape))


def test_field_builder_flattens_growth_functions_in_channel_order():
    # helpers.py:490-516: the growth functions of every channel, in order,
    # and the weighted mean (or sum)
    from leniax_gb300 import core, growth_functions, helpers
    fn = helpers.build_get_field_fn([['gaussian', 'poly_quad4'], [], ['step']], average=False)
    assert fn.keywords['growth_fn_t'] == (growth_functions.gaussian, growth_functions.poly_quad4,
                                          growth_functions.step)
    assert fn.keywords['weighted_fn'] is core.weighted_sum
    assert helpers.build_get_field_fn([['identity']]).keywords['weighted_fn'] is core.weighted_mean
    assert growth_functions.engine_id('triangle') == growth_functions.triangle.id


def test_check_spectra_names_the_expected_layout():
    # the engine reads [*lead, C, max_k, *world[:-1], W//2+1] complex values through a bare pointer
    from leniax_gb300.core import check_spectra
    import torch
    check_spectra(torch.zeros((2, 3, 4, 24, 17, 2)), (2, ), 3, 4, (24, 32))
    check_spectra(torch.zeros((1, 1, 1, 8, 6, 5, 2)), (1, ), 1, 1, (8, 6, 8))
    for bad in ((2, 3, 4, 12, 17, 2), (2, 2, 4, 24, 17, 2), (2, 3, 3, 24, 17, 2), (2, 3, 4, 24, 32, 2),
                (3, 3, 4, 24, 17, 2), (3, 4, 24, 17, 2)):
        with pytest.raises(ValueError, match='do not match'):
            check_spectra(torch.zeros(bad), (2, ), 3, 4, (24, 32))
