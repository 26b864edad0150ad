"""Centring and cropping of found creatures (leniax utils.py:270-385), on
the CPU, by properties: the mass centroid lands on the midpoint, and a
creature placed anywhere on the torus -- cut by a border or not -- centres
and crops to the same array."""
import numpy as np
import pytest
import torch

from leniax_gb300 import utils


def _creature(C=2, h=7, w=9, seed=0):
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.random((C, h, w)).astype(np.float32) * (rng.random((C, h, w)) > 0.3)
    c[:, 0, 0] = c[:, -1, -1] = 0.5  # a non-empty first and last row and column
    return c


def _place(creature, world, offset):
    out = np.zeros((creature.shape[0], ) + world, np.float32)
    idx = np.ix_(range(creature.shape[0]), *[(np.arange(n) + o) % s for n, o, s in
                                             zip(creature.shape[1:], offset, world)])
    out[idx] = creature
    return torch.from_numpy(out)


def test_auto_center_puts_the_centroid_on_the_midpoint():
    cells = _place(_creature(), (48, 48), (3, 30))
    centred = utils.auto_center(cells)
    coords = np.indices((48, 48)) - 24
    m = centred.numpy().sum(0)
    centroid = np.array([(m * c).sum() for c in coords]) / m.sum()
    assert np.all(np.abs(centroid) <= 0.5 + 1e-4)


@pytest.mark.parametrize('world', [(48, 48), (40, 40)])
def test_center_and_crop_is_translation_invariant_on_the_torus(world):
    creature = _creature(seed=sum(world))
    want = utils.center_and_crop(_place(creature, world, (10, 12)))
    assert want.shape[1:] == creature.shape[1:]  # cropped to the creature's support
    for offset in [(0, 0), (world[0] - 3, 5), (7, world[1] - 4), (world[0] - 2, world[1] - 6)]:
        got = utils.center_and_crop(_place(creature, world, offset))  # the last three cut by a border
        assert torch.equal(got, want), offset


def test_center_world_rolls_each_batch_entry():
    x = torch.arange(2 * 4 * 5, dtype=torch.float32).reshape(2, 4, 5)
    c, f, p = utils.center_world(x, 2 * x, 3 * x, [[1, 2], [0, -1]], (-2, -1))
    assert torch.equal(c[0], torch.roll(x[0], (-1, -2), (0, 1))) and torch.equal(c[1], torch.roll(x[1], (0, 1), (0, 1)))
    assert torch.equal(f, 2 * c) and torch.equal(p, 3 * c)


def test_empty_state_crops_to_zeros():
    got = utils.center_and_crop(torch.zeros(3, 16, 16))
    assert tuple(got.shape) == (3, 1, 1) and float(got.abs().sum()) == 0


def test_st2fracs2float_kat():
    # tests/test_utils.py:11-16
    out = utils.st2fracs2float('1/2,2/3')
    assert out[0] == .5 and out[1] == 2 / 3


@pytest.mark.parametrize('case', ['orbium', 'orbium_scutium', 'aquarium'])
def test_v1_configs_migrate_to_the_golden_kernel_params(case):
    # the fixtures' own v1 kernel entries against the v2 params the golden
    # last frames are reproduced from
    import copy
    import json
    import os
    d = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', f'{case}.json')))
    cfg = {'version': 1, 'world_params': {'get_state_fn_slug': d['get_state_fn_slug']},
           'kernels_params': {'k': copy.deepcopy(d['kernels_params_v1'])}, 'algo': {'init_slug': 'x'},
           'genotype': [{'key': 'kernels_params.k.0.m'}, {'key': 'world_params.R'}],
           'phenotype': ['kernels_params.k.0.s', 'mass']}
    out = utils.update_config_v1_v2(cfg)
    assert out['version'] == 2 and out['kernels_params'] == d['kernels_params']
    assert [g['key'] for g in out['genotype']] == ['kernels_params.0.gf_params.0', 'world_params.R']
    assert out['phenotype'] == ['kernels_params.0.gf_params.1', 'mass']
    assert out['algo'] == {'init_slug': 'perlin' if d['get_state_fn_slug'] == 'v1' else 'perlin_local',
                           'init_param': []}


def test_set_param_kat():
    # tests/test_utils.py:65-93
    dic = {'test': {'hip': 2.}}
    utils.set_param(dic, 'test.hop', 1.)
    assert dic == {'test': {'hip': 2., 'hop': 1.}}
    utils.set_param(dic, 'test.pim.pouf', 1.)
    assert dic == {'test': {'hip': 2., 'hop': 1., 'pim': {'pouf': 1.}}}
    utils.set_param(dic, 'test_arr.0.pouf', 1.)
    assert dic == {'test_arr': [{'pouf': 1}], 'test': {'hip': 2., 'hop': 1., 'pim': {'pouf': 1.}}}
    utils.set_param(dic, 'test_arr.2.woo', 2)
    assert dic == {'test_arr': [{'pouf': 1}, {}, {'woo': 2}], 'test': {'hip': 2., 'hop': 1., 'pim': {'pouf': 1.}}}
    assert utils.get_param(dic, 'test_arr.2.woo') == 2.0 and utils.get_param(dic, 'test.pim.pouf') == 1.0
