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
