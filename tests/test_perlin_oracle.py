"""The oracle's restatement of leniax's Perlin initial states
(perlin.py:16-71, initializations.py:35-116, loader.py:16-30): invariants of
the construction, checked on the CPU."""
import numpy as np

from oracle import lenia_oracle as O


def _angles(n, res, seed=0):
    return np.random.Generator(np.random.PCG64(seed)).random((n, ) + tuple(res)) * 2 * np.pi


def test_noise_vanishes_on_the_lattice_and_is_bounded():
    # shape a multiple of the periods: every lattice point has zero ramps, so
    # the noise is 0 there; |noise| <= sqrt(2) * max |ramp . gradient| <= 2
    res, shape = (4, 8), (64, 128)
    n = O.perlin_noise_2d(_angles(3, res), shape, res)
    assert n.shape == (3, 64, 128)
    assert np.abs(n[:, ::16, ::16]).max() < 1e-12
    assert np.abs(n).max() <= 2.0


def test_noise_is_the_gradient_dot_product_next_to_a_lattice_point():
    # one cell right of the origin: ramps (0, 1/d), the interpolant ~0, so the
    # noise is sqrt(2) * g00 . ramp = sqrt(2) * sin(a00) / d to first order
    res, shape = (2, 2), (64, 64)
    a = _angles(1, res, seed=3)
    n = O.perlin_noise_2d(a, shape, res)
    d = shape[1] // res[1]
    assert abs(n[0, 0, 1] - np.sqrt(2) * np.sin(a[0, 0, 0]) / d) < 1e-3


def test_perlin_init_normalises_scales_and_rounds():
    world, R, m, nb = [128, 128], 13, 0.15, 4
    res = O.perlin_res(world, R)
    assert res == [128 // 39, 128 // 26]
    cells = O.perlin_init(_angles(nb, res), world, R, m)
    assert cells.shape == (nb, 1, 128, 128) and cells.dtype == np.float32
    q = cells * (O.NB_CHARS**2 - 1)
    assert np.abs(q - np.round(q)).max() < 1e-2  # on the compressible grid
    for i in range(nb):
        scale = m + i / nb * (min(1, 3 * m) - m)
        assert cells[i].min() == 0.0 and abs(cells[i].max() - scale) <= 1 / (O.NB_CHARS**2 - 1)


def test_cropped_perlin_keeps_one_centred_square():
    world, R, m = [128, 128], 13, 0.2
    a = _angles(2, O.perlin_res(world, R), seed=5)
    full = O.perlin_init(a, world, R, m)
    crop = O.cropped_perlin_init(a, world, R, m)
    size = 2 * 13
    lo = (128 - size) // 2
    np.testing.assert_array_equal(crop[:, :, lo:lo + size, lo:lo + size], full[:, :, 24:24 + size, 24:24 + size])
    crop[:, :, lo:lo + size, lo:lo + size] = 0
    assert not crop.any()


def test_product_noise_function_matches_the_oracle():
    # leniax_gb300.perlin.generate_perlin_noise_2d (the torch form of perlin.py:16-71)
    import torch
    from leniax_gb300 import perlin
    for res, shape, n in (((4, 8), (64, 128), 3), ((3, 2), (48, 40), 2), ((1, 1), (16, 16), 1)):
        a = _angles(n, res, seed=sum(shape))
        want = O.perlin_noise_2d(a, shape, res)
        got = perlin.generate_perlin_noise_2d(torch.from_numpy(a), shape, res, n).numpy()
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)
        got32 = perlin.generate_perlin_noise_2d(torch.from_numpy(a.astype(np.float32)), shape, res, n).numpy()
        np.testing.assert_allclose(got32, want, atol=2e-6)
    assert abs(float(perlin.interpolant(torch.tensor(0.5))) - 0.5) < 1e-12
