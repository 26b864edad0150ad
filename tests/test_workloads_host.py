"""The benchmark's seeded workload generators and the host helpers of the
initial states, on the CPU: the uneven batch's class mix and per-world
ranges, the multi-channel model's kernels and weights, the SplitMix64 seed
step (a published known answer), the Perlin periods and the compressible
rounding."""
import math

import numpy as np
import torch

from leniax_gb300 import initializations, workloads
from leniax_gb300.constant import NB_CHARS
from oracle import lenia_oracle as O


def test_search_mix_is_the_largest_remainder_split_of_4096():
    shares = [0.50, 0.30, 0.15, 0.05]
    exact = [4096 * s for s in shares]
    counts = [math.floor(e) for e in exact]
    for i in sorted(range(4), key=lambda i: -(exact[i] - counts[i]))[:4096 - sum(counts)]:
        counts[i] += 1
    assert [n for _, n in workloads.SEARCH_MIX] == counts == [2048, 1229, 614, 205]
    assert [w for w, _ in workloads.SEARCH_MIX] == [(64, 64), (128, 128), (256, 256), (64, 64, 64)]


def test_class_inputs_ranges_and_patches():
    rng = np.random.Generator(np.random.PCG64(0))
    for world in ((64, 64), (32, 32, 32)):
        cells, R, p = workloads.class_inputs(world, 12, rng)
        size, nd = world[0], len(world)
        lo, q = (size - size // 3) // 2, size // 3
        inside = (slice(None), ) + (slice(lo, lo + q), ) * nd
        assert cells.shape == (12, ) + world and cells.dtype == np.float32
        outside = cells.copy()
        outside[inside] = 0
        assert not outside.any() and 0 <= cells.min() and cells.max() < 1
        assert np.all(R == np.round(R)) and R.min() >= 5 and R.max() <= 26
        m, s, T = p.T
        assert np.all((0.1 <= m) & (m < 0.35)) and np.all((0.01 <= s) & (s < 0.05))
        assert set(np.unique(T)) <= {np.float32(20), np.float32(10), np.float32(5)}


def test_multichannel_model_kernels_and_weights():
    kp = workloads.multichannel_params(3, 5, seed=0)
    assert len(kp) == 15 and [sum(p['c_in'] == c for p in kp) for c in range(3)] == [5, 5, 5]
    for p in kp:
        r, b = p['k_params']
        assert 0.5 <= r < 1.0 and 1 <= len(b) <= 3 and max(b) == 1.0
        assert 0.1 <= p['gf_params'][0] < 0.4 and 0.01 <= p['gf_params'][1] < 0.05
    for c in range(3):
        hs = [p['h'] for p in kp if p['c_out'] == c]
        assert not hs or abs(sum(hs) - 1.0) < 1e-12  # weights into each fed channel sum to 1
    cells = workloads.multichannel_cells(2, 3, 32, 10, seed=1)
    assert cells.shape == (2, 3, 32, 32) and not cells[:, :, :11].any() and cells[:, :, 11:21, 11:21].all()


def test_seed_step_perlin_periods_and_compressible_rounding():
    # SplitMix64: the first output from state 0 is 0xE220A8397B1DCDAF (Steele, Lea, Flood 2014)
    assert initializations.next_key(0) == 0xE220A8397B1DCDAF
    keys = [initializations.next_key(s) for s in range(64)]
    assert len(set(keys)) == 64 and all(0 <= k < 2**64 for k in keys)
    for world, R in (([128, 128], 13), ([256, 128], 9.5), ([64, 64], 20)):
        assert list(initializations.perlin_res(world, R)) == list(O.perlin_res(world, R))
    x = torch.rand(1000, dtype=torch.float32)
    q = initializations.make_array_compressible(x)
    grid = q * (NB_CHARS**2 - 1)
    assert torch.allclose(grid, grid.round(), atol=1e-3) and (q - x).abs().max() <= 0.5 / (NB_CHARS**2 - 1) + 1e-7
    assert torch.equal(initializations.make_array_compressible(q), q)
