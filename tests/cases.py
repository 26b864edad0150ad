"""Shared test cases: golden fixtures and seeded synthetic worlds.

Inputs are generated with numpy PCG64 so the oracle and the engine consume
identical bytes."""
import json
import os

import numpy as np

from oracle import lenia_oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def golden_case(name):
    cfg = json.load(open(os.path.join(GOLDEN, f'{name}.json')))
    init = np.load(os.path.join(GOLDEN, f'{name}_init.npy'))
    last = np.load(os.path.join(GOLDEN, f'{name}_last.npy'))
    return cfg, init, last


def golden_world(cfg, init, dtype=np.float32):
    cells = O.create_init_cells(cfg['world_size'], cfg['nb_channels'], [init]).astype(dtype)
    K, mp = O.get_kernels_and_mapping(cfg['kernels_params'], cfg['world_size'], cfg['nb_channels'], cfg['R'], True,
                                      dtype)
    return cells, K, mp


# The 1-channel 1-kernel model of the single-world / search-batch workloads:
# R=13, one ring b=[1], kernel exp(4 - 1/(r(1-r))) (= gauss_bump q=1 up to a
# constant the sum-normalisation cancels), gaussian growth m=0.15 s=0.015.
def bump_kernel_params(m=0.15, s=0.015, r=1.0, b=(1.0, ), q=1.0):
    return [{
        'k_slug': 'circle_2d', 'k_params': [r, list(b)], 'kf_slug': 'gauss_bump', 'kf_params': [q],
        'gf_slug': 'gaussian', 'gf_params': [m, s], 'h': 1.0, 'c_in': 0, 'c_out': 0
    }]


def patch_init(n, size, patch, seed=0, scale_range=None, channels=1):
    """n worlds [n, C, size, size]: uniform[0,1) in a central patch x patch
    square (per-world factor in scale_range if given), zeros elsewhere."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cells = np.zeros((n, channels, size, size), dtype=np.float32)
    lo = (size - patch) // 2
    noise = rng.random((n, channels, patch, patch), dtype=np.float32)
    if scale_range is not None:
        f = rng.uniform(scale_range[0], scale_range[1], size=(n, 1, 1, 1)).astype(np.float32)
        noise = noise * f
    cells[:, :, lo:lo + patch, lo:lo + patch] = noise
    return cells


def random_multichannel_params(C, per_channel, seed, R_range=(10, 20), world_R=None):
    """Seeded multi-channel kernel set: per_channel kernels per input channel,
    1-3 rings with b in [0,1], growth m in [0.1,0.4], s in [0.01,0.05],
    target-channel weights in [0,1]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    params = []
    for c_in in range(C):
        for j in range(per_channel):
            nb = int(rng.integers(1, 4))
            b = [float(x) for x in rng.random(nb)]
            b[int(rng.integers(0, nb))] = 1.0
            params.append({
                'k_slug': 'circle_2d',
                'k_params': [float(rng.uniform(R_range[0], R_range[1])) / world_R, b],
                'kf_slug': 'gauss_bump',
                'kf_params': [1.0],
                'gf_slug': 'gaussian',
                'gf_params': [float(rng.uniform(0.1, 0.4)), float(rng.uniform(0.01, 0.05))],
                'h': float(rng.random()),
                'c_in': c_in,
                'c_out': int(rng.integers(0, C)),
            })
    return params
