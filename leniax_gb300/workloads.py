"""Seeded synthetic workloads of the benchmark (numpy PCG64).

* uneven search batch: worlds of several shapes, each a C = K = 1 Lenia world
  with the one-ring gauss_bump kernel (k_params [1, [1]]) at its own R,
  gaussian growth with its own (m, s) and its own dt = 1/T, initialised with
  uniform[0, 1) noise in a central patch of side size/3 scaled by a
  per-world factor in [0.5, 1];
* multi-channel model: C channels, K kernels drawn from a seed (per-kernel R,
  1-3 rings, growth m and s, target-channel weights normalised per channel),
  worlds initialised with uniform[0, 1) central patches per channel."""
from typing import List, Sequence, Tuple

import numpy as np
import torch

from .batch import WorldClass, world_spectra

RING = {'k_slug': 'circle_2d', 'k_params': [1.0, [1.0]], 'kf_slug': 'gauss_bump', 'kf_params': [1.0],
        'gf_slug': 'gaussian', 'gf_params': [0.15, 0.015], 'h': 1.0, 'c_in': 0, 'c_out': 0}

# 4096 worlds: 50 % 64^2, 30 % 128^2, 15 % 256^2, 5 % 3D 64^3
SEARCH_MIX = [((64, 64), 2048), ((128, 128), 1229), ((256, 256), 614), ((64, 64, 64), 205)]


def class_inputs(world: Sequence[int], n: int, rng: np.random.Generator, R_range=(5, 26), m_range=(0.1, 0.35),
                 s_range=(0.01, 0.05), dts=(0.05, 0.1, 0.2)) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(cells [n, *world] float32, R [n], params [n, 3] = m, s, T)."""
    world = tuple(int(w) for w in world)
    nd = len(world)
    size = world[0]
    p = size // 3
    lo = (size - p) // 2
    cells = np.zeros((n, ) + world, np.float32)
    noise = rng.random((n, ) + (p, ) * nd, dtype=np.float32)
    f = rng.uniform(0.5, 1.0, size=(n, ) + (1, ) * nd).astype(np.float32)
    cells[(slice(None), ) + (slice(lo, lo + p), ) * nd] = noise * f
    R = rng.integers(R_range[0], R_range[1] + 1, size=n).astype(np.float32)
    m = rng.uniform(*m_range, size=n).astype(np.float32)
    s = rng.uniform(*s_range, size=n).astype(np.float32)
    T = (1.0 / rng.choice(np.asarray(dts, np.float64), size=n)).astype(np.float32)
    return cells, R, np.stack([m, s, T], 1)


def build_classes(mix=SEARCH_MIX, seed=3, device=None) -> List[WorldClass]:
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for world, n in mix:
        cells, R, p = class_inputs(world, n, rng)
        K = world_spectra(world, R, RING, device)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(K.device)
        out.append(WorldClass(cells0=t(cells), K=K, gf_params=t(p[:, :2]), weights=torch.ones(n, device=K.device),
                              T=t(p[:, 2]), R=t(R)))
    return out


def multichannel_params(C=3, per_channel=5, seed=0, R_range=(10, 20), world_R=20.0, m_range=(0.1, 0.4),
                        s_range=(0.01, 0.05)):
    """leniax kernels_params list of C * per_channel ring kernels: kernel
    radius R_k in R_range expressed as k_params r = R_k / world_R, 1-3 rings
    with b in [0, 1] (the largest set to 1), gauss_bump kernel function,
    gaussian growth (m, s), a random target channel and weight h in [0, 1],
    h normalised so the weights into each target channel sum to 1."""
    rng = np.random.Generator(np.random.PCG64(seed))
    params = []
    for c_in in range(C):
        for _ in range(per_channel):
            nb = int(rng.integers(1, 4))
            b = [float(x) for x in rng.random(nb)]
            b[int(np.argmax(b))] = 1.0
            params.append({
                'k_slug': 'circle_2d', 'k_params': [float(rng.uniform(*R_range)) / world_R, b],
                'kf_slug': 'gauss_bump', 'kf_params': [1.0], 'gf_slug': 'gaussian',
                'gf_params': [float(rng.uniform(*m_range)), float(rng.uniform(*s_range))],
                'h': float(rng.random()), 'c_in': c_in, 'c_out': int(rng.integers(0, C))
            })
    for c_out in range(C):
        tot = sum(p['h'] for p in params if p['c_out'] == c_out)
        for p in params:
            if p['c_out'] == c_out and tot > 0:
                p['h'] = p['h'] / tot
    return params


def multichannel_cells(n, C, size, patch, seed=0) -> np.ndarray:
    """[n, C, size, size] float32: uniform[0, 1) in a central patch per channel."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cells = np.zeros((n, C, size, size), np.float32)
    lo = (size - patch) // 2
    cells[:, :, lo:lo + patch, lo:lo + patch] = rng.random((n, C, patch, patch), dtype=np.float32)
    return cells
