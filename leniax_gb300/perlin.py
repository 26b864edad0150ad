"""2D Perlin noise (leniax ``perlin.py``): the noise a Perlin initial state is
made of, from given lattice gradient angles.  ``lgx_init_cells`` builds the
Perlin initial states on the device in one launch; this module gives the
noise itself for callers of ``generate_perlin_noise_2d``, as torch ops on the
angles' device."""
import math
from typing import Sequence

import torch


def interpolant(t):
    """perlin.py:12-13: the quintic fade 6t^5 - 15t^4 + 10t^3."""
    return t * t * t * (t * (t * 6 - 15) + 10)


def generate_perlin_noise_2d(angles, shape: Sequence[int], res: Sequence[int], nb_noise: int = 1,
                             interpolant=interpolant) -> torch.Tensor:
    """perlin.py:16-71: ``[nb_noise, *shape]`` noise from the gradient angles
    ``[nb_noise, res0, res1]`` (radians) of a lattice of ``res`` periods that
    wraps around.  Pixel (i, j) lies in lattice cell (i // d0, j // d1), d =
    shape // res, at fraction (i mod d0 / d0, j mod d1 / d1); each corner
    contributes the dot product of its unit gradient (cos a, sin a) with the
    offset from that corner, blended by the fade of the fractions, times
    sqrt(2)."""
    a = torch.as_tensor(angles)
    if not a.is_floating_point():
        a = a.to(torch.float32)
    if a.dim() == 2:
        a = a[None]
    H, W = int(shape[0]), int(shape[1])
    r0, r1 = int(res[0]), int(res[1])
    if tuple(a.shape[1:]) != (r0, r1):
        raise ValueError(f'angles {tuple(a.shape)} are not [nb_noise, {r0}, {r1}]')
    if H % r0 or W % r1:
        raise ValueError(f'shape {shape} must be a multiple of res {res}')
    d0, d1 = H // r0, W // r1
    i = torch.arange(H, device=a.device)
    j = torch.arange(W, device=a.device)
    fx = ((i % d0).to(a.dtype) / d0)[:, None]  # [H, 1]
    fy = ((j % d1).to(a.dtype) / d1)[None, :]  # [1, W]
    ci, cj = (i // d0)[:, None], (j // d1)[None, :]
    gx, gy = torch.cos(a), torch.sin(a)

    def corner(di, dj):
        ii, jj = (ci + di) % r0, (cj + dj) % r1
        return (fx - di) * gx[:, ii, jj] + (fy - dj) * gy[:, ii, jj]  # [n, H, W]

    tx, ty = interpolant(fx), interpolant(fy)
    n0 = corner(0, 0) * (1 - tx) + tx * corner(1, 0)
    n1 = corner(0, 1) * (1 - tx) + tx * corner(1, 1)
    return math.sqrt(2) * ((1 - ty) * n0 + ty * n1)
