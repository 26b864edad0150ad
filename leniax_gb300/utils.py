"""Utilities of leniax ``utils.py`` used around the path: rolling a world
onto its mass centroid and cropping it (``center_world`` 270-293,
``auto_center`` 320-349, ``center_and_crop`` 352-385), what the reference
applies to a found creature before encoding it (``qd.py:422``), as torch ops
on the state's own device (``crop_zero`` is the kernel builder's,
``utils.py:296-317``); the dotted-path configuration accessors
(``get_param`` / ``set_param`` 153-210) and the migration of version-1
configurations, whose kernels are described by numeric ids
(``update_config_v1_v2`` 91-150, ``st2fracs2float`` 214-225)."""
from fractions import Fraction
from typing import Dict, List, Sequence, Tuple

import numpy as np
import torch

from .constant import EPSILON
from .kernels import crop_zero as _crop_zero_np


def center_world(cells: torch.Tensor, field: torch.Tensor, potential: torch.Tensor, shift_idx,
                 axes: Sequence[int]) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """utils.py:270-293: every entry ``b`` of the batch axis rolled by
    ``-shift_idx[b]`` (``[bs, len(axes)]``) over ``axes``."""
    shift = torch.as_tensor(shift_idx).reshape(len(cells), len(axes)).tolist()
    axes = tuple(int(a) for a in axes)

    def roll(t):
        return torch.stack([torch.roll(t[b], [-int(s) for s in shift[b]], [a - 1 if a > 0 else a for a in axes])
                            for b in range(len(t))])

    return roll(cells), roll(field), roll(potential)


def crop_zero(cells: torch.Tensor) -> torch.Tensor:
    """utils.py:296-317 on ``[C, *world]``: every index of a world axis at
    which all channels are zero is dropped."""
    return torch.from_numpy(_crop_zero_np(cells.detach().cpu().numpy())).to(cells.device)


def _mass_shift(cells: torch.Tensor) -> torch.Tensor:
    """round(mass centroid relative to the world's midpoint), per world axis."""
    world = cells.shape[1:]
    coords = torch.stack(torch.meshgrid(*[torch.arange(n, device=cells.device, dtype=torch.float32) - (n // 2)
                                          for n in world], indexing='ij'))
    m00 = cells.sum()
    centroid = torch.stack([(cells * c).sum() for c in coords]) / (m00 + EPSILON)
    return torch.round(centroid).to(torch.int64)


def auto_center(cells: torch.Tensor) -> torch.Tensor:
    """utils.py:320-349: ``cells`` ``[C, *world]`` rolled so that the total
    mass centroid (rounded, half to even) sits at the world's midpoint
    ``size // 2``."""
    axes = tuple(range(-(cells.dim() - 1), 0))
    shift = _mass_shift(cells)
    return center_world(cells[None], cells[None], cells[None], shift[None], axes)[0][0]


def center_and_crop(cells: torch.Tensor) -> torch.Tensor:
    """utils.py:352-385: a pattern cut by a world border (occupied indices at
    both ends of an axis, empty ones in between) is first rolled by half the
    world (the first axis's ``size // 2`` for every axis, as the
    reference), then the state is centred on its mass (:func:`auto_center`)
    and cropped to its support (:func:`crop_zero`); an empty state gives
    zeros ``[C, 1, ...]``."""
    world = cells.shape[1:]
    nd = len(world)
    axes = tuple(range(-nd, 0))
    pre = [0] * nd
    for i in range(nd):
        occupied = (cells != 0).movedim(i + 1, 0).reshape(world[i], -1).any(dim=1)
        if bool(occupied[0]) and bool(occupied[-1]) and not bool(occupied.all()):
            pre[i] = int(world[0] // 2)
    cells = center_world(cells[None], cells[None], cells[None], torch.tensor([pre]), axes)[0][0]
    cells = crop_zero(auto_center(cells))
    if 0 in cells.shape:
        cells = torch.zeros([cells.shape[0]] + [1] * (cells.dim() - 1), dtype=cells.dtype, device=cells.device)
    return cells


# version-1 numeric ids of the growth and kernel functions (utils.py:104-105)
V1_GROWTH_SLUGS = {0: 'poly_quad4', 1: 'gaussian', 2: 'gaussian_target', 3: 'step'}
V1_KERNEL_FUNCTION_SLUGS = {0: 'poly_quad', 1: 'gauss_bump', 2: 'step', 3: 'staircase', 4: 'gauss'}


def st2fracs2float(st: str) -> List[float]:
    """utils.py:214-225: ``'1,2/3,6.7'`` -> ``[1.0, 0.666..., 6.7]``."""
    return [float(Fraction(part)) for part in st.split(',')]


def _v2_key(key: str) -> str:
    # a version-1 parameter path (kernels_params.k.<i>.m / .s) in version-2 terms
    return key.replace('kernels_params.k', 'kernels_params').replace('.m', '.gf_params.0').replace('.s', '.gf_params.1')


def update_config_v1_v2(config: Dict) -> Dict:
    """utils.py:91-150, in place: each version-1 kernel entry (``r``, ring
    weights ``b`` -- a list or a string of fractions --, ``k_id`` / ``q``,
    ``gf_id`` / ``m`` / ``s``, ``h``, ``c_in``, ``c_out``) becomes a
    ``circle_2d`` kernel with its kernel and growth functions named by slug;
    genotype keys and phenotype entries are renamed alike; the initial-state
    slug follows the state function (``perlin`` for v1, ``perlin_local``
    for v2)."""
    config['version'] = 2
    kernels = []
    for k in config['kernels_params']['k']:
        kernels.append({
            'k_slug': 'circle_2d',
            'k_params': [k.get('r', 1.), st2fracs2float(k['b']) if isinstance(k['b'], str) else k['b']],
            'kf_slug': V1_KERNEL_FUNCTION_SLUGS[k['k_id']],
            'kf_params': [k['q']],
            'gf_slug': V1_GROWTH_SLUGS[k['gf_id']],
            'gf_params': [k['m'], k['s']],
            'h': k['h'],
            'c_in': k['c_in'],
            'c_out': k['c_out'],
        })
    config['kernels_params'] = kernels
    for gene in config.get('genotype', []):
        if 'kernels_params.k' in gene['key']:
            gene['key'] = _v2_key(gene['key'])
    if 'phenotype' in config:
        config['phenotype'] = [_v2_key(p) if 'kernels_params.k' in p else p for p in config['phenotype']]
    slug = config['world_params'].get('get_state_fn_slug', 'v1')
    algo = config.setdefault('algo', {})
    if slug == 'v1':
        algo['init_slug'] = 'perlin'
    elif slug == 'v2':
        algo['init_slug'] = 'perlin_local'
    algo['init_param'] = []
    return config


def get_param(dic: Dict, key_string: str):
    """utils.py:153-177"""
    for key in key_string.split('.'):
        dic = dic[int(key)] if key.isdigit() else dic[key]
    if isinstance(dic, torch.Tensor):
        return float(dic.float().mean())
    if isinstance(dic, np.ndarray):
        return float(np.mean(dic))
    if type(dic) in (int, float):
        return float(dic)
    if type(dic) == str:
        return dic
    raise ValueError(f'dic type {type(dic)} not supported')


def set_param(dic: Dict, key_string: str, value):
    """utils.py:180-210"""
    keys = key_string.split('.')
    for i, key in enumerate(keys[:-1]):
        if key.isdigit():
            if not isinstance(dic, list):
                raise Exception('This key should be an array')
            idx = int(key)
            while len(dic) < idx + 1:
                dic.append({})
            dic = dic[idx]
        else:
            dic = dic.setdefault(key, [] if keys[i + 1].isdigit() else {})
    last = keys[-1]
    if last.isdigit():
        idx = int(last)
        while len(dic) < idx + 1:
            dic.append(None)
        dic[idx] = value
    else:
        dic[last] = value


__all__ = ['center_world', 'crop_zero', 'auto_center', 'center_and_crop', 'st2fracs2float', 'update_config_v1_v2',
           'get_param', 'set_param']
