"""Pipeline builders (leniax ``helpers.py``): ``build_update_fn``
(helpers.py:401-427), ``build_get_potential_fn`` (430-487),
``build_get_field_fn`` (490-516), ``init`` (35-88), ``create_init_cells``
(91-128) and ``init_and_run`` (131-189) for v2 configurations whose cells
are arrays."""
import copy
import functools
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import core as lcore
from . import growth_functions as lgf
from . import kernels as lkernels
from . import runner as lrunner
from . import statistics as lstat
from .core import UpdateFn


def build_update_fn(kernel_shape: Sequence[int], mapping: lkernels.KernelMapping, get_state_fn_slug: str = 'v1',
                    average_weight: bool = True, fft: bool = True) -> UpdateFn:
    """helpers.py:401-427"""
    return UpdateFn(kernel_shape, mapping, get_state_fn_slug, average_weight, fft)


def build_get_potential_fn(kernel_shape: Sequence[int], true_channels: Optional[List[bool]] = None, fft: bool = True,
                           channel_first: bool = True):
    """helpers.py:430-487: ``core.get_potential_fft`` (fft) or
    ``core.get_potential`` with the wrap padding of the kernel shape, keeping
    the true channels."""
    tc_indices = None if true_channels is None else tuple(i for i, t in enumerate(true_channels) if t is True)
    if fft:
        return functools.partial(lcore.get_potential_fft, tc_indices=tc_indices, channel_first=channel_first)
    if not channel_first:
        raise NotImplementedError('the engine takes channel-first states')
    pad = [(0, 0), (0, 0)]
    for d in tuple(kernel_shape)[2:]:
        pad.append((d // 2, d // 2 - 1) if d % 2 == 0 else (d // 2, d // 2))
    return functools.partial(lcore.get_potential, tc_indices=tc_indices, padding=tuple(pad),
                             channel_first=channel_first)


def build_get_field_fn(cin_gfs: List[List[str]], average: bool = True):
    """helpers.py:490-516: ``core.get_field`` with the flattened growth
    functions and the weighted mean (or sum)."""
    growth_fn_t = tuple(lgf.register[slug] for per_channel in cin_gfs for slug in per_channel)
    weighted_fn = lcore.weighted_mean if average else lcore.weighted_sum
    return functools.partial(lcore.get_field, growth_fn_t=growth_fn_t, weighted_fn=weighted_fn)


def merge_cells(cells: np.ndarray, other: np.ndarray, offset=None) -> np.ndarray:
    """utils.py:231-263"""
    assert cells.ndim == other.ndim and cells.shape[0] == other.shape[0]
    offset = offset or [0] * cells.ndim
    pads = []
    for i in range(cells.ndim):
        ps = int(max((cells.shape[i] - other.shape[i]) // 2 + offset[i], 0))
        pads.append((ps, int(cells.shape[i] - other.shape[i] - ps)))
    return cells + np.pad(other, pads)


def create_init_cells(world_size: List[int], nb_channels: int, other_cells=(), offsets=()) -> np.ndarray:
    """helpers.py:91-128 (list-of-patterns form) -> [1, C, *world] float32."""
    cells = np.zeros([nb_channels] + list(world_size), dtype=np.float32)
    offsets = list(offsets)
    for i, c in enumerate(other_cells):
        c = np.asarray(c, dtype=np.float32)
        if c.size:
            cells = merge_cells(cells, c, offsets[i] if len(offsets) == len(other_cells) else None)
    return cells[np.newaxis]


def init(config: Dict, use_init_cells: bool = True, fft: bool = True, device=None):
    """helpers.py:35-88 for cells given as arrays / nested lists."""
    wp, rp = config['world_params'], config['render_params']
    nb_dims, C = wp['nb_dims'], wp['nb_channels']
    world_size = rp['world_size']
    rpp = config['run_params']
    cells = rpp.get('init_cells', rpp.get('cells')) if use_init_cells else rpp.get('cells')
    if isinstance(cells, str):
        raise NotImplementedError('string-encoded cells: decode them to an array before calling init')
    raw_cells = np.asarray(cells, dtype=np.float32)
    if raw_cells.ndim == nb_dims and C == 1:
        raw_cells = raw_cells[np.newaxis]
    if raw_cells.ndim > 1 + nb_dims:
        init_cells = raw_cells
    else:
        init_cells = create_init_cells(world_size, C, [raw_cells])
    K, mapping = lkernels.get_kernels_and_mapping(config['kernels_params'], world_size, C, wp['R'], fft, device)
    return torch.from_numpy(np.ascontiguousarray(init_cells)).to(K.device), K, mapping


def init_and_run(rng_key, config: Dict, use_init_cells: bool = True, with_jit: bool = True, fft: bool = True,
                 stat_trunc: bool = False, device=None, engine: str = 'auto'):
    """helpers.py:131-189"""
    config = copy.deepcopy(config)
    cells, K, mapping = init(config, use_init_cells, fft, device)
    gf_params = mapping.get_gf_params(K.device)
    weights = mapping.get_kernels_weight_per_channel(K.device)
    wp = config['world_params']
    update_fn = build_update_fn(K.shape, mapping, wp.get('get_state_fn_slug', 'v1'), wp.get('weighted_average', True),
                                fft)
    compute_stats_fn = lstat.build_compute_stats_fn(wp, config['render_params'])
    T = torch.tensor(wp['T'], dtype=torch.float32, device=K.device)
    max_run_iter = config['run_params']['max_run_iter']
    if with_jit:
        out = lrunner.run_scan(rng_key, cells, K, gf_params, weights, T, max_run_iter, wp['R'], update_fn,
                               compute_stats_fn, engine)
    else:
        out = lrunner.run(rng_key, cells, K, gf_params, weights, T, max_run_iter, wp['R'], update_fn,
                          compute_stats_fn, stat_trunc, engine)
    all_cells, all_fields, all_pots, stats = out
    stats = {k: v.squeeze() for k, v in stats.items()}
    if stat_trunc:
        n = int(stats['N'])
        all_cells, all_fields, all_pots = all_cells[:n], all_fields[:n], all_pots[:n]
    return all_cells, all_fields, all_pots, stats
