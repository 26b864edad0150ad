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
from . import loader as lloader
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
    """helpers.py:35-88: the configuration's cells (encoded strings, nested
    lists or arrays, ``loader.load_raw_cells``) placed in the world."""
    wp, rp = config['world_params'], config['render_params']
    nb_dims, C = wp['nb_dims'], wp['nb_channels']
    world_size = rp['world_size']
    raw_cells = lloader.load_raw_cells(config, use_init_cells).numpy()
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


def _model_setup(config: Dict, use_init_cells: bool, fft: bool, device):
    wp = config['world_params']
    cells, K, mapping = init(config, use_init_cells, fft, device)
    update_fn = build_update_fn(K.shape, mapping, wp.get('get_state_fn_slug', 'v1'), wp.get('weighted_average', True),
                                fft)
    return cells, K, mapping, update_fn, lstat.build_compute_stats_fn(wp, config['render_params'])


def multi_init_and_run(rng_key, main_config: Dict, configs: List[Dict], use_init_cells: bool = True, fft: bool = True,
                       device=None, engine: str = 'auto'):
    """helpers.py:192-237: ``run_scan`` of every configuration in ``configs``
    with the model of ``main_config`` (same shapes; leniax vmaps run_scan
    over them), here one engine launch for all of them.  Returns ``(cells,
    fields, potentials, stats)`` with a leading configuration axis:
    ``[n_cfg, T, N_init, C|K, *world]`` and ``stats[k]`` ``[n_cfg, T,
    N_init]``, squeezed as in the reference."""
    main = copy.deepcopy(main_config)
    wp = main['world_params']
    _, _, _, update_fn, compute_stats_fn = _model_setup(main, use_init_cells, fft, device)
    cells_l, K_l, gf_l, w_l, T_l = [], [], [], [], []
    for cfg in configs:
        cells, K, mapping = init(copy.deepcopy(cfg), use_init_cells, fft, device)
        cells_l.append(cells)
        K_l.append(K[0] if fft else K)
        gf_l.append(mapping.get_gf_params(K.device))
        w_l.append(mapping.get_kernels_weight_per_channel(K.device))
        T_l.append(float(cfg['world_params']['T']))
    dev = cells_l[0].device
    cells0 = torch.stack(cells_l)  # [n_cfg, N_init, C, *world]
    final, stats, ncont, _, traj, _ = lrunner._rollout(update_fn, compute_stats_fn, cells0, torch.stack(K_l),
                                                       torch.stack(gf_l), torch.stack(w_l),
                                                       torch.tensor(T_l, device=dev), main['run_params']['max_run_iter'],
                                                       True, engine, False)
    n_cfg, n_init = cells0.shape[:2]
    out = []
    for t in traj:  # [T, n_cfg * N_init, ...] -> [n_cfg, T, N_init, ...]
        out.append(t.reshape((t.shape[0], n_cfg, n_init) + tuple(t.shape[2:])).transpose(0, 1))
    sd = lstat.split_stats(stats, update_fn.model_for(cells0.shape[3:]).C)
    sd['N'] = ncont
    sd = {k: v.squeeze() for k, v in sd.items()}
    return out[0], out[1], out[2], sd


def search_for_init(rng_key: int, config: Dict, fft: bool = True, device=None, engine: str = 'auto'):
    """helpers.py:319-393: draw ``run_params.nb_init_search`` initial states
    with ``algo.init_slug`` and return the first that lasts
    ``run_params.max_run_iter`` steps (else the longest before it), as
    ``({'N', 'all_cells', 'all_stats'}, index)``.  All candidates run in one
    engine launch; the chosen one is run again with its trajectory (the
    engine computes each world on its own, so it is the same run).  The
    states come from the engine's seeded stream (an integer ``rng_key``), not
    JAX's."""
    from . import initializations as linit
    wp, rp, run = config['world_params'], config['render_params'], config['run_params']
    C, R = wp['nb_channels'], wp['R']
    world_size = list(rp['world_size'])
    nb_init_search, max_run_iter = run['nb_init_search'], run['max_run_iter']
    kp = [dict(p) for p in config['kernels_params']]
    K, mapping = lkernels.get_kernels_and_mapping(kp, world_size, C, R, fft, device)
    dev = K.device
    gf, w = mapping.get_gf_params(dev), mapping.get_kernels_weight_per_channel(dev)
    update_fn = build_update_fn(K.shape, mapping, wp.get('get_state_fn_slug', 'v1'), wp.get('weighted_average', True),
                                fft)
    compute_stats_fn = lstat.build_compute_stats_fn(wp, rp)
    T = torch.tensor(float(wp['T']), dtype=torch.float32, device=dev)
    rng_key, noises = linit.register[config['algo']['init_slug']](rng_key, C * nb_init_search, world_size, R,
                                                                  kp[0]['gf_params'])
    noises = noises.reshape([nb_init_search, C] + world_size).cpu().numpy()
    cells0 = np.concatenate([create_init_cells(world_size, C, [noises[i]]) for i in range(nb_init_search)])
    cells0 = torch.from_numpy(cells0).to(dev)  # [nb_init_search, C, *world]
    sd, _ = lrunner.run_scan_mem_optimized(None, cells0[None], K[None], gf[None], w[None],
                                           T.reshape(1), max_run_iter, R, update_fn, compute_stats_fn, engine)
    n_done = [int(v) for v in sd['N'][0].tolist()]
    best_i, current_max, i = None, 0, 0
    for i, n in enumerate(n_done):  # the reference's sequential selection
        if current_max < n:
            current_max, best_i = n, i
        if n >= max_run_iter:
            break
    if best_i is None:
        return {}, i
    all_cells, _, _, all_stats = lrunner.run_scan(None, cells0[best_i:best_i + 1], K, gf, w, T, max_run_iter, R,
                                                  update_fn, compute_stats_fn, engine)
    return {'N': all_stats['N'], 'all_cells': all_cells, 'all_stats': all_stats}, i


def search_for_mutation(rng_key: int, config: Dict, nb_scale_for_stability: int = 1, use_init_cells: bool = True,
                        fft: bool = True, mutation_rate: float = 1e-5, device=None):
    """helpers.py:240-316: up to ``run_params.nb_mut_search`` mutations of the
    ``genotype`` genes (a normal step of ``mutation_rate`` each), each run at
    ``nb_scale_for_stability`` world scales; returns the mutation that lasts
    longest over the scales (stopping at one that lasts every step) and its
    index.  The normal draws come from numpy's PCG64 seeded with the integer
    ``rng_key``, not JAX's stream."""
    from .qd import get_param, set_param
    world_size = config['render_params']['world_size']
    run = config['run_params']
    nb_mut_search, max_run_iter = run['nb_mut_search'], run['max_run_iter']
    genes = config['genotype']
    noise = np.random.Generator(np.random.PCG64(int(rng_key))).standard_normal(nb_mut_search * len(genes),
                                                                                dtype=np.float32)
    best_run, current_max, i = {}, 0, 0
    for i in range(nb_mut_search):
        copied = copy.deepcopy(config)
        for g_i, gene in enumerate(genes):
            val = np.float32(get_param(copied, gene['key'])) + noise[i * len(genes) + g_i] * np.float32(mutation_rate)
            set_param(copied, gene['key'], float(val))
        total_iter_done, nb_iter_done = 0, 0
        all_cells = stats_dict = None
        for scale_power in range(nb_scale_for_stability):
            scaled = copy.deepcopy(copied)
            scaled['render_params']['world_size'] = [ws * 2**scale_power for ws in world_size]
            scaled['world_params']['scale'] = 2**scale_power
            all_cells, _, _, stats_dict = init_and_run(rng_key, scaled, use_init_cells=use_init_cells, with_jit=True,
                                                       fft=fft, device=device)
            all_cells = all_cells[:, 0]
            n = int(stats_dict['N'])
            nb_iter_done = max(nb_iter_done, n)
            total_iter_done += n
        if current_max < total_iter_done:
            current_max = total_iter_done
            best_run = {'N': nb_iter_done, 'all_cells': all_cells, 'all_stats': stats_dict, 'config': copied}
        if total_iter_done >= max_run_iter * nb_scale_for_stability:
            break
    return best_run, i
