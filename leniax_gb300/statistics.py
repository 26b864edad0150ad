"""Statistics descriptors and stop heuristics (leniax ``statistics.py``).

On the hot path the statistics (statistics.py:36-126) and the stop count
``N`` (check_heuristics, statistics.py:134-205) are computed on the device by
the engine inside ``runner.run_scan*``.  This module provides the
``compute_stats_fn`` descriptor those runners take, and torch versions of the
heuristics for callers that post-process a stats dict themselves.
"""
from typing import Dict, List, Sequence, Tuple

import torch

from .constant import EPSILON

STAT_KEYS = ('channel_mass', 'mass', 'mass_volume', 'mass_density', 'growth', 'growth_volume', 'growth_density',
             'mass_speed', 'mass_angle_speed', 'mass_growth_dist', 'inertia', 'potential_volume')
MONOTONIC_STOP_STEP = 128
MASS_VOLUME_THRESHOLD = 10.
MASS_VOLUME_STOP_STEP = 128


class ComputeStatsFn:
    """What ``build_compute_stats_fn`` closes over (statistics.py:22-33): the
    world size, the static kernel radius ``R`` and the static ``T``."""

    def __init__(self, world_size: Sequence[int], R: float, T: float):
        self.world_size = tuple(int(s) for s in world_size)
        self.R = float(R)
        self.T = float(T)

    def __repr__(self):
        return f'ComputeStatsFn(world_size={self.world_size}, R={self.R}, T={self.T})'


def build_compute_stats_fn(world_params: Dict, render_params: Dict) -> ComputeStatsFn:
    """statistics.py:11-128"""
    return ComputeStatsFn(render_params['world_size'], world_params['R'], world_params['T'])


def split_stats(packed: torch.Tensor, C: int) -> Dict[str, torch.Tensor]:
    """Engine stats ``[..., C + 11]`` -> leniax's dict of arrays."""
    out = {'channel_mass': packed[..., :C].contiguous()}
    for i, k in enumerate(STAT_KEYS[1:]):
        out[k] = packed[..., C + i].contiguous()
    return out


def min_channel_mass_heuristic(epsilon, channel_mass):
    """statistics.py:224-236"""
    return (channel_mass >= epsilon).all(dim=1)


def max_channel_mass_heuristic(init_channel_mass, channel_mass):
    """statistics.py:239-251"""
    return (channel_mass <= 3 * init_channel_mass).all(dim=1)


def min_mass_heuristic(epsilon, mass):
    """statistics.py:254-266"""
    return mass >= epsilon


def max_mass_heuristic(init_mass, mass):
    """statistics.py:269-281"""
    return mass <= 3 * init_mass


def monotonic_heuristic(sign, previous_sign, monotone_counter) -> Tuple[torch.Tensor, torch.Tensor]:
    """statistics.py:287-306"""
    sign_cond = (sign == previous_sign)
    monotone_counter = monotone_counter * sign_cond + 1
    return monotone_counter <= MONOTONIC_STOP_STEP, monotone_counter


def mass_volume_heuristic(mass_volume, mass_volume_counter) -> Tuple[torch.Tensor, torch.Tensor]:
    """statistics.py:317-333"""
    volume_cond = mass_volume > MASS_VOLUME_THRESHOLD
    mass_volume_counter = mass_volume_counter * volume_cond + 1
    return mass_volume_counter <= MASS_VOLUME_STOP_STEP, mass_volume_counter


def init_counters(N: int, device=None) -> Dict[str, torch.Tensor]:
    """statistics.py:208-221"""
    z = lambda: torch.zeros(N, dtype=torch.int32, device=device)  # noqa: E731
    return {'nb_monotone_step': z(), 'nb_slow_mass_step': z(), 'nb_max_volume_step': z()}


def check_heuristics(stats: Dict[str, torch.Tensor]) -> torch.Tensor:
    """statistics.py:134-205 on a stats dict with ``[T, N]`` values."""
    mass = stats['mass']
    cm = stats['channel_mass']
    T, N = mass.shape
    dev = mass.device
    should = torch.ones(N, dtype=mass.dtype, device=dev)
    init_cm = cm[0]
    prev_mass = mass[0]
    prev_sign = torch.zeros(N, dtype=mass.dtype, device=dev)
    counters = init_counters(N, dev)
    out = torch.empty((T, N), dtype=mass.dtype, device=dev)
    for t in range(T):
        cond = min_channel_mass_heuristic(EPSILON, cm[t]) & max_channel_mass_heuristic(init_cm, cm[t])
        sign = torch.sign(mass[t] - prev_mass)
        c1, counters['nb_monotone_step'] = monotonic_heuristic(sign, prev_sign, counters['nb_monotone_step'])
        c2, counters['nb_max_volume_step'] = mass_volume_heuristic(stats['mass_volume'][t],
                                                                   counters['nb_max_volume_step'])
        should = should * (cond & c1 & c2)
        out[t] = should
        prev_mass = mass[t]
        prev_sign = sign
    return out


def stats_list_to_dict(all_stats: List[Dict]) -> Dict[str, torch.Tensor]:
    """statistics.py:339-360"""
    if not all_stats:
        return {}
    return {k: torch.stack([torch.as_tensor(s[k]) for s in all_stats]) for k in all_stats[0]}
