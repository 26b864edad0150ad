"""Quality-diversity evaluation glue: the caller that feeds batches of
candidate individuals into the batched engine.

Mirror of leniax ``qd.py`` (``build_eval_lenia_config_mem_optimized_fn``
33-77, ``get_dynamic_args`` 80-147, ``update_individuals`` 150-188) and of
``lenia.py`` (``LeniaIndividual`` 8-72, ``update_config`` /
``get_update_config`` / ``linear_scale`` / ``log_scale`` 75-160) with the
config path helpers of ``utils.py`` (``get_param`` / ``set_param``
153-210).  The search loop itself (pyribs optimizers, archives, plotting) is
the caller's.

GB300 layout: for a batch of individuals the kernels of each kernel slot are
built together on the GPU (``kernels.ring_kernels``), the initial states of
all individuals by one ``lgx_init_cells`` launch, and the fitness and
behaviour reductions of ``update_individuals`` run on the device with one
copy to the host at the end.
"""
import copy
from typing import Callable, Dict, List, Sequence, Tuple

import numpy as np
import torch

from . import helpers, initializations, kernels, runner, statistics
from .utils import get_param, set_param


# ------------------------------------------------------------------ config paths (utils.py:153-210)
# ------------------------------------------------------------------ individuals (lenia.py)
def linear_scale(raw_value: float, domain: Sequence[float]) -> float:
    """lenia.py:124-136"""
    return domain[0] + (domain[1] - domain[0]) * raw_value


def log_scale(raw_value: float, domain: Sequence[float]) -> float:
    """lenia.py:139-151"""
    return domain[0] * (domain[1] / domain[0])**raw_value


def get_update_config(genotype: List[Dict], raw_values: List[float]) -> Dict:
    """lenia.py:96-121: raw values in [0, 1] -> typed values in each gene's domain."""
    to_update: Dict = {}
    for gene, raw_val in zip(genotype, raw_values):
        domain, val_type = gene['domain'], gene['type']
        if val_type == 'float':
            val = float(linear_scale(raw_val, domain))
        elif val_type == 'int':
            val = int(linear_scale(raw_val, (domain[0], domain[1] + 1)) - 0.5)
        elif val_type == 'choice':
            val = domain[int(linear_scale(raw_val, (0, len(domain))) - 0.5)]
        else:
            raise ValueError(f'type {val_type} unknown')
        set_param(to_update, gene['key'], val)
    return to_update


def update_config(config: Dict, to_update: Dict) -> Dict:
    """lenia.py:75-93"""
    new_config = copy.deepcopy(config)
    if 'kernels_params' in to_update:
        for i, kernel in enumerate(to_update['kernels_params']):
            new_config['kernels_params'][i].update(kernel)
    if 'world_params' in to_update:
        new_config['world_params'].update(to_update['world_params'])
    return new_config


class LeniaIndividual:
    """lenia.py:8-72.  ``rng_key`` is an integer seed (see
    :mod:`leniax_gb300.initializations`)."""

    def __init__(self, config: Dict, rng_key: int, params: List = ()):
        self.qd_config = copy.deepcopy(config)
        self.rng_key = int(rng_key)
        self.params = list(params)
        self.fitness = None
        self.features = None
        if 'genotype' in self.qd_config:
            for gene in self.get_genotype():
                get_param(self.qd_config, gene['key'])  # genes only update existing values

    def set_init_props(self, rng_key: int, best_init_idxs: List[int]):
        self.qd_config['algo']['init_rng_key'] = int(rng_key)
        self.qd_config['algo']['best_init_idxs'] = best_init_idxs

    def set_cells(self, cells: str):
        self.qd_config['run_params']['cells'] = cells

    def set_init_cells(self, init_cells: str):
        self.qd_config['run_params']['init_cells'] = init_cells

    def get_config(self) -> Dict:
        if 'genotype' not in self.qd_config:
            return self.qd_config
        genotype = self.get_genotype()
        raw_values = [round(v, 8) for v in self.params]  # lenia.py:61
        assert len(raw_values) == len(genotype)
        return update_config(self.qd_config, get_update_config(genotype, raw_values))

    def get_genotype(self):
        return self.qd_config['genotype']


# ------------------------------------------------------------------ dynamic arguments (qd.py:80-147)
def _topology(kparams):
    return [(p['c_in'], p['c_out']) for p in sorted(kparams, key=lambda d: d['c_in'])]


def _hermitian_full(kh: torch.Tensor, W: int) -> torch.Tensor:
    """Full spectrum [..., H, W] of a real 2D signal from its half [..., H, W//2+1]."""
    H = kh.shape[-2]
    rest = kh[..., 1:W - W // 2].flip(-1)  # columns W//2-1 .. 1
    rows = (-torch.arange(H, device=kh.device)) % H
    return torch.cat([kh, rest[..., rows, :].conj()], dim=-1)


def get_dynamic_args(qd_config: Dict, leniax_sols: List[LeniaIndividual], fft: bool = True,
                     full_spectrum: bool = True, device=None) -> Tuple[int, Tuple[torch.Tensor, ...]]:
    """qd.py:80-147: the batched arguments of ``run_scan_mem_optimized`` for a
    list of individuals: ``cells0 [N_sols, N_init, C, *world]``,
    ``K [N_sols, 1, C, max_k, *world]`` (``fft``; the Hermitian half
    ``[..., W//2+1]`` with ``full_spectrum=False``; real cropped kernels
    ``[N_sols, C*max_k, 1, kh, kw]`` without ``fft``), ``gf_params
    [N_sols, K, 2]``, ``kernels_weight_per_channel [N_sols, C, K]``,
    ``T [N_sols]``.  Returns ``(rng_key, args)``."""
    if device is None:
        device = torch.device('cuda', torch.cuda.current_device())
    world_params, render_params = qd_config['world_params'], qd_config['render_params']
    C, R = world_params['nb_channels'], world_params['R']
    world_size = list(render_params['world_size'])
    nb_init_search = qd_config['run_params']['nb_init_search']
    init_slug = qd_config['algo']['init_slug']
    configs = [ind.get_config() for ind in leniax_sols]
    n = len(configs)
    kps = [sorted([dict(p) for p in c['kernels_params']], key=lambda d: d['c_in']) for c in configs]
    topo = _topology(kps[0])
    same_topology = all(_topology(k) == topo for k in kps)
    ring_only = all(p.get('k_slug', 'circle_2d') == 'circle_2d' for k in kps for p in k)
    Ks = []
    if fft and same_topology and ring_only:
        # one device build per kernel slot for every individual
        nk = len(topo)
        per_slot = []
        for k in range(nk):
            slugs = {kp[k]['kf_slug'] for kp in kps}
            kh = torch.empty((n, ) + tuple(world_size[:-1]) + (world_size[-1] // 2 + 1, ), dtype=torch.complex64,
                             device=device)
            for slug in slugs:
                idx = [i for i, kp in enumerate(kps) if kp[k]['kf_slug'] == slug]
                _, part = kernels.ring_kernels(world_size, [R] * len(idx), [kps[i][k]['k_params'][0] for i in idx],
                                               [list(kps[i][k]['k_params'][1]) for i in idx], slug,
                                               [list(kps[i][k]['kf_params']) for i in idx], spectrum=True,
                                               device=device)
                kh[torch.tensor(idx, device=device)] = part
            per_slot.append(kh)
        # assemble [n, C, max_k, *half] by the (c_in, slot) table of leniax's mapping (kernels.py:122-143)
        cin = [kp['c_in'] for kp in kps[0]]
        lists = [[k for k in range(nk) if cin[k] == c] for c in range(C)]
        max_k = max(map(len, lists))
        half = torch.zeros((n, C, max_k) + tuple(per_slot[0].shape[1:]), dtype=torch.complex64, device=device)
        for c, lst in enumerate(lists):
            for j, k in enumerate(lst):
                half[:, c, j] = per_slot[k]
        K = _hermitian_full(half, world_size[-1]) if full_spectrum else half
        K = K[:, None]
        gf = torch.tensor([[p['gf_params'] for p in kp] for kp in kps], dtype=torch.float32, device=device)
        w = torch.zeros((n, C, nk), dtype=torch.float32, device=device)
        for i, kp in enumerate(kps):
            for k, p in enumerate(kp):
                w[i, p['c_out'], k] = float(p['h'])
    else:
        # host construction per individual (leniax's own path), also for conv kernels
        gfs, ws = [], []
        for c in configs:
            Kc, mp = kernels.get_kernels_and_mapping([dict(p) for p in c['kernels_params']], world_size, C, R, fft,
                                                     device)
            if fft and not full_spectrum:
                Kc = Kc[..., :world_size[-1] // 2 + 1]
            Ks.append(Kc)
            gfs.append(mp.get_gf_params(device))
            ws.append(mp.get_kernels_weight_per_channel(device))
        K, gf, w = torch.stack(Ks), torch.stack(gfs), torch.stack(ws)
    # initial states: nb_channels * nb_init_search per individual, one launch for all
    seeds = [initializations.next_key(ind.rng_key) for ind in leniax_sols]
    gf_m = [float(kp[0]['gf_params'][0]) for kp in kps]
    nb_init = C * nb_init_search
    cells = initializations.generate(init_slug, seeds, nb_init, world_size, R, gf_m, True, device)
    cells0 = cells.reshape([n, nb_init_search, C] + world_size)
    T = torch.tensor([float(c['world_params']['T']) for c in configs], dtype=torch.float32, device=device)
    rng_key = initializations.next_key(seeds[-1]) if seeds else 0
    return rng_key, (cells0, K, gf, w, T)


# ------------------------------------------------------------------ fitness and behaviours (qd.py:150-188)
def update_individuals(inds: List[LeniaIndividual], stats: Dict[str, torch.Tensor],
                       fitness_coef: float = 1.) -> List[LeniaIndividual]:
    """qd.py:150-188: fitness = fitness_coef * max over inits of N, best init
    indices, and for a configuration with a ``phenotype`` the mean of every
    statistic over the 128 steps before ``max(int(fitness), 128)`` of the
    first best init.  Reductions run where ``stats`` live (GPU or CPU); one
    copy to the host at the end."""
    Ns = stats['N']
    Ns = Ns if isinstance(Ns, torch.Tensor) else torch.as_tensor(np.asarray(Ns))
    max_N, best = Ns.max(dim=1)  # first maximal index, as jnp.argmax
    fitness = fitness_coef * max_N.to(torch.float64)
    ties = (Ns == max_N[:, None])
    want_pheno = any('phenotype' in ind.qd_config for ind in inds)
    behaviours = {}
    if want_pheno:
        ns = torch.clamp(fitness.to(torch.int64), min=128)  # max(int(fitness), 128)
        for k, v in stats.items():
            if k == 'N':
                continue
            v = v if isinstance(v, torch.Tensor) else torch.as_tensor(np.asarray(v))
            if v.dim() != 3:
                continue  # channel_mass [Ns, T, Ni, C] is not a leniax behaviour scalar
            sel = v.gather(2, best.view(-1, 1, 1).expand(-1, v.shape[1], 1))[..., 0].to(torch.float64)  # [Ns, T]
            T = sel.shape[1]
            csum = torch.cat([torch.zeros_like(sel[:, :1]), sel.cumsum(1)], 1)
            end = torch.clamp(ns, max=T)
            start = torch.clamp(ns - 128, max=T)
            cnt = (end - start).to(torch.float64)
            tot = csum.gather(1, end[:, None])[:, 0] - csum.gather(1, start[:, None])[:, 0]
            behaviours[k] = tot / cnt  # empty window -> nan, as the mean of an empty slice
    # one host copy of everything the individuals need
    fitness_h = fitness.cpu().tolist()
    ties_h = ties.cpu().numpy()
    beh_h = {k: v.cpu().tolist() for k, v in behaviours.items()}
    for i, ind in enumerate(inds):
        ind.set_init_props(ind.rng_key, [int(x) for x in np.nonzero(ties_h[i])[0]])
        ind.fitness = fitness_h[i]
        if 'phenotype' in ind.qd_config:
            tmp_config = ind.get_config()
            tmp_config['behaviours'] = {k: float(v[i]) for k, v in beh_h.items()}
            ind.features = [get_param(tmp_config, key) for key in ind.qd_config['phenotype']]
    return inds


# ------------------------------------------------------------------ evaluation function (qd.py:33-77)
def build_eval_lenia_config_mem_optimized_fn(qd_config: Dict, fitness_coef: float = 1., fft: bool = True,
                                             device=None) -> Callable:
    """qd.py:33-77: ``eval(individuals) -> individuals`` with fitness and
    features set, one batched engine rollout per call."""
    if not fft:
        raise ValueError('the engine evaluates FFT potentials only')
    if device is None:
        device = torch.device('cuda', torch.cuda.current_device())
    max_run_iter = qd_config['run_params']['max_run_iter']
    world_params, render_params = qd_config['world_params'], qd_config['render_params']
    R = world_params['R']
    slug = world_params.get('get_state_fn_slug', 'v1')
    avg = world_params.get('weighted_average', True)
    K, mapping = kernels.get_kernels_and_mapping([dict(p) for p in qd_config['kernels_params']],
                                                 render_params['world_size'], world_params['nb_channels'], R, True,
                                                 device)
    update_fn = helpers.build_update_fn(K.shape, mapping, slug, avg)
    compute_stats_fn = statistics.build_compute_stats_fn(world_params, render_params)

    def eval_lenia_config_mem_optimized(leniax_sols: List[LeniaIndividual]) -> List[LeniaIndividual]:
        cfg = leniax_sols[0].qd_config
        rng_key, args = get_dynamic_args(cfg, leniax_sols, True, full_spectrum=False, device=device)
        stats, _ = runner.run_scan_mem_optimized(rng_key, *args, max_run_iter, R, update_fn, compute_stats_fn)
        return update_individuals(leniax_sols, stats, fitness_coef)

    return eval_lenia_config_mem_optimized
