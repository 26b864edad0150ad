"""Scan drivers on the GB300 engine: drop-in for leniax ``runner.py``.

``run_scan`` (runner.py:119-164) and ``run_scan_mem_optimized``
(runner.py:167-215) keep leniax's positional arguments and output layouts and
run the whole rollout -- Euler steps, per-step statistics, the stop
heuristics -- on the device in one engine call (``lgx_run``).  ``run``
(runner.py:16-116) is the eager driver with leniax's total-mass heuristics.
"""
import torch

from . import _lib
from .constant import EPSILON, START_CHECK_STOP
from .core import UpdateFn, _require_cuda, _stream_handle, check_spectra, workspace
from .statistics import ComputeStatsFn, split_stats
from . import statistics as lstat


def _rollout(update_fn: UpdateFn, compute_stats_fn: ComputeStatsFn, cells0, K, gf_params, w, T, max_run_iter,
             keep_intermediary: bool, engine: str, with_box: bool, with_centroid: bool = False,
             check_status: bool = False):
    """cells0 [Ns, Ni, C, *world], K [Ns, C, max_k, *world(-half)] (fft=True) or [Ns, C*max_k, 1,
    *kernel_dims] (fft=False), gf [Ns, K, 2], w [Ns, C, K], T [Ns]."""
    _require_cuda('cells0', cells0)
    m = update_fn.model_for(cells0.shape[3:])
    dev = cells0.device
    Ns, Ni = cells0.shape[0], cells0.shape[1]
    if tuple(cells0.shape[2:]) != (m.C, ) + m.world:
        raise ValueError(f'cells0 {tuple(cells0.shape)} does not match [Ns, Ni, {m.C}, *{m.world}]')
    steps = int(max_run_iter)
    if steps < 0:
        raise ValueError('max_run_iter must be >= 0')
    cells0 = cells0.contiguous()
    kh = update_fn.spectra(K if K.device == dev else K.to(dev), m.world)
    if kh.dim() < 1 or kh.shape[0] != Ns:
        raise ValueError('K must hold one spectrum per solution')
    check_spectra(kh, (Ns, ), m.C, m.max_k, m.world)
    gf = gf_params.to(dev, torch.float32).reshape(Ns, m.K, 2).contiguous()
    ww = w.to(dev, torch.float32).reshape(Ns, m.C, m.K).contiguous()
    Tt = torch.as_tensor(T, dtype=torch.float32, device=dev).reshape(-1)
    if Tt.numel() == 1 and Ns > 1:
        Tt = Tt.expand(Ns)
    if Tt.numel() != Ns:
        raise ValueError(f'T has {Tt.numel()} values for {Ns} solutions')
    Tt = Tt.contiguous()
    nw = Ns * Ni
    S = m.C + _lib.NSTAT_SCALAR
    final = torch.empty_like(cells0)
    stats = torch.empty((Ns, steps, Ni, S), dtype=torch.float32, device=dev)
    ncont = torch.empty((Ns, Ni), dtype=torch.float32, device=dev)
    nbox = torch.empty((Ns, Ni), dtype=torch.float32, device=dev) if with_box else None
    cen = torch.empty((Ns, steps, Ni, len(m.world)), dtype=torch.float32, device=dev) if with_centroid else None
    traj = None
    if keep_intermediary:
        traj = (torch.empty((steps, nw, m.C) + m.world, dtype=torch.float32, device=dev),
                torch.empty((steps, nw, m.C) + m.world, dtype=torch.float32, device=dev),
                torch.empty((steps, nw, m.K) + m.world, dtype=torch.float32, device=dev))
    lib = _lib.load()
    eng = _lib.ENGINES[engine]
    if lib.lgx_select_engine(m.plan.handle, Ns, Ni, eng) < 0:
        raise _lib.LgxError(_lib.LGX_ERR_UNSUPPORTED, f'no {engine} engine for this model')
    ws = workspace(lib.lgx_run_workspace_bytes(m.plan.handle, Ns, Ni, steps, eng), dev)
    job = _lib.Rollout()
    job.n_sols, job.n_init, job.steps = Ns, Ni, steps
    job.cells0 = cells0.data_ptr()
    job.k_half = kh.data_ptr()
    job.gf_params = gf.data_ptr()
    job.weights = ww.data_ptr()
    job.T = Tt.data_ptr()
    job.stats_R = compute_stats_fn.R
    job.stats_T = compute_stats_fn.T
    job.final_cells = final.data_ptr()
    job.stats = stats.data_ptr() if steps else None
    job.n_continue = ncont.data_ptr()
    job.n_box = nbox.data_ptr() if nbox is not None else None
    if traj is not None:
        job.traj_cells, job.traj_field, job.traj_potential = (t.data_ptr() for t in traj)
    job.engine = eng
    job.centroid = cen.data_ptr() if (cen is not None and steps) else None
    _lib.check(lib.lgx_run(m.plan.handle, job, ws.data_ptr(), ws.numel(), _stream_handle(dev)))
    if check_status:
        code = _lib.workspace_status(ws.data_ptr(), _stream_handle(dev))
        if code != 0:
            raise _lib.LgxError(_lib.LGX_ERR_TIMEOUT, f'device status {code}: a staged copy did not complete')
    return final, stats, ncont, nbox, traj, cen


def run_scan(rng_key, cells0, K, gf_params, kernels_weight_per_channel, T, max_run_iter: int, R: float,
             update_fn: UpdateFn, compute_stats_fn: ComputeStatsFn, engine: str = 'auto',
             with_box: bool = False, with_centroid: bool = False, check_status: bool = False):
    """runner.py:119-164.

    cells0 ``[N_init, C, *world]``; K ``[1, C, max_k, *world]`` complex64
    (or, for an fft=False update function, the direct path's real kernels
    ``[C*max_k, 1, *kernel_dims]``);
    returns ``(cells, field, potential, stats)`` with ``cells``/``field``
    ``[T, N_init, C, *world]``, ``potential`` ``[T, N_init, K, *world]`` and
    ``stats[k]`` ``[T, N_init]`` (``channel_mass`` ``[T, N_init, C]``) plus
    ``stats['N']`` ``[N_init]``.  Extensions: ``with_box`` adds ``'N_box'``
    (box stop set) and ``with_centroid`` adds ``'mass_centroid'`` ``[T,
    N_init, nb_dims]``, the per-step mass centroid as an absolute torus
    position.
    """
    _require_cuda('cells0', cells0)
    m = update_fn.model_for(cells0.shape[2:])
    Kb = K.reshape((1, ) + tuple(K.shape[1:])) if update_fn.fft else K.unsqueeze(0)
    final, stats, ncont, nbox, traj, cen = _rollout(update_fn, compute_stats_fn, cells0.unsqueeze(0), Kb,
                                                    gf_params.unsqueeze(0), kernels_weight_per_channel.unsqueeze(0), T,
                                                    max_run_iter, True, engine, with_box, with_centroid, check_status)
    sd = split_stats(stats[0], m.C)
    sd['N'] = ncont[0]
    if nbox is not None:
        sd['N_box'] = nbox[0]
    if cen is not None:
        sd['mass_centroid'] = cen[0]
    cells, field, potential = traj
    return cells, field, potential, sd


def run_scan_mem_optimized(rng_key, cells0, K, gf_params, kernels_weight_per_channel, T, max_run_iter: int, R: float,
                           update_fn: UpdateFn, compute_stats_fn: ComputeStatsFn, engine: str = 'auto',
                           with_box: bool = False, with_centroid: bool = False, check_status: bool = False):
    """runner.py:167-215: all solutions x inits in one engine launch.

    cells0 ``[N_sols, N_init, C, *world]``; K ``[N_sols, 1, C, max_k, *world]``
    (fft=False: ``[N_sols, C*max_k, 1, *kernel_dims]``);
    gf_params ``[N_sols, K, 2]``; weights ``[N_sols, C, K]``; T ``[N_sols]``.
    Returns ``(stats, final_cells)``: ``stats[k]`` ``[N_sols, T, N_init]``
    (``channel_mass`` ``[N_sols, T, N_init, C]``), ``stats['N']``
    ``[N_sols, N_init]``; ``final_cells`` ``[N_sols, N_init, C, *world]``.
    ``check_status=True`` synchronises after the launch and raises if the
    engine's device status word reports a staged copy that never landed.
    """
    _require_cuda('cells0', cells0)
    m = update_fn.model_for(cells0.shape[3:])
    Ns = cells0.shape[0]
    Kr = K.reshape((Ns, ) + tuple(K.shape[2:])) if update_fn.fft and K.dim() == 3 + len(m.world) + 1 else K
    final, stats, ncont, nbox, _, cen = _rollout(update_fn, compute_stats_fn, cells0, Kr, gf_params,
                                                 kernels_weight_per_channel, T, max_run_iter, False, engine, with_box,
                                                 with_centroid, check_status)
    sd = split_stats(stats, m.C)
    sd['N'] = ncont
    if nbox is not None:
        sd['N_box'] = nbox
    if cen is not None:
        sd['mass_centroid'] = cen
    return sd, final


def run_scan_mem_optimized_pmap(rng_key, cells0, K, gf_params, kernels_weight_per_channel, T, max_run_iter: int,
                                R: float, update_fn: UpdateFn, compute_stats_fn: ComputeStatsFn, engine: str = 'auto'):
    """runner.py:218-268: ``run_scan_mem_optimized`` over a leading device
    axis (``cells0`` ``[N_device, N_sols, N_init, C, *world]``, the other
    arguments ``[N_device, N_sols, ...]``).  Slice d runs on CUDA device
    ``d mod device_count`` (launches are asynchronous, so the devices work
    together); results come back stacked on the first slice's device.  The
    one-process-per-GPU form of the same sharding is ``leniax_gb300.sharding``.
    """
    n_dev = int(cells0.shape[0])
    count = max(1, torch.cuda.device_count())
    home = cells0.device
    parts = []
    for d in range(n_dev):
        dev = torch.device('cuda', d % count) if count > 1 else home
        with torch.cuda.device(dev):
            Td = torch.as_tensor(T)[d] if torch.as_tensor(T).dim() else torch.as_tensor(T)
            parts.append(run_scan_mem_optimized(rng_key, cells0[d].to(dev), K[d].to(dev), gf_params[d].to(dev),
                                                kernels_weight_per_channel[d].to(dev), Td, max_run_iter, R,
                                                update_fn, compute_stats_fn, engine))
    stats = {k: torch.stack([p[0][k].to(home) for p in parts]) for k in parts[0][0]}
    return stats, torch.stack([p[1].to(home) for p in parts])


def run(rng_key, cells, K, gf_params, kernels_weight_per_channel, T, max_run_iter: int, R: float,
        update_fn: UpdateFn, compute_stats_fn: ComputeStatsFn, stat_trunc: bool = False, engine: str = 'auto'):
    """runner.py:16-116: single configuration with the eager total-mass
    heuristics.  The rollout runs on the device in one call; the reference's
    early ``break`` (runner.py:103-104) truncates the returned trajectory."""
    assert max_run_iter > 0, f'max_run_iter must be positive, value given: {max_run_iter}'
    assert cells.shape[0] == 1
    all_cells, all_fields, all_pots, stats = run_scan(rng_key, cells, K, gf_params, kernels_weight_per_channel, T,
                                                      max_run_iter, R, update_fn, compute_stats_fn, engine)
    mass = stats['mass']
    init_mass = cells.sum()
    dev = mass.device
    prev_mass = init_mass
    prev_sign = torch.zeros(1, dtype=torch.int32, device=dev)
    counters = lstat.init_counters(1, dev)
    should = torch.ones(1, dtype=torch.int32, device=dev)
    last = max_run_iter - 1
    for it in range(max_run_iter):
        mt = mass[it]
        cond = lstat.min_mass_heuristic(EPSILON, mt) & lstat.max_mass_heuristic(init_mass, mt)
        sign = torch.sign(mt - prev_mass)
        c1, counters['nb_monotone_step'] = lstat.monotonic_heuristic(sign, prev_sign, counters['nb_monotone_step'])
        c2, counters['nb_max_volume_step'] = lstat.mass_volume_heuristic(stats['mass_volume'][it],
                                                                         counters['nb_max_volume_step'])
        should = should * (cond & c1 & c2)
        prev_mass = mt
        prev_sign = sign
        if stat_trunc and it >= START_CHECK_STOP and int(should[0]) == 0:
            last = it
            break
    n = last + 1
    out_stats = {k: v[:n] for k, v in stats.items() if k not in ('N', 'N_box')}
    out_stats['N'] = torch.tensor(last, device=dev)
    return all_cells[:n], all_fields[:n], all_pots[:n], out_stats


# ---------------------------------------------------------------- differentiable pipelines
def normalize_fn(g: torch.Tensor) -> torch.Tensor:
    """runner.py:447-448: ``g`` divided by its 2-norm (over all entries) + 1e-8."""
    return g / (torch.linalg.vector_norm(g) + 1e-8)


def _flatten(tree):
    """Leaves (tensors) of nested dicts / lists / tuples, and a rebuild function."""
    if isinstance(tree, dict):
        keys = sorted(tree)
        parts = [_flatten(tree[k]) for k in keys]
        leaves = [leaf for p in parts for leaf in p[0]]
        sizes = [len(p[0]) for p in parts]

        def rebuild(vals):
            out, i = {}, 0
            for k, (_, rb), n in zip(keys, parts, sizes):
                out[k] = rb(vals[i:i + n])
                i += n
            return out

        return leaves, rebuild
    if isinstance(tree, (list, tuple)):
        parts = [_flatten(v) for v in tree]
        leaves = [leaf for p in parts for leaf in p[0]]
        sizes = [len(p[0]) for p in parts]

        def rebuild_seq(vals):
            out, i = [], 0
            for (_, rb), n in zip(parts, sizes):
                out.append(rb(vals[i:i + n]))
                i += n
            return type(tree)(out)

        return leaves, rebuild_seq
    return [tree], lambda vals: vals[0]


def make_pipeline_fn(max_run_iter: int, dt: float, apply_fn, loss_fn, keep_intermediary_data: bool = False,
                     keep_all_timesteps: bool = True):
    """runner.py:363-423: ``fn(rng_key, params, variables, state0, targets)
    -> (loss, rest)`` runs ``max_run_iter`` steps of ``apply_fn({'params':
    params, **variables}, rng_key, state, dt=dt)`` from ``state0`` and
    returns ``loss_fn(rng_key, preds, targets)`` split as ``(loss, rest)``.
    ``preds['cells']`` is every pre-update state ``[max_run_iter, *state0]``
    (``keep_all_timesteps``) or the last state; with
    :class:`leniax_gb300.grad.LeniaApply` the last-state form runs as one
    engine rollout.  The engine's adjoint differentiates cell states, so
    ``keep_intermediary_data`` (fields and potentials in ``preds``) is
    refused."""
    if keep_intermediary_data:
        raise NotImplementedError('the engine adjoint differentiates cell states only: use '
                                  'keep_intermediary_data=False')
    steps = int(max_run_iter)

    def fn(rng_key, params, variables, state0, targets):
        vs = {'params': params, **variables}
        if keep_all_timesteps:
            states, cur = [], state0
            for _ in range(steps):
                states.append(cur)
                cur = apply_fn(vs, rng_key, cur, dt=dt)[0]
            cells = torch.stack(states) if states else state0.new_empty((0, ) + tuple(state0.shape))
        elif hasattr(apply_fn, 'rollout'):
            cells = apply_fn.rollout(vs, state0, steps, dt)
        else:
            cells = state0
            for _ in range(steps):
                cells = apply_fn(vs, rng_key, cells, dt=dt)[0]
        loss, *rest = loss_fn(rng_key, {'cells': cells}, targets)
        return loss, rest

    return fn


def make_gradient_fn(pipeline_fn, normalize: bool = True):
    """runner.py:426-444: ``fn(rng_key, params, variables, state0, targets)
    -> ((loss, aux), grads)``, ``grads`` shaped like ``params`` (nested
    dicts / sequences of tensors), each divided by its norm
    (:func:`normalize_fn`) when ``normalize``."""

    def fn(rng_key, params, variables, state0, targets):
        leaves, rebuild = _flatten(params)
        leaves = [t.detach().requires_grad_(True) for t in leaves]
        with torch.enable_grad():
            loss, aux = pipeline_fn(rng_key, rebuild(leaves), variables, state0, targets)
            grads = torch.autograd.grad(loss, leaves, allow_unused=True)
        grads = [torch.zeros_like(p) if g is None else g for p, g in zip(leaves, grads)]
        if normalize:
            grads = [normalize_fn(g) for g in grads]
        return (loss.detach(), aux), rebuild(grads)

    return fn
