"""Lenia step on the GB300 engine: drop-in for leniax ``core.py``.

``UpdateFn`` is what leniax's ``helpers.build_update_fn`` returns
(``functools.partial(core.update, get_potential_fn=..., get_field_fn=...,
get_state_fn=...)``, helpers.py:401-427): a callable
``update_fn(rng_key, state, K, gf_params, kernels_weight_per_channel, dt)``
returning ``(state, field, potential)`` (core.py:13-49).  Tensors are CUDA
torch tensors; every call runs the engine's CUDA kernels through the C ABI.
"""
from typing import Optional, Sequence

import torch

from . import _lib
from .kernels import KernelMapping

# get_state plugin registry, core.py:322-326 (slug -> engine id)
register = dict(_lib.STATE_IDS)


def _stream_handle(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _require_cuda(name, t: torch.Tensor, dtype=torch.float32):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f'{name} must be a torch tensor')
    if not t.is_cuda:
        raise ValueError(f'{name} must be a CUDA tensor: the engine has no CPU path')
    if t.dtype != dtype:
        raise TypeError(f'{name} must be {dtype}, got {t.dtype}')


def half_spectrum(K: torch.Tensor, world: Sequence[int]) -> torch.Tensor:
    """leniax's full complex spectrum ``[..., *world]`` (or an already sliced
    half ``[..., W//2+1]``) -> contiguous float32 view of the Hermitian half."""
    W = int(world[-1])
    if K.dtype != torch.complex64:
        raise TypeError(f'K must be complex64, got {K.dtype}')
    if K.shape[-1] == W:
        K = K[..., :W // 2 + 1]
    elif K.shape[-1] != W // 2 + 1:
        raise ValueError(f'K last axis {K.shape[-1]} matches neither W={W} nor W//2+1')
    return torch.view_as_real(K.contiguous())


def workspace(nbytes: int, device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


class Model:
    """Static model of a Lenia configuration: world axes, channel/kernel graph,
    growth functions, state update and weighting (what leniax closes over)."""

    def __init__(self, world: Sequence[int], nb_channels: int, mapping: KernelMapping, get_state_fn_slug='v1',
                 average_weight=True):
        cin, slot, gfs, max_k = mapping.kernel_table()
        for g in gfs:
            if g not in _lib.GF_IDS:
                raise ValueError(f'unknown growth function slug {g!r}')
        if get_state_fn_slug not in register:
            raise ValueError(f'unknown get_state_fn slug {get_state_fn_slug!r}')
        self.world = tuple(int(w) for w in world)
        self.C = nb_channels
        self.K = len(cin)
        self.max_k = max_k
        self.cin, self.slot = list(cin), list(slot)  # spectrum position [c_in, slot] of each true kernel
        self.gf_slugs = gfs
        self.state_slug = get_state_fn_slug
        self.average = bool(average_weight)
        self.plan = _lib.Plan(len(self.world), self.world, nb_channels, cin, slot, [_lib.GF_IDS[g] for g in gfs], max_k,
                              register[get_state_fn_slug], average_weight)


class UpdateFn:
    """``update_fn(rng_key, state, K, gf_params, kernels_weight_per_channel, dt)``.

    ``state`` ``[N, C, *world]`` float32; ``K`` ``[1, C, max_k, *world]``
    complex64 (or its half ``[..., W//2+1]``); ``gf_params`` ``[K, 2]``;
    ``kernels_weight_per_channel`` ``[C, K]``; ``dt`` a scalar (python or
    0-d/1-element tensor) or ``[N]`` per-world rates.  ``rng_key`` is unused by
    every get_state function of the reference (core.py:245-319).
    """

    def __init__(self, kernel_shape: Sequence[int], mapping: KernelMapping, get_state_fn_slug='v1',
                 average_weight=True, fft=True):
        if not fft:
            raise NotImplementedError('the engine computes the potential by FFT only (core.get_potential_fft)')
        kernel_shape = tuple(int(s) for s in kernel_shape)
        self.kernel_shape = kernel_shape
        self.model = Model(kernel_shape[3:], kernel_shape[1], mapping, get_state_fn_slug, average_weight)

    def __call__(self, rng_key, state, K, gf_params, kernels_weight_per_channel, dt):
        m = self.model
        _require_cuda('state', state)
        if tuple(state.shape[2:]) != m.world or state.shape[1] != m.C:
            raise ValueError(f'state shape {tuple(state.shape)} does not match [N, {m.C}, *{m.world}]')
        dev = state.device
        N = state.shape[0]
        state = state.contiguous()
        kh = half_spectrum(K.to(dev), m.world)
        if kh.shape[0] != 1:
            raise ValueError('update shares one spectrum across the batch: K must be [1, C, max_k, ...]')
        gf = gf_params.to(dev, torch.float32).contiguous()
        w = kernels_weight_per_channel.to(dev, torch.float32).contiguous()
        if gf.shape != (m.K, 2) or w.shape != (m.C, m.K):
            raise ValueError(f'gf_params {tuple(gf.shape)} / weights {tuple(w.shape)} do not match K={m.K}, C={m.C}')
        dtt = torch.as_tensor(dt, dtype=torch.float32, device=dev).reshape(-1).contiguous()
        per_world = dtt.numel() > 1
        if per_world and dtt.numel() != N:
            raise ValueError(f'dt has {dtt.numel()} values for {N} worlds')
        out = torch.empty_like(state)
        field = torch.empty_like(state)
        potential = torch.empty((N, m.K) + m.world, dtype=torch.float32, device=dev)
        lib = _lib.load()
        ws_bytes = lib.lgx_update_workspace_bytes(m.plan.handle, N)
        ws = workspace(ws_bytes, dev)
        _lib.check(
            lib.lgx_update(m.plan.handle, N, state.data_ptr(), kh.data_ptr(), gf.data_ptr(), w.data_ptr(),
                           dtt.data_ptr(), 1 if per_world else 0, out.data_ptr(), field.data_ptr(),
                           potential.data_ptr(), ws.data_ptr(), ws.numel(), _stream_handle(dev)))
        return out, field, potential


def update(rng_key, state, K, gf_params, kernels_weight_per_channel, dt, update_fn: UpdateFn):
    """core.py:13-49 with the static functions bundled in ``update_fn``."""
    return update_fn(rng_key, state, K, gf_params, kernels_weight_per_channel, dt)
