"""Lenia step on the GB300 engine: drop-in for leniax ``core.py``.

``UpdateFn`` is what leniax's ``helpers.build_update_fn`` returns
(``functools.partial(core.update, get_potential_fn=..., get_field_fn=...,
get_state_fn=...)``, helpers.py:401-427): a callable
``update_fn(rng_key, state, K, gf_params, kernels_weight_per_channel, dt)``
returning ``(state, field, potential)`` (core.py:13-49).  Tensors are CUDA
torch tensors; every call runs the engine's CUDA kernels through the C ABI.
"""
import ctypes
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


def check_spectra(kh: torch.Tensor, lead: Sequence[int], nb_channels: int, max_k: int, world: Sequence[int]):
    """Raise unless ``kh`` (the float32 view of half spectra) is ``[*lead,
    C, max_k, *world[:-1], W//2+1, 2]``: the engine reads exactly that many
    values through a bare pointer."""
    world = tuple(int(w) for w in world)
    want = tuple(int(v) for v in lead) + (nb_channels, max_k) + world[:-1] + (world[-1] // 2 + 1, 2)
    if tuple(kh.shape) != want:
        got = ', '.join(map(str, tuple(kh.shape)[:-1]))
        raise ValueError(f'K spectra [{got}] (half spectrum) do not match [{", ".join(map(str, want[:-1]))}]: '
                         f'{nb_channels} channels, max_k = {max_k}, world {world}')


def direct_spectrum(K: torch.Tensor, world: Sequence[int], nb_channels: int, max_k: int,
                    pads: Optional[Sequence[int]] = None) -> torch.Tensor:
    """The real kernels of leniax's direct-convolution path, ``[...,
    C*max_k, 1, *kernel_dims]``, as the engine's half spectra ``[..., C,
    max_k, *world[:-1], W//2+1]`` complex64.

    leniax applies them with ``core.get_potential`` (core.py:105-146): the
    state wrap-padded by ``k//2`` before each axis (helpers.py:465-481), then
    a VALID cross-correlation, i.e. potential[x] = sum_d state[x + d - k//2]
    K[d].  Placing tap d of every axis at the world index (k//2 - d) mod n
    (taps that land on the same index add up when a kernel is longer than
    the world) gives a world-sized kernel whose FFT convolution is that same
    sum, so the engine's FFT path computes the direct path's potential.
    ``pads`` gives another leading wrap pad per axis (tap d then lands at
    (pad - d) mod n)."""
    from .grad import kernel_spectrum  # the device real-to-half FFT of world-sized kernels
    nd = len(world)
    world = tuple(int(w) for w in world)
    if K.dim() < nd + 2 or K.shape[-nd - 1] != 1 or K.shape[-nd - 2] != nb_channels * max_k:
        raise ValueError(f'direct-path kernels {tuple(K.shape)} are not [..., {nb_channels * max_k}, 1, *kernel_dims]')
    _require_cuda('K', K)
    lead = tuple(K.shape[:-nd - 2])
    kd = tuple(int(k) for k in K.shape[-nd:])
    dev = K.device
    vals = K.reshape((-1, ) + kd)  # [planes, *kernel_dims]
    planes = vals.shape[0]
    kw = torch.zeros((planes, ) + world, dtype=torch.float32, device=dev)
    lo = [k // 2 for k in kd] if pads is None else [int(p) for p in pads]
    axes = [(p - torch.arange(k, device=dev)) % n for p, k, n in zip(lo, kd, world)]
    grids = torch.meshgrid(*axes, indexing='ij')
    pidx = torch.arange(planes, device=dev).view((planes, ) + (1, ) * nd).expand((planes, ) + kd)
    kw.index_put_((pidx, ) + tuple(g.unsqueeze(0).expand((planes, ) + kd) for g in grids), vals,
                  accumulate=True)
    half = kernel_spectrum(kw, nd)
    return half.reshape(lead + (nb_channels, max_k) + tuple(half.shape[1:]))


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
        kernel_shape = tuple(int(s) for s in kernel_shape)
        self.kernel_shape = kernel_shape
        self.fft = bool(fft)
        self._mapping, self._slug, self._average = mapping, get_state_fn_slug, average_weight
        self._models = {}
        self._cached = None  # (K, K._version, world, half spectra) of the direct path
        if self.fft:
            self._model = Model(kernel_shape[3:], kernel_shape[1], mapping, get_state_fn_slug, average_weight)
            self._models[self._model.world] = self._model
        else:
            # fft=False (helpers.py:465-487): K is [C*max_k, 1, *kernel_dims];
            # the world is the state's, known at the first call
            nb_channels = len(mapping.cin_kernels)
            max_k = mapping.kernel_table()[3]
            if len(kernel_shape) not in (4, 5) or kernel_shape[0] != nb_channels * max_k or kernel_shape[1] != 1:
                raise ValueError(f'direct-path kernel shape {kernel_shape} is not [{nb_channels * max_k}, 1, '
                                 '*kernel_dims]')
            self._nb_channels = nb_channels
            self._model = None

    @property
    def model(self) -> Model:
        if self._model is None:
            raise ValueError('a direct-path (fft=False) update function learns its world from the first state it '
                             'is given: use model_for(world)')
        return self._model

    def model_for(self, world: Sequence[int]) -> Model:
        """The engine model for worlds of shape ``world`` (the one fixed
        model for fft=True, one per world shape for fft=False)."""
        world = tuple(int(w) for w in world)
        if self.fft:
            if world != self._model.world:
                raise ValueError(f'world {world} does not match the kernels\' world {self._model.world}')
            return self._model
        m = self._models.get(world)
        if m is None:
            m = Model(world, self._nb_channels, self._mapping, self._slug, self._average)
            self._models[world] = m
        self._model = m
        return m

    def spectra(self, K: torch.Tensor, world: Sequence[int]) -> torch.Tensor:
        """The engine's half spectra (float32 view ``[..., C, max_k,
        *world_half, 2]``) of ``K``: leniax's FFT kernels (full or half
        spectrum) for fft=True, the direct path's real kernels for fft=False
        (converted once per tensor and in-place version)."""
        if self.fft:
            return half_spectrum(K, world)
        world = tuple(int(w) for w in world)
        c = self._cached
        if c is not None and c[0] is K and c[1] == K._version and c[2] == world:
            return c[3]
        m = self.model_for(world)
        kh = torch.view_as_real(direct_spectrum(K.to(torch.float32), world, m.C, m.max_k).contiguous())
        self._cached = (K, K._version, world, kh)
        return kh

    def __call__(self, rng_key, state, K, gf_params, kernels_weight_per_channel, dt):
        _require_cuda('state', state)
        m = self.model_for(state.shape[2:])
        if state.shape[1] != m.C:
            raise ValueError(f'state shape {tuple(state.shape)} does not match [N, {m.C}, *{m.world}]')
        dev = state.device
        N = state.shape[0]
        state = state.contiguous()
        kh = self.spectra(K if K.device == dev else K.to(dev), m.world)
        if not self.fft:
            kh = kh.unsqueeze(0)
        if kh.dim() < 1 or kh.shape[0] != 1:
            raise ValueError('update shares one spectrum across the batch: K must be [1, C, max_k, ...]')
        check_spectra(kh, (1, ), m.C, m.max_k, m.world)
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


# ---------------------------------------------------------------------------
# The step's building blocks (core.py:52-319), each on the device
_POT_PLANS = {}


def _potential_plan(world, C, max_k, tc):
    key = (tuple(world), C, max_k, tuple(tc))
    p = _POT_PLANS.get(key)
    if p is None:
        # identity growth, zero weights summed, v1: the plan computes the
        # potentials; its field and state outputs are discarded
        p = _lib.Plan(len(world), tuple(world), C, [t // max_k for t in tc], [t % max_k for t in tc],
                      [_lib.GF_IDS['identity']] * len(tc), max_k, register['v1'], False)
        _POT_PLANS[key] = p
    return p


def _potentials(state: torch.Tensor, kh: torch.Tensor, C: int, max_k: int, tc_indices) -> torch.Tensor:
    _require_cuda('state', state)
    if state.shape[1] != C:
        raise ValueError(f'state {tuple(state.shape)} has not {C} channels')
    world = tuple(int(w) for w in state.shape[2:])
    tc = list(range(C * max_k)) if tc_indices is None else [int(t) for t in tc_indices]
    if not tc or min(tc) < 0 or max(tc) >= C * max_k:
        raise ValueError(f'tc_indices {tc} outside [0, {C * max_k})')
    plan = _potential_plan(world, C, max_k, tc)
    dev = state.device
    N = state.shape[0]
    state = state.contiguous()
    gf = torch.tensor([[0., 1.]] * len(tc), dtype=torch.float32, device=dev)
    w = torch.zeros((C, len(tc)), dtype=torch.float32, device=dev)
    dt = torch.zeros(1, dtype=torch.float32, device=dev)
    out, field = torch.empty_like(state), torch.empty_like(state)
    potential = torch.empty((N, len(tc)) + world, dtype=torch.float32, device=dev)
    lib = _lib.load()
    ws = workspace(lib.lgx_update_workspace_bytes(plan.handle, N), dev)
    _lib.check(
        lib.lgx_update(plan.handle, N, state.data_ptr(), kh.data_ptr(), gf.data_ptr(), w.data_ptr(), dt.data_ptr(), 0,
                       out.data_ptr(), field.data_ptr(), potential.data_ptr(), ws.data_ptr(), ws.numel(),
                       _stream_handle(dev)))
    return potential


def get_potential_fft(state: torch.Tensor, K: torch.Tensor, tc_indices=None, channel_first: bool = True):
    """core.py:52-102: the potential of every kernel, ``real(ifftn(fftn(state)
    * K))``, for ``state`` ``[N, C, *world]`` and leniax's spectrum ``K``
    ``[1, C, max_k, *world]`` (or its half); returns ``[N, C*max_k, *world]``,
    or the ``tc_indices`` kernels only."""
    if not channel_first:
        raise NotImplementedError('the engine takes channel-first states')
    world = tuple(int(w) for w in state.shape[2:])
    if K.dim() != 3 + len(world) or K.shape[0] != 1 or K.shape[1] != state.shape[1]:
        raise ValueError(f'K {tuple(K.shape)} is not [1, {state.shape[1]}, max_k, *{world}]')
    kh = half_spectrum(K if K.device == state.device else K.to(state.device), world)
    check_spectra(kh, (1, ), int(K.shape[1]), int(K.shape[2]), world)
    return _potentials(state, kh, int(K.shape[1]), int(K.shape[2]), tc_indices)


def get_potential(state: torch.Tensor, K: torch.Tensor, padding, tc_indices=None, channel_first: bool = True):
    """core.py:105-146: the wrap-padded VALID cross-correlation of ``state``
    ``[N, C, *world]`` with the real kernels ``K`` ``[C*max_k, 1,
    *kernel_dims]`` and ``padding`` ``[(0, 0), (0, 0), (lo, hi), ...]``
    (helpers.py:465-481), computed by the engine's FFT path on the equivalent
    world-sized kernels (``direct_spectrum``)."""
    if not channel_first:
        raise NotImplementedError('the engine takes channel-first states')
    world = tuple(int(w) for w in state.shape[2:])
    nd = len(world)
    C = int(state.shape[1])
    kd = tuple(int(k) for k in K.shape[2:])
    pads = [tuple(int(v) for v in p) for p in padding][2:]
    if len(kd) != nd or len(pads) != nd or K.shape[0] % C:
        raise ValueError(f'K {tuple(K.shape)} / padding {padding} do not fit states {tuple(state.shape)}')
    for (lo, hi), k in zip(pads, kd):
        if lo + hi != k - 1:
            raise ValueError('padding must keep the world size (lo + hi = kernel size - 1 on every axis)')
    max_k = int(K.shape[0]) // C
    Kd = (K if K.device == state.device else K.to(state.device)).to(torch.float32)
    kh = torch.view_as_real(direct_spectrum(Kd, world, C, max_k, [lo for lo, _ in pads]).unsqueeze(0).contiguous())
    return _potentials(state, kh, C, max_k, tc_indices)


def _merge_mode(weighted_fn) -> int:
    if weighted_fn is weighted_mean:
        return 1
    if weighted_fn is weighted_sum:
        return 0
    return -1


def get_field(potential: torch.Tensor, gf_params: torch.Tensor, kernels_weight_per_channel: torch.Tensor,
              growth_fn_t, weighted_fn) -> torch.Tensor:
    """core.py:163-199: per-kernel growth of ``potential`` ``[N, K, *world]``
    (``growth_fn_t``: K growth functions of ``growth_functions``, slugs or
    engine ids; ``gf_params`` ``[K, 2]``) merged per channel by
    ``weighted_fn`` (``weighted_mean`` / ``weighted_sum`` fused on the
    device, or any callable applied to the ``[N, K, *world]`` growth
    fields) with ``kernels_weight_per_channel`` ``[C, K]``."""
    from .growth_functions import engine_id
    _require_cuda('potential', potential)
    dev = potential.device
    N, K = int(potential.shape[0]), int(potential.shape[1])
    ids = [engine_id(g) for g in growth_fn_t]
    if len(ids) != K:
        raise ValueError(f'{len(ids)} growth functions for {K} potentials')
    gf = gf_params.to(dev, torch.float32).reshape(K, 2).contiguous()
    w = kernels_weight_per_channel.to(dev, torch.float32).contiguous()
    C = int(w.shape[0])
    if tuple(w.shape) != (C, K):
        raise ValueError(f'weights {tuple(w.shape)} are not [C, {K}]')
    pot = potential.contiguous()
    cells = int(pot[0, 0].numel()) if N else 1
    ida = (ctypes.c_int * K)(*ids)
    lib = _lib.load()
    mode = _merge_mode(weighted_fn)
    if mode < 0:  # a caller's own merge over the device growth fields
        fields = torch.empty_like(pot)
        _lib.check(lib.lgx_growth(N, K, cells, ida, pot.data_ptr(), gf.data_ptr(), fields.data_ptr(),
                                  _stream_handle(dev)))
        return weighted_fn(fields, w)
    field = torch.empty((N, C) + tuple(pot.shape[2:]), dtype=torch.float32, device=dev)
    _lib.check(lib.lgx_field(N, K, C, cells, ida, pot.data_ptr(), gf.data_ptr(), w.data_ptr(), mode,
                             field.data_ptr(), _stream_handle(dev)))
    return field


def _weighted(fields: torch.Tensor, weights: torch.Tensor, mean: int) -> torch.Tensor:
    _require_cuda('fields', fields)
    dev = fields.device
    N, K = int(fields.shape[0]), int(fields.shape[1])
    w = weights.to(dev, torch.float32).contiguous()
    C = int(w.shape[0])
    if tuple(w.shape) != (C, K):
        raise ValueError(f'weights {tuple(w.shape)} are not [C, {K}]')
    f = fields.contiguous()
    out = torch.empty((N, C) + tuple(f.shape[2:]), dtype=torch.float32, device=dev)
    cells = int(f[0, 0].numel()) if N else 1
    _lib.check(_lib.load().lgx_weighted(N, K, C, cells, f.data_ptr(), w.data_ptr(), mean, out.data_ptr(),
                                        _stream_handle(dev)))
    return out


def weighted_sum(fields: torch.Tensor, weights: torch.Tensor) -> torch.Tensor:
    """core.py:202-225: ``[N, K, *world]`` fields -> ``[N, C, *world]``,
    ``sum_k weights[c, k] fields[:, k]``."""
    return _weighted(fields, weights, 0)


def weighted_mean(fields: torch.Tensor, weights: torch.Tensor) -> torch.Tensor:
    """core.py:228-242: ``weighted_sum`` divided by ``weights.sum(1)``."""
    return _weighted(fields, weights, 1)


def _state(slug, state, field, dt):
    _require_cuda('state', state)
    _require_cuda('field', field)
    if field.shape != state.shape:
        raise ValueError(f'field {tuple(field.shape)} and state {tuple(state.shape)} differ')
    dev = state.device
    N, C = int(state.shape[0]), int(state.shape[1])
    s, f = state.contiguous(), field.contiguous()
    dtt = torch.as_tensor(dt, dtype=torch.float32, device=dev).reshape(-1).contiguous()
    per_world = dtt.numel() > 1
    if per_world and dtt.numel() != N:
        raise ValueError(f'dt has {dtt.numel()} values for {N} worlds')
    out = torch.empty_like(s)
    cells = int(s[0, 0].numel()) if N else 1
    _lib.check(_lib.load().lgx_state(N, C, cells, register[slug], s.data_ptr(), f.data_ptr(), dtt.data_ptr(),
                                     1 if per_world else 0, out.data_ptr(), _stream_handle(dev)))
    return out


def get_state(rng_key, state: torch.Tensor, field: torch.Tensor, dt) -> torch.Tensor:
    """core.py:245-272: ``clip(state + dt * field, 0, 1)`` (the engine's
    adjoint takes the straight-through or mask gradient, ``grad.rollout``)."""
    return _state('v1', state, field, dt)


def get_state_v2(rng_key, state: torch.Tensor, field: torch.Tensor, dt) -> torch.Tensor:
    """core.py:275-297: ``state * (1 - dt) + dt * field``."""
    return _state('v2', state, field, dt)


def get_state_simple(rng_key, state: torch.Tensor, field: torch.Tensor, dt) -> torch.Tensor:
    """core.py:300-319: ``state + dt * field``."""
    return _state('simple', state, field, dt)
