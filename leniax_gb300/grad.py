"""Differentiable Lenia rollouts on the GB300 engine.

leniax differentiates a rollout with ``jax.value_and_grad`` through the FFT
(``runner.py:363-448``: ``make_pipeline_fn`` / ``make_gradient_fn``; the v1
clip's gradient is the straight-through estimator, ``core.py:267-270``).
Here the reverse pass is the engine's hand-written adjoint (``lgx_adjoint``)
behind a ``torch.autograd.Function``:

* forward: ``steps`` Euler steps, keeping the state every ``checkpoint_every``
  steps in HBM;
* backward: for each segment, newest first, recompute its states and
  potentials from the checkpoint, then run the adjoint steps (conjugate-
  spectrum correlation, growth derivative, clip gradient ``'ste'`` or
  ``'mask'``).

Gradients flow to the initial cells, each kernel's world-sized fftshifted
real kernel (and through :func:`ring_kernel` to the ring weights ``b``), the
growth parameters ``(m, s)`` of every kernel and the full
``kernels_weight_per_channel`` matrix.  Models: every model ``lgx_run`` runs
-- 2D and 3D worlds, any number of channels and kernels, weighted mean or
sum; 2D one-kernel square worlds of 32..256 take the engine's specialised
one-kernel adjoint, all others its general N-D adjoint.
"""
import ctypes
import math
from typing import Sequence

import torch

from . import _lib
from .core import UpdateFn, _require_cuda, _stream_handle, workspace

CLIP_GRAD = {'ste': 0, 'mask': 1}
ENGINES = ('auto', 'nd')  # 'nd': the general N-D engine for the forward segments and the adjoint


def _bind(lib):
    if getattr(lib, '_lgx_grad_bound', False):
        return lib
    lib.lgx_adjoint_workspace_bytes.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    lib.lgx_adjoint_workspace_bytes.restype = ctypes.c_size_t
    lib.lgx_adjoint.argtypes = [ctypes.c_void_p, ctypes.POINTER(AdjointJob), ctypes.c_void_p, ctypes.c_size_t,
                                ctypes.c_void_p]
    lib.lgx_adjoint.restype = ctypes.c_int
    lib.lgx_adjoint_kernel_grad.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    lib.lgx_adjoint_kernel_grad.restype = ctypes.c_int
    lib.lgx_kernel_spectrum.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    lib.lgx_kernel_spectrum.restype = ctypes.c_int
    lib.lgx_kernel_spectrum_nd_workspace_bytes.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int]
    lib.lgx_kernel_spectrum_nd_workspace_bytes.restype = ctypes.c_size_t
    lib.lgx_kernel_spectrum_nd.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    lib.lgx_kernel_spectrum_nd.restype = ctypes.c_int
    lib.lgx_adjoint_kernel_grad_acc_bytes.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    lib.lgx_adjoint_kernel_grad_acc_bytes.restype = ctypes.c_size_t
    lib.lgx_plan_set_adjoint_engine.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.lgx_plan_set_adjoint_engine.restype = ctypes.c_int
    lib._lgx_grad_bound = True
    return lib


class AdjointJob(ctypes.Structure):
    _fp = ctypes.c_void_p
    _fields_ = [
        ('n_sols', ctypes.c_int), ('n_init', ctypes.c_int), ('steps', ctypes.c_int), ('k_half', _fp),
        ('gf_params', _fp), ('weights', _fp), ('T', _fp), ('traj_cells', _fp), ('traj_potential', _fp),
        ('lambda_in', _fp), ('lambda_out', _fp), ('kernel_grad_acc', _fp), ('grad_gf', _fp), ('grad_weights', _fp),
        ('clip_grad', ctypes.c_int), ('cells_after', _fp)
    ]


def kernel_spectrum(k_real: torch.Tensor, nb_dims: int = 2) -> torch.Tensor:
    """fftn over the last ``nb_dims`` axes of world-sized fftshifted real
    kernels ``[..., *world]`` on the device (leniax ``kernels.py:145-149``) ->
    Hermitian halves ``[..., *world[:-1], W//2+1]`` complex64."""
    _require_cuda('k_real', k_real)
    world = tuple(int(w) for w in k_real.shape[-nb_dims:])
    lead = k_real.shape[:-nb_dims]
    planes = int(math.prod(lead)) if lead else 1
    kr = k_real.contiguous()
    out = torch.empty(lead + world[:-1] + (world[-1] // 2 + 1, ), dtype=torch.complex64, device=k_real.device)
    lib = _bind(_lib.load())
    H, W = world[-2], world[-1]
    if nb_dims == 2 and H == W and H in (32, 64, 128, 256):
        ws = workspace(planes * H * W * 4, k_real.device)
        _lib.check(lib.lgx_kernel_spectrum(H, W, planes, kr.data_ptr(), out.data_ptr(), ws.data_ptr(), ws.numel(),
                                           _stream_handle(k_real.device)))
        return out
    wa = (ctypes.c_int * 3)(*world)
    nbytes = lib.lgx_kernel_spectrum_nd_workspace_bytes(nb_dims, wa, planes)
    if nbytes == 0:
        raise _lib.LgxError(_lib.LGX_ERR_UNSUPPORTED, f'no kernel spectrum for world {world}')
    ws = workspace(nbytes, k_real.device)
    _lib.check(lib.lgx_kernel_spectrum_nd(nb_dims, wa, planes, kr.data_ptr(), out.data_ptr(), ws.data_ptr(),
                                          ws.numel(), _stream_handle(k_real.device)))
    return out


def _engine_spectra(m, k_half: torch.Tensor) -> torch.Tensor:
    """Per-kernel half spectra ``[Ns, K, ...]`` placed at leniax's spectrum
    positions ``[Ns, C, max_k, ...]`` (kernels.py:122-152; padded slots zero)."""
    Ns = k_half.shape[0]
    out = torch.zeros((Ns, m.C, m.max_k) + tuple(k_half.shape[2:]), dtype=k_half.dtype, device=k_half.device)
    for k, (c, j) in enumerate(zip(m.cin, m.slot)):
        out[:, c, j] = k_half[:, k]
    return out


# ---------------------------------------------------------------------------
# differentiable kernel construction (kernels.py:176-212 with kernel_functions)
def _kf_torch(slug, q, X):
    if slug == 'gauss_bump':  # kernel_functions.py:40-69
        return torch.exp(q * (q - 1 / (X * (1 - X) + 1e-7)))
    if slug == 'poly_quad':  # kernel_functions.py:7-37
        return (4 * X * (1 - X))**q
    if slug == 'gauss':  # kernel_functions.py:105-134
        return torch.exp(-(((X - q) / (0.3 * q))**2) / 2)
    raise NotImplementedError(f'kernel function {slug!r} has no differentiable form here')


def ring_kernel(R: float, r: float, b: torch.Tensor, kf_slug: str, kf_params: Sequence[float],
                world: Sequence[int]) -> torch.Tensor:
    """World-sized, fftshifted ring kernel (what leniax FFTs), differentiable
    in the ring weights ``b`` (1-D tensor).  Mirrors ``circle_2d``
    (kernels.py:176-212) -- over every world axis for 3D worlds, the distance
    taken over all axes -- the centring pad (kernels.py:93-101) and the
    fftshift (kernels.py:148)."""
    dev, dt = b.device, torch.float32
    nd = len(world)
    k = math.ceil(r * R)
    idx = torch.arange(2 * k, device=dev, dtype=dt) - k
    grids = torch.meshgrid(*([idx] * nd), indexing='ij')
    dist = torch.sqrt(sum((g / (r * R))**2 for g in grids))
    nb = b.shape[0]
    bdist = nb * dist
    ring = torch.clamp(torch.floor(bdist).long(), max=nb - 1)
    raw = _kf_torch(kf_slug, float(kf_params[0]), torch.remainder(bdist, 1.0))
    kern = (dist < 1).to(dt) * raw * b[ring]
    kern = kern / kern.sum()
    pads = []
    for ws in reversed(list(world)):  # F.pad lists the last axis first
        need = ws - 2 * k
        pads += [need // 2, need - need // 2]
    full = torch.nn.functional.pad(kern, pads)
    # fftshift (a roll by n // 2 along every axis, also for odd sides)
    return torch.roll(full, shifts=tuple(ws // 2 for ws in world), dims=tuple(range(nd)))


# ---------------------------------------------------------------------------
class LeniaRolloutFunction(torch.autograd.Function):
    """``final = LeniaRolloutFunction.apply(cells0, k_real, gf_params, weights,
    T, update_fn, steps, checkpoint_every, clip_grad, engine)``

    cells0 ``[Ns, Ni, C, *world]``; k_real ``[Ns, K, *world]`` (or
    ``[Ns, *world]`` for one kernel): each true kernel's world-sized
    fftshifted real kernel in leniax's channel-sorted order; gf_params
    ``[Ns, K, 2]``; weights ``[Ns, C, K]``; T ``[Ns]``.  Returns the state
    after ``steps`` steps ``[Ns, Ni, C, *world]``.  ``engine`` ``'auto'`` runs
    the engines lgx_run and lgx_adjoint pick; ``'nd'`` runs the general N-D
    engine for both (any model).
    """

    @staticmethod
    def forward(ctx, cells0, k_real, gf_params, weights, T, update_fn: UpdateFn, steps: int, checkpoint_every: int,
                clip_grad: str, engine: str = 'auto'):
        _require_cuda('cells0', cells0)
        m = update_fn.model_for(cells0.shape[3:])
        if cells0.dim() != 3 + len(m.world) or tuple(cells0.shape[2:]) != (m.C, ) + m.world:
            raise ValueError(f'cells0 {tuple(cells0.shape)} does not match [Ns, Ni, {m.C}, *{m.world}]')
        dev = cells0.device
        Ns, Ni = cells0.shape[:2]
        nd = len(m.world)
        kr = k_real.detach().float().reshape((Ns, m.K) + m.world)
        k_half = _engine_spectra(m, kernel_spectrum(kr, nd))
        gf = gf_params.detach().float().reshape(Ns, m.K, 2).contiguous()
        w = weights.detach().float().reshape(Ns, m.C, m.K).contiguous()
        for name, t in (('k_real', kr), ('gf_params', gf), ('weights', w)):
            _require_cuda(name, t)
            if t.device != dev:
                raise ValueError(f'{name} is on {t.device}, cells0 on {dev}')
        Tt = torch.as_tensor(T, dtype=torch.float32, device=dev).reshape(-1).expand(Ns).contiguous()
        k = max(1, int(checkpoint_every))
        ckpts = [cells0.detach().contiguous()]
        cur = ckpts[0]
        done = 0
        while done < steps:
            n = min(k, steps - done)
            cur = _segment(update_fn, cur, k_half, gf, w, Tt, n, traj=False, engine=engine)
            done += n
            if done < steps:
                ckpts.append(cur)
        ctx.save_for_backward(k_half, gf, w, Tt, *ckpts, cur)
        ctx.update_fn, ctx.steps, ctx.k, ctx.clip = update_fn, steps, k, CLIP_GRAD[clip_grad]
        ctx.k_shape = tuple(k_real.shape)
        ctx.engine = engine
        return cur

    @staticmethod
    def backward(ctx, grad_final):
        k_half, gf, w, Tt, *ckpts, final = ctx.saved_tensors
        after = ckpts[1:] + [final]  # the state after each segment
        update_fn, steps, k = ctx.update_fn, ctx.steps, ctx.k
        if steps == 0:
            return grad_final, torch.zeros(ctx.k_shape, device=grad_final.device), torch.zeros_like(gf), \
                torch.zeros_like(w), None, None, None, None, None, None
        m = update_fn.model_for(ckpts[0].shape[3:])
        dev = grad_final.device
        Ns, Ni = ckpts[0].shape[:2]
        lib = _bind(_lib.load())
        handle = m.plan.handle
        _lib.check(lib.lgx_plan_set_adjoint_engine(handle, _lib.ENGINES[ctx.engine]))
        lam = grad_final.detach().float().contiguous().clone()
        lam_out = torch.empty_like(lam)
        acc_bytes = lib.lgx_adjoint_kernel_grad_acc_bytes(handle, Ns, Ni)
        ws_bytes = lib.lgx_adjoint_workspace_bytes(handle, Ns, Ni)
        if acc_bytes == 0 or ws_bytes == 0:
            raise _lib.LgxError(_lib.LGX_ERR_UNSUPPORTED, 'no adjoint for this model')
        acc = torch.zeros(acc_bytes // 4, dtype=torch.float32, device=dev)
        g_gf = torch.zeros((Ns, m.K, 2), dtype=torch.float32, device=dev)
        g_w = torch.zeros((Ns, m.C, m.K), dtype=torch.float32, device=dev)
        ws = workspace(ws_bytes, dev)
        seg_starts = list(range(0, steps, k))
        # Segment j - 1's trajectory is recomputed on a side stream while
        # segment j's adjoint runs: the two launches take different SMs when
        # a batch fills fewer than half of them.
        main = torch.cuda.current_stream(dev)
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(main)

        def recompute(j):
            with torch.cuda.stream(side):
                tr = _segment(update_fn, ckpts[j], k_half, gf, w, Tt, min(k, steps - seg_starts[j]), traj=True,
                              engine=ctx.engine)
                ev = torch.cuda.Event()
                ev.record(side)
            return tr, ev

        kh = torch.view_as_real(k_half.contiguous())
        nxt = recompute(len(seg_starts) - 1)
        for j in reversed(range(len(seg_starts))):
            n = min(k, steps - seg_starts[j])
            (tc, tp), ready = nxt
            if j > 0:
                nxt = recompute(j - 1)
            main.wait_event(ready)
            tc.record_stream(main)
            tp.record_stream(main)
            job = AdjointJob()
            job.n_sols, job.n_init, job.steps = Ns, Ni, n
            job.k_half, job.gf_params, job.weights, job.T = (kh.data_ptr(), gf.data_ptr(), w.data_ptr(),
                                                             Tt.data_ptr())
            job.traj_cells, job.traj_potential = tc.data_ptr(), tp.data_ptr()
            job.lambda_in, job.lambda_out = lam.data_ptr(), lam_out.data_ptr()
            job.kernel_grad_acc = acc.data_ptr()
            job.grad_gf, job.grad_weights = g_gf.data_ptr(), g_w.data_ptr()
            job.clip_grad = ctx.clip
            job.cells_after = after[j].data_ptr()
            _lib.check(lib.lgx_adjoint(handle, job, ws.data_ptr(), ws.numel(), _stream_handle(dev)))
            lam, lam_out = lam_out, lam
        g_k = torch.empty((Ns, m.K) + m.world, dtype=torch.float32, device=dev)
        _lib.check(lib.lgx_adjoint_kernel_grad(handle, Ns, Ni, acc.data_ptr(), g_k.data_ptr(), ws.data_ptr(),
                                               ws.numel(), _stream_handle(dev)))
        return lam, g_k.reshape(ctx.k_shape), g_gf, g_w, None, None, None, None, None, None


def _segment(update_fn, cells, k_half, gf, w, Tt, n, traj, engine='auto'):
    """n Euler steps from `cells` through lgx_run (no statistics needed)."""
    m = update_fn.model_for(cells.shape[3:])
    dev = cells.device
    Ns, Ni = cells.shape[:2]
    lib = _lib.load()
    final = torch.empty_like(cells)
    job = _lib.Rollout()
    job.n_sols, job.n_init, job.steps = Ns, Ni, n
    kh = torch.view_as_real(k_half.contiguous())
    job.cells0, job.k_half, job.gf_params, job.weights, job.T = (cells.data_ptr(), kh.data_ptr(), gf.data_ptr(),
                                                                  w.data_ptr(), Tt.data_ptr())
    job.stats_R, job.stats_T = 1.0, 1.0
    job.final_cells = final.data_ptr()
    tc = tp = None
    if traj:
        tc = torch.empty((n, Ns * Ni, m.C) + m.world, dtype=torch.float32, device=dev)
        tp = torch.empty((n, Ns * Ni, m.K) + m.world, dtype=torch.float32, device=dev)
        job.traj_cells, job.traj_potential = tc.data_ptr(), tp.data_ptr()
    eng = _lib.ENGINES[engine]
    ws = workspace(lib.lgx_run_workspace_bytes(m.plan.handle, Ns, Ni, n, eng), dev)
    job.engine = eng
    _lib.check(lib.lgx_run(m.plan.handle, job, ws.data_ptr(), ws.numel(), _stream_handle(dev)))
    return (tc, tp) if traj else final


def rollout(cells0, k_real, gf_params, weights, T, update_fn: UpdateFn, steps: int, checkpoint_every: int = 16,
            clip_grad: str = 'ste', engine: str = 'auto'):
    """Differentiable rollout (see :class:`LeniaRolloutFunction`)."""
    if clip_grad not in CLIP_GRAD:
        raise ValueError("clip_grad must be 'ste' or 'mask'")
    if engine not in ENGINES:
        raise ValueError(f'engine must be one of {ENGINES}')
    return LeniaRolloutFunction.apply(cells0, k_real, gf_params, weights, T, update_fn, steps, checkpoint_every,
                                      clip_grad, engine)


def direct_world_kernels(K: torch.Tensor, world: Sequence[int], nb_channels: int, max_k: int, cin: Sequence[int],
                         slot: Sequence[int]) -> torch.Tensor:
    """leniax's direct-path kernels ``[*lead, C*max_k, 1, *kernel_dims]``
    (``kernels.get_kernels_and_mapping(..., fft=False)``) as the world-sized
    real kernels ``[*lead, K, *world]`` of the true kernels (``cin``,
    ``slot``), the layout :func:`rollout` takes; differentiable in ``K``.

    ``core.get_potential`` (core.py:105-146) wrap-pads the state by ``k//2``
    before each axis and cross-correlates: potential[x] = sum_d state[x + d -
    k//2] K[d].  A world kernel with tap d at index (k//2 - d) mod n gives the
    same sum as a circular convolution (taps landing on one index add up when
    a kernel is longer than the world), the placement of
    ``core.direct_spectrum``."""
    world = tuple(int(w) for w in world)
    nd = len(world)
    if K.dim() < nd + 2 or K.shape[-nd - 1] != 1 or K.shape[-nd - 2] != nb_channels * max_k:
        raise ValueError(f'direct-path kernels {tuple(K.shape)} are not [..., {nb_channels * max_k}, 1, *kernel_dims]')
    kd = tuple(int(k) for k in K.shape[-nd:])
    lead = tuple(K.shape[:-nd - 2])
    flat = torch.zeros(kd, dtype=torch.long)
    stride = 1
    for ax in reversed(range(nd)):
        pos = (kd[ax] // 2 - torch.arange(kd[ax])) % world[ax]
        shape = [1] * nd
        shape[ax] = kd[ax]
        flat = flat + pos.reshape(shape) * stride
        stride *= world[ax]
    taps = K.reshape(lead + (nb_channels * max_k, -1))
    sel = torch.tensor([c * max_k + s for c, s in zip(cin, slot)], dtype=torch.long, device=K.device)
    taps = taps.index_select(-2, sel)  # [*lead, K, taps]
    out = torch.zeros(lead + (len(sel), stride), dtype=K.dtype, device=K.device)
    out = out.index_add(out.dim() - 1, flat.reshape(-1).to(K.device), taps)
    return out.reshape(lead + (len(sel), ) + world)


class LeniaApply:
    """The per-step ``apply_fn`` of leniax's differentiable pipelines
    (``runner.make_pipeline_fn``, runner.py:363-423; the flax ``Step`` of the
    reference's kernel-learning example) on the engine:
    ``apply_fn(variables, rng_key, state, dt=dt) -> (state, field,
    potential)``, differentiable through :func:`rollout`.

    ``variables['params']`` (then ``variables``) holds ``'K'`` -- leniax's
    direct-path kernels ``[C*max_k, 1, *kernel_dims]`` or world-sized real
    kernels ``[K, *world]`` (fftshifted: the kernel's centre at index 0) --
    ``'gf_params'`` ``[K, 2]`` and ``'kernels_weight_per_channel'`` ``[C,
    K]``; ``state`` is ``[N, C, *world]``.  The adjoint differentiates cell
    states only, so ``field`` and ``potential`` come back as ``None``.
    :meth:`rollout` advances several steps in one engine call (what
    ``make_pipeline_fn`` uses when it keeps only the last state)."""

    def __init__(self, update_fn: UpdateFn, checkpoint_every: int = 16, clip_grad: str = 'ste', engine: str = 'auto'):
        if clip_grad not in CLIP_GRAD:
            raise ValueError("clip_grad must be 'ste' or 'mask'")
        if engine not in ENGINES:
            raise ValueError(f'engine must be one of {ENGINES}')
        self.update_fn = update_fn
        self.checkpoint_every = int(checkpoint_every)
        self.clip_grad = clip_grad
        self.engine = engine

    def kernels(self, variables, world):
        """(world-sized real kernels ``[K, *world]``, gf_params, weights) of ``variables``."""
        p = {k: v for k, v in variables.items() if k != 'params'}
        p.update(variables.get('params', {}))
        missing = [k for k in ('K', 'gf_params', 'kernels_weight_per_channel') if k not in p]
        if missing:
            raise KeyError(f'variables hold no {missing}')
        m = self.update_fn.model_for(world)
        K = p['K']
        if K.dim() == 2 + len(m.world):
            K = direct_world_kernels(K, m.world, m.C, m.max_k, m.cin, m.slot)
        elif tuple(K.shape) != (m.K, ) + m.world:
            raise ValueError(f'K {tuple(K.shape)} is neither [{m.C * m.max_k}, 1, *kernel_dims] nor '
                             f'[{m.K}, *{m.world}]')
        return K, p['gf_params'], p['kernels_weight_per_channel']

    def rollout(self, variables, state: torch.Tensor, steps: int, dt) -> torch.Tensor:
        """The state after ``steps`` Euler steps of ``dt`` from ``state``."""
        k_real, gf, w = self.kernels(variables, tuple(state.shape[2:]))
        T = torch.full((1, ), 1.0 / float(dt), dtype=torch.float32)
        fin = rollout(state[None], k_real[None], gf[None], w[None], T, self.update_fn, int(steps),
                      self.checkpoint_every, self.clip_grad, self.engine)
        return fin[0]

    def __call__(self, variables, rng_key, state: torch.Tensor, dt):
        return self.rollout(variables, state, 1, dt), None, None
