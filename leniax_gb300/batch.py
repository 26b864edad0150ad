"""Uneven batches: worlds of different shapes, kernels, growth parameters and
time steps advanced together in ONE persistent launch.

leniax batches a search with ``jax.vmap`` over identically shaped worlds
(``runner.py:167-215`` ``run_scan_mem_optimized``; ``experiments`` vmaps one
world size and one R at a time).  Here every world carries its own kernel
spectrum (its own R), ``(m, s)``, kernel weight and ``T``; worlds of one shape
form a :class:`WorldClass`, and :class:`UnevenBatch` runs up to eight classes
(2D 32^2/64^2/128^2/256^2, 3D 32^3/64^3) through ``lgx_batch_run``, and any
number of classes of other shapes (every world the N-D engine takes: odd,
prime, non-square, large, other 3D sides) through one ``lgx_run`` each on the
same stream (every world its own solution, with its own statistics R and T):

* a device work queue (one item = 8, 4 or 1 small 2D worlds, or one large
  world) consumed by one 512-thread CTA per SM with an atomic counter,
  largest items first;
* per-class statistics (``compute_stats``, ``check_heuristics`` N, the
  bounding-box N) after the launch;
* the whole sequence captured once in a CUDA graph and replayed
  (:meth:`UnevenBatch.capture`), inputs refreshed in place between replays.

The queue order, the grid and the 3D line-transform width are chosen by the
autotuner in :mod:`leniax_gb300.autotune`.
"""
import ctypes
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _lib
from . import kernels as lkernels
from .core import _require_cuda, _stream_handle, workspace
from .statistics import split_stats

MAX_CLASSES = 8
ORDERS = {'largest_first': 0, 'as_given': 1, 'explicit': 2}
SHAPES = {(2, 32), (2, 64), (2, 128), (2, 256), (3, 32), (3, 64)}
_fp = ctypes.c_void_p


class BatchClassC(ctypes.Structure):
    _fields_ = [
        ('nb_dims', ctypes.c_int), ('size', ctypes.c_int), ('n_worlds', ctypes.c_int), ('gf_id', ctypes.c_int),
        ('state_fn', ctypes.c_int), ('mean', ctypes.c_int), ('cells0', _fp), ('k_half', _fp), ('gf_params', _fp),
        ('weights', _fp), ('T', _fp), ('stats_R', _fp), ('stats_T', _fp), ('final_cells', _fp), ('stats', _fp),
        ('n_continue', _fp), ('n_box', _fp), ('centroid', _fp)
    ]


class BatchJobC(ctypes.Structure):
    _fields_ = [('n_classes', ctypes.c_int), ('steps', ctypes.c_int), ('classes', ctypes.POINTER(BatchClassC)),
                ('order', ctypes.c_int), ('grid', ctypes.c_int), ('line_group', ctypes.c_int),
                ('class_order', ctypes.POINTER(ctypes.c_int))]


def _bind(lib):
    if getattr(lib, '_lgx_batch_bound', False):
        return lib
    lib.lgx_batch_workspace_bytes.argtypes = [ctypes.POINTER(BatchJobC), ctypes.POINTER(ctypes.c_size_t)]
    lib.lgx_batch_workspace_bytes.restype = ctypes.c_int
    lib.lgx_batch_run.argtypes = [ctypes.POINTER(BatchJobC), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    lib.lgx_batch_run.restype = ctypes.c_int
    lib._lgx_batch_bound = True
    return lib


def persistent_shape(world: Sequence[int]) -> bool:
    """Whether worlds of this shape run in the persistent launch (square or
    cubic sides of ``SHAPES``); every other shape runs through ``lgx_run``."""
    return (len(world), world[0]) in SHAPES and all(w == world[0] for w in world)


@dataclass
class WorldClass:
    """Worlds of one shape.  ``cells0`` ``[n, *world]`` float32; ``K`` each
    world's kernel spectrum, full ``[n, *world]`` or Hermitian half
    ``[n, *world[:-1], W//2+1]`` complex64 (leniax's fftn of the fftshifted
    kernel, kernels.py:145-152); ``gf_params`` ``[n, 2]``; ``weights``,
    ``T``, ``R`` ``[n]``.  ``T_static`` is the T of ``compute_stats``
    (defaults to ``T``)."""
    cells0: torch.Tensor
    K: torch.Tensor
    gf_params: torch.Tensor
    weights: torch.Tensor
    T: torch.Tensor
    R: torch.Tensor
    gf_slug: str = 'gaussian'
    state_slug: str = 'v1'
    average: bool = True
    T_static: Optional[torch.Tensor] = None

    @property
    def world(self):
        return tuple(self.cells0.shape[1:])

    @property
    def n(self):
        return int(self.cells0.shape[0])


def world_spectra(world: Sequence[int], R: Sequence[float], kernel_params: Dict, device=None) -> torch.Tensor:
    """Per-world kernel spectra ``[n, *world[:-1], W//2+1]`` complex64 for
    one ring-kernel recipe (a leniax kernels_params entry: ``k_params`` [r,
    b], ``kf_slug``, ``kf_params``) at per-world radii ``R``, built on the GPU
    by :func:`leniax_gb300.kernels.ring_kernels` (kernels.py:66-212 per
    world)."""
    kp = kernel_params
    if kp.get('k_slug', 'circle_2d') != 'circle_2d':
        raise ValueError('world_spectra builds circle_2d ring kernels only')
    r, b = kp['k_params'][0], kp['k_params'][1]
    n = len(R)
    _, K = lkernels.ring_kernels(world, list(R), [r] * n, [list(b)] * n, kp['kf_slug'], list(kp['kf_params']),
                                 spectrum=True, device=device)
    return K


def _half(K: torch.Tensor, world, n: int) -> torch.Tensor:
    W = world[-1]
    if K.dtype != torch.complex64:
        raise TypeError(f'K must be complex64, got {K.dtype}')
    _require_cuda('K', K, torch.complex64)
    if K.shape[-1] == W:
        K = K[..., :W // 2 + 1]
    if tuple(K.shape) != (n, ) + tuple(world[:-1]) + (W // 2 + 1, ):
        raise ValueError(f'K has shape {tuple(K.shape)}; expected [{n}, {", ".join(map(str, world[:-1]))}, '
                         f'{W // 2 + 1}]')
    return torch.view_as_real(K.contiguous())


class UnevenBatch:
    """A fixed set of world classes advanced ``steps`` steps per :meth:`run`.

    Outputs live in preallocated tensors (``results()``).  The device
    tensors the launches read are ``inputs[i]`` (``cells0``, ``k_half``,
    ``gf_params``, ``weights``, ``T``, ``R``, ``T_static``); rewrite them in
    place between runs or graph replays to start a new search generation.  ``order`` is ``'largest_first'`` (estimated item cost),
    ``'as_given'`` or ``'explicit'`` (queue order of the classes in
    ``class_order``); ``grid`` 0 means one CTA per SM; ``line_group`` is the
    number of lanes per 3D line transform (2 or 4)."""

    def __init__(self, classes: List[WorldClass], steps: int, order='largest_first', grid=0, line_group=4,
                 with_stats=True, class_order: Optional[Sequence[int]] = None):
        if not classes:
            raise ValueError('an uneven batch needs at least one world class')
        if order not in ORDERS:
            raise ValueError(f'order must be one of {sorted(ORDERS)}')
        self.lib = _bind(_lib.load())
        self.classes = classes
        self.steps = int(steps)
        self.order, self.grid, self.line_group = order, int(grid), int(line_group)
        self.with_stats = bool(with_stats)
        self.device = classes[0].cells0.device
        self.inputs = []
        self.outputs = []
        # classes of the persistent launch; the others run through lgx_run
        self._persistent = [i for i, c in enumerate(classes) if persistent_shape(c.world)]
        if len(self._persistent) > MAX_CLASSES:
            raise ValueError(f'at most {MAX_CLASSES} classes of the persistent shapes, got {len(self._persistent)}')
        self._generic = []  # (class index, plan, Rollout, workspace)
        arr = (BatchClassC * max(1, len(self._persistent)))()
        for i, c in enumerate(classes):
            nd, size = len(c.world), c.world[0]
            for name in ('cells0', 'gf_params', 'weights', 'T', 'R'):
                _require_cuda(f'class {i} {name}', getattr(c, name))
            if c.gf_slug not in _lib.GF_IDS or c.state_slug not in _lib.STATE_IDS:
                raise ValueError(f'class {i}: unknown growth or state slug')
            n = c.n
            for name, shape in (('gf_params', (n, 2)), ('weights', (n, )), ('T', (n, )), ('R', (n, ))):
                t = getattr(c, name)
                if tuple(t.shape) != shape:
                    raise ValueError(f'class {i}: {name} has shape {tuple(t.shape)}, expected {shape}')
            kh = _half(c.K, c.world, n)
            if c.T_static is not None:
                _require_cuda(f'class {i} T_static', c.T_static)
                if tuple(c.T_static.shape) != (n, ):
                    raise ValueError(f'class {i}: T_static has shape {tuple(c.T_static.shape)}, expected ({n},)')
            tst = (c.T_static if c.T_static is not None else c.T).float().contiguous()
            ins = [c.cells0.contiguous(), kh, c.gf_params.contiguous(), c.weights.contiguous(), c.T.contiguous(),
                   c.R.float().contiguous(), tst]
            out = {'final': torch.empty_like(ins[0])}
            if self.with_stats:
                out['stats'] = torch.empty((n, max(self.steps, 1), 12), device=self.device)
                out['N'] = torch.empty((n, ), device=self.device)
                out['N_box'] = torch.empty((n, ), device=self.device)
                out['centroid'] = torch.empty((n, max(self.steps, 1), nd), device=self.device)
            self.inputs.append(dict(zip(('cells0', 'k_half', 'gf_params', 'weights', 'T', 'R', 'T_static'), ins)))
            self.outputs.append(out)
            if i not in self._persistent:
                self._generic.append(self._generic_run(i, c, ins, out))
                continue
            a = arr[self._persistent.index(i)]
            a.nb_dims, a.size, a.n_worlds = nd, size, n
            a.gf_id, a.state_fn, a.mean = _lib.GF_IDS[c.gf_slug], _lib.STATE_IDS[c.state_slug], int(c.average)
            a.cells0, a.k_half, a.gf_params, a.weights, a.T, a.stats_R, a.stats_T = [t.data_ptr() for t in ins]
            a.final_cells = out['final'].data_ptr()
            if self.with_stats:
                a.stats, a.n_continue = out['stats'].data_ptr(), out['N'].data_ptr()
                a.n_box, a.centroid = out['N_box'].data_ptr(), out['centroid'].data_ptr()
        self._arr = arr
        job = BatchJobC()
        job.n_classes, job.steps, job.classes = len(self._persistent), self.steps, arr
        job.order, job.grid, job.line_group = ORDERS[order], self.grid, self.line_group
        self.class_order = list(class_order) if class_order is not None else None
        if order == 'explicit':
            if self.class_order is None:
                raise ValueError("order='explicit' needs class_order")
            # the queue order of the persistent classes, in their own indices
            persistent_order = [self._persistent.index(i) for i in self.class_order if i in self._persistent]
            self._order_arr = (ctypes.c_int * max(1, len(persistent_order)))(*persistent_order)
            job.class_order = self._order_arr
        self._job = job
        self.ws = None
        if self._persistent:
            nbytes = ctypes.c_size_t(0)
            _lib.check(self.lib.lgx_batch_workspace_bytes(ctypes.byref(job), ctypes.byref(nbytes)))
            self.ws = workspace(nbytes.value, self.device)
        self.graph = None

    def _generic_run(self, i, c, ins, out):
        """The lgx_run job of a class the persistent launch does not take:
        its n worlds as n solutions of one init each."""
        nd = len(c.world)
        plan = _lib.Plan(nd, tuple(c.world), 1, [0], [0], [_lib.GF_IDS[c.gf_slug]], 1, _lib.STATE_IDS[c.state_slug],
                         bool(c.average))
        job = _lib.Rollout()
        job.n_sols, job.n_init, job.steps = c.n, 1, self.steps
        job.cells0, job.k_half, job.gf_params, job.weights, job.T = [t.data_ptr() for t in ins[:5]]
        job.stats_R, job.stats_T = 1.0, 1.0  # overridden per world below
        job.stats_R_sol, job.stats_T_sol = ins[5].data_ptr(), ins[6].data_ptr()
        job.final_cells = out['final'].data_ptr()
        if self.with_stats:
            # [n, steps, 12] / [n] / [n, steps, nd] are lgx_run's [Ns, steps, Ni = 1, ...] layouts
            job.stats, job.n_continue = out['stats'].data_ptr(), out['N'].data_ptr()
            job.n_box, job.centroid = out['N_box'].data_ptr(), out['centroid'].data_ptr()
        job.engine = 0
        ws = workspace(self.lib.lgx_run_workspace_bytes(plan.handle, c.n, 1, self.steps, 0), self.device)
        return i, plan, job, ws

    @property
    def cells_per_run(self) -> int:
        return sum(c.n * int(np.prod(c.world)) for c in self.classes) * self.steps

    def launch(self, stream=None):
        """Enqueue one rollout on ``stream`` (default: the current stream)."""
        h = stream.cuda_stream if stream is not None else _stream_handle(self.device)
        if self._persistent:
            _lib.check(self.lib.lgx_batch_run(ctypes.byref(self._job), self.ws.data_ptr(), self.ws.numel(), h))
        for _, plan, job, ws in self._generic:
            _lib.check(self.lib.lgx_run(plan.handle, ctypes.byref(job), ws.data_ptr(), ws.numel(), h))

    def capture(self):
        """Capture :meth:`launch` in a CUDA graph; :meth:`run` then replays it."""
        self.launch()  # warm-up: kernel attributes and lazy module loading happen outside capture
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.launch(s)
        torch.cuda.current_stream(self.device).wait_stream(s)
        self.graph = g
        return self

    def run(self):
        if self.graph is not None:
            self.graph.replay()
        else:
            self.launch()
        return self

    def status(self) -> int:
        """Device status word of the last run (0: ok; 1: a staged copy did not
        land within its bounded wait).  Synchronises the current stream."""
        h = torch.cuda.current_stream(self.device).cuda_stream
        code = _lib.workspace_status(self.ws.data_ptr(), h) if self.ws is not None else 0
        for _, _, _, ws in self._generic:
            code = code or _lib.workspace_status(ws.data_ptr(), h)
        return code

    def results(self) -> List[Dict[str, torch.Tensor]]:
        """Per class: ``final`` cells and, with statistics, leniax's stats dict
        (arrays ``[n, steps, 1]``), ``N``, ``N_box`` and ``mass_centroid``."""
        res = []
        for c, out in zip(self.classes, self.outputs):
            r = {'final': out['final']}
            if self.with_stats:
                st = split_stats(out['stats'][:, :self.steps, None, :], 1)
                st['N'] = out['N'][:, None]
                st['N_box'] = out['N_box'][:, None]
                st['mass_centroid'] = out['centroid'][:, :self.steps, None, :]
                r['stats'] = st
            res.append(r)
        return res


def run_uneven(classes: List[WorldClass], steps: int, tune=True, graph=True, **kw) -> List[Dict]:
    """One-shot helper: build (and optionally autotune and capture) an
    :class:`UnevenBatch`, run it once, return its results."""
    if tune:
        from .autotune import tuned_settings
        kw = {**tuned_settings(classes, steps), **kw}
    b = UnevenBatch(classes, steps, **kw)
    if graph:
        b.capture()
    b.run()
    return b.results()
