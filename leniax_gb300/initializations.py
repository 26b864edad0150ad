"""Initial states generated on the GPU.

Mirror of leniax ``initializations.py`` (``random_uniform`` 10-32,
``perlin`` 35-77, ``cropped_perlin`` 80-116, ``register`` 119-123) and
``loader.make_array_compressible`` (loader.py:16-30), run by the engine's
``lgx_init_cells`` kernels for whole batches of worlds at once.

leniax threads a JAX PRNG key through these functions; here a key is a
64-bit integer seed.  The numbers come from a counter-based SplitMix64 hash of
(seed, stream, index): the same constructions and distributions as leniax,
not JAX's threefry stream (``next_key`` plays the role of ``jax.random.split``).
"""
import ctypes
import math
from typing import List, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from .constant import NB_CHARS

KINDS = {'random_uniform': 0, 'perlin': 1, 'cropped_perlin': 2}
_MASK64 = (1 << 64) - 1


class InitJobC(ctypes.Structure):
    _fields_ = [('kind', ctypes.c_int), ('n_worlds', ctypes.c_int), ('nb_init', ctypes.c_int), ('H', ctypes.c_int),
                ('W', ctypes.c_int), ('R', ctypes.c_float), ('compressible', ctypes.c_int), ('seeds', ctypes.c_void_p),
                ('gf_m', ctypes.c_void_p), ('out', ctypes.c_void_p), ('angles', ctypes.c_void_p)]


def _bind(lib):
    if not getattr(lib, '_lgx_init_bound', False):
        lib.lgx_init_cells_workspace_bytes.argtypes = [ctypes.POINTER(InitJobC), ctypes.POINTER(ctypes.c_size_t)]
        lib.lgx_init_cells_workspace_bytes.restype = ctypes.c_int
        lib.lgx_init_cells.argtypes = [ctypes.POINTER(InitJobC), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
        lib.lgx_init_cells.restype = ctypes.c_int
        lib._lgx_init_bound = True
    return lib


def next_key(seed: int) -> int:
    """SplitMix64 step: the seed handed back to the caller after a draw."""
    z = (int(seed) + 0x9E3779B97F4A7C15) & _MASK64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK64
    return z ^ (z >> 31)


def perlin_res(world_size: Sequence[int], R: float) -> Tuple[int, int]:
    """Perlin periods of a world (initializations.py:57-58)."""
    kr = math.ceil(R)
    return int(world_size[0]) // (kr * 3), int(world_size[1]) // (kr * 2)


def generate(kind: str, seeds: Sequence[int], nb_init: int, world_size: Sequence[int], R: float,
             gf_m: Sequence[float] = None, compressible: bool = True, device=None,
             angles: torch.Tensor = None) -> torch.Tensor:
    """``[len(seeds), nb_init, H, W]`` float32 initial states on the GPU, one
    block of ``nb_init`` states per seed.  ``gf_m`` (the m of each world's
    first kernel) sets the Perlin scaling.  ``angles`` ``[len(seeds), nb_init,
    *perlin_res(world_size, R)]`` (radians) supplies the Perlin gradient field
    as leniax's ``generate_perlin_noise_2d`` takes it (perlin.py:16-71);
    without it the angles are drawn from the seeds."""
    if kind not in KINDS:
        raise ValueError(f'unknown initialisation {kind!r}')
    if len(world_size) != 2:
        raise ValueError('initial-state generators are 2D')
    if device is None:
        device = torch.device('cuda', torch.cuda.current_device())
    n = len(seeds)
    H, W = int(world_size[0]), int(world_size[1])
    # 64-bit seeds passed bit for bit (two's complement in an int64 tensor)
    sd = torch.tensor([(int(s) & _MASK64) - (1 << 64) if (int(s) & _MASK64) >> 63 else int(s) & _MASK64 for s in seeds],
                      dtype=torch.int64, device=device)
    gm = torch.tensor(list(gf_m) if gf_m is not None else [0.0] * n, dtype=torch.float32, device=device)
    out = torch.empty((n, nb_init, H, W), dtype=torch.float32, device=device)
    job = InitJobC()
    job.kind, job.n_worlds, job.nb_init, job.H, job.W = KINDS[kind], n, int(nb_init), H, W
    job.R, job.compressible = float(R), int(bool(compressible))
    job.seeds, job.gf_m, job.out = sd.data_ptr(), gm.data_ptr(), out.data_ptr()
    if angles is not None:
        if kind == 'random_uniform':
            raise ValueError('angles apply to the Perlin initialisations')
        want = (n, int(nb_init)) + perlin_res(world_size, R)
        if tuple(angles.shape) != want:
            raise ValueError(f'angles has shape {tuple(angles.shape)}, expected {want}')
        angles = angles.to(device=device, dtype=torch.float32).contiguous()
        job.angles = angles.data_ptr()
    lib = _bind(_lib.load())
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.lgx_init_cells_workspace_bytes(ctypes.byref(job), ctypes.byref(nbytes)))
    ws = torch.empty(max(int(nbytes.value), 256), dtype=torch.uint8, device=device)
    _lib.check(lib.lgx_init_cells(ctypes.byref(job), ws.data_ptr(), ws.numel(),
                                  torch.cuda.current_stream(device).cuda_stream))
    return out


def random_uniform(rng_key: int, nb_init: int, world_size: List[int], R: float,
                   gf_params: List) -> Tuple[int, torch.Tensor]:
    """initializations.py:10-32: ``[nb_init, *world]`` uniform in
    ``[0, linspace(0.4, 1, nb_init)[i])``, made compressible."""
    cells = generate('random_uniform', [next_key(rng_key)], nb_init, world_size, R)[0]
    return next_key(next_key(rng_key)), cells


def perlin(rng_key: int, nb_init: int, world_size: List[int], R: float, gf_params: List) -> Tuple[int, torch.Tensor]:
    """initializations.py:35-77: ``[nb_init, 1, *world]`` Perlin noise with
    periods ``(H // (3 ceil R), W // (2 ceil R))``, normalised to [0, 1] and
    scaled by ``m + i / nb_init * (min(1, 3 m) - m)``."""
    cells = generate('perlin', [next_key(rng_key)], nb_init, world_size, R, [gf_params[0]])[0]
    return next_key(next_key(rng_key)), cells[:, None]


def cropped_perlin(rng_key: int, nb_init: int, world_size: List[int], R: float,
                   gf_params: List) -> Tuple[int, torch.Tensor]:
    """initializations.py:80-116: the Perlin state's ``2 ceil(R)`` square at
    rows / columns ``[24, 24 + 2 ceil(R))`` centred on a zero 128 x 128 world."""
    cells = generate('cropped_perlin', [next_key(rng_key)], nb_init, world_size, R, [gf_params[0]])[0]
    return next_key(next_key(rng_key)), cells[:, None]


register = {'random_uniform': random_uniform, 'perlin': perlin, 'cropped_perlin': cropped_perlin}


def make_array_compressible(cells: torch.Tensor) -> torch.Tensor:
    """loader.py:16-30: round to the ``NB_CHARS**2 - 1`` grid (half to even);
    a tensor or an array in, a float32 tensor out."""
    max_val = NB_CHARS**2 - 1
    t = cells if isinstance(cells, torch.Tensor) else torch.as_tensor(np.asarray(cells))
    return (torch.round(t * max_val).to(torch.int32) / max_val).to(torch.float32)
