"""Growth functions and their plugin registry (leniax ``growth_functions.py``).

Each function has leniax's signature ``fn(params, X)`` (``params`` = ``[m,
s]``, ``X`` any CUDA float32 tensor) and runs on the device through
``lgx_growth``; ``register`` maps the reference's slugs to them
(growth_functions.py:256-264).  The formulas, in the reference's op order,
are in ``csrc/common.cuh`` (``growth_fn``); ``fn.id`` is the engine's
function id (``LGX_GF_*`` in ``include/lenia_gb300.h``), which is what the
engine's models and ``core.get_field`` use.
"""
import ctypes

import torch

from . import _lib
from ._lib import GF_IDS


class GrowthFn:
    """One growth function of the engine, callable as ``fn(params, X)``."""

    def __init__(self, slug: str):
        self.slug = slug
        self.id = GF_IDS[slug]
        self.__name__ = slug

    def __call__(self, params, X: torch.Tensor) -> torch.Tensor:
        if not (isinstance(X, torch.Tensor) and X.is_cuda and X.dtype == torch.float32):
            raise TypeError('X must be a float32 CUDA tensor: the engine has no CPU path')
        dev = X.device
        p = torch.as_tensor(params, dtype=torch.float32, device=dev).reshape(-1)[:2].contiguous()
        if p.numel() != 2:
            raise ValueError('growth parameters are [m, s]')
        x = X.contiguous()
        out = torch.empty_like(x)
        if x.numel() == 0:
            return out
        ids = (ctypes.c_int * 1)(self.id)
        lib = _lib.load()
        _lib.check(lib.lgx_growth(1, 1, x.numel(), ids, x.data_ptr(), p.data_ptr(), out.data_ptr(),
                                  torch.cuda.current_stream(dev).cuda_stream))
        return out

    def __repr__(self):
        return f'growth_functions.{self.slug}'


poly_quad4 = GrowthFn('poly_quad4')
gaussian = GrowthFn('gaussian')
gaussian_target = GrowthFn('gaussian_target')
step = GrowthFn('step')
staircase = GrowthFn('staircase')
triangle = GrowthFn('triangle')
identity = GrowthFn('identity')

register = {fn.slug: fn for fn in (poly_quad4, gaussian, gaussian_target, step, staircase, triangle, identity)}


def engine_id(fn) -> int:
    """Engine id of a growth function given as a registered function, a slug
    or an id."""
    if isinstance(fn, GrowthFn):
        return fn.id
    if isinstance(fn, str):
        return GF_IDS[fn]
    if isinstance(fn, int) and fn in GF_IDS.values():
        return fn
    raise ValueError(f'{fn!r} is not one of the engine growth functions {sorted(GF_IDS)}')
