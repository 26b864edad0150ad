"""State utilities of leniax ``utils.py`` used around the path: rolling a
world onto its mass centroid and cropping it (``center_world`` 270-293,
``auto_center`` 320-349, ``center_and_crop`` 352-385), what the reference
applies to a found creature before encoding it (``qd.py:422``).  Torch ops
on the state's own device; ``crop_zero`` is the kernel builder's
(``utils.py:296-317``)."""
from typing import Sequence, Tuple

import torch

from .constant import EPSILON
from .kernels import crop_zero as _crop_zero_np


def center_world(cells: torch.Tensor, field: torch.Tensor, potential: torch.Tensor, shift_idx,
                 axes: Sequence[int]) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """utils.py:270-293: every entry ``b`` of the batch axis rolled by
    ``-shift_idx[b]`` (``[bs, len(axes)]``) over ``axes``."""
    shift = torch.as_tensor(shift_idx).reshape(len(cells), len(axes)).tolist()
    axes = tuple(int(a) for a in axes)

    def roll(t):
        return torch.stack([torch.roll(t[b], [-int(s) for s in shift[b]], [a - 1 if a > 0 else a for a in axes])
                            for b in range(len(t))])

    return roll(cells), roll(field), roll(potential)


def crop_zero(cells: torch.Tensor) -> torch.Tensor:
    """utils.py:296-317 on ``[C, *world]``: every index of a world axis at
    which all channels are zero is dropped."""
    return torch.from_numpy(_crop_zero_np(cells.detach().cpu().numpy())).to(cells.device)


def _mass_shift(cells: torch.Tensor) -> torch.Tensor:
    """round(mass centroid relative to the world's midpoint), per world axis."""
    world = cells.shape[1:]
    coords = torch.stack(torch.meshgrid(*[torch.arange(n, device=cells.device, dtype=torch.float32) - (n // 2)
                                          for n in world], indexing='ij'))
    m00 = cells.sum()
    centroid = torch.stack([(cells * c).sum() for c in coords]) / (m00 + EPSILON)
    return torch.round(centroid).to(torch.int64)


def auto_center(cells: torch.Tensor) -> torch.Tensor:
    """utils.py:320-349: ``cells`` ``[C, *world]`` rolled so that the total
    mass centroid (rounded, half to even) sits at the world's midpoint
    ``size // 2``."""
    axes = tuple(range(-(cells.dim() - 1), 0))
    shift = _mass_shift(cells)
    return center_world(cells[None], cells[None], cells[None], shift[None], axes)[0][0]


def center_and_crop(cells: torch.Tensor) -> torch.Tensor:
    """utils.py:352-385: a pattern cut by a world border (occupied indices at
    both ends of an axis, empty ones in between) is first rolled by half the
    world (the first axis's ``size // 2`` for every axis, as the
    reference), then the state is centred on its mass (:func:`auto_center`)
    and cropped to its support (:func:`crop_zero`); an empty state gives
    zeros ``[C, 1, ...]``."""
    world = cells.shape[1:]
    nd = len(world)
    axes = tuple(range(-nd, 0))
    pre = [0] * nd
    for i in range(nd):
        occupied = (cells != 0).movedim(i + 1, 0).reshape(world[i], -1).any(dim=1)
        if bool(occupied[0]) and bool(occupied[-1]) and not bool(occupied.all()):
            pre[i] = int(world[0] // 2)
    cells = center_world(cells[None], cells[None], cells[None], torch.tensor([pre]), axes)[0][0]
    cells = crop_zero(auto_center(cells))
    if 0 in cells.shape:
        cells = torch.zeros([cells.shape[0]] + [1] * (cells.dim() - 1), dtype=cells.dtype, device=cells.device)
    return cells


__all__ = ['center_world', 'crop_zero', 'auto_center', 'center_and_crop']
