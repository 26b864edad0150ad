"""Cell-state codec: the on-disk string format of found creatures.

Mirror of leniax ``loader.py`` (``make_array_compressible`` 16-30,
``compress_array`` 33-66, ``decompress_array`` 69-102,
``decompress_array_gzip`` 105-129, ``ch2val`` / ``val2ch`` 147-203).
A state is quantised to int32 on the ``NB_CHARS**2 - 1`` grid, laid out as
``[count][values][shape]`` little-endian int32 words, gzip-compressed and
base64-encoded.

GB300 split: the quantisation of a whole batch of states runs on the device
with one copy of the int32 words to the host; the byte work (gzip, base64) is
host work by nature and runs on a thread pool (zlib releases the GIL).
The pickle / npz fallbacks of ``decompress_array`` are not supported:
unpickling untrusted strings executes code.
"""
import base64
import codecs
import gzip
from concurrent.futures import ThreadPoolExecutor
from typing import List

import numpy as np
import torch

from .constant import NB_CHARS
from .initializations import make_array_compressible  # noqa: F401  (loader.py:16-30)

MAX_VAL = NB_CHARS**2 - 1


def _quantise(cells: torch.Tensor) -> torch.Tensor:
    return torch.round(cells.to(torch.float32) * MAX_VAL).to(torch.int32)


def _pack(q: np.ndarray) -> str:
    shape = b''.join(int(s).to_bytes(4, 'little') for s in q.shape)
    flat = np.ascontiguousarray(q.reshape(-1), dtype='<i4')
    raw = len(flat).to_bytes(4, 'little') + flat.tobytes() + shape
    return str(codecs.encode(gzip.compress(raw), 'base64'), 'utf-8')


def compress_array(cells) -> str:
    """loader.py:33-66: one state -> base64(gzip([n][int32 values][shape]))."""
    t = cells if isinstance(cells, torch.Tensor) else torch.as_tensor(np.asarray(cells))
    return _pack(_quantise(t).cpu().numpy())


def compress_batch(cells: torch.Tensor, workers: int = 8) -> List[str]:
    """``compress_array`` of every ``cells[i]``: one device quantisation and
    one host copy for the batch, gzip on ``workers`` threads."""
    q = _quantise(cells).cpu().numpy()
    with ThreadPoolExecutor(max_workers=max(1, workers)) as ex:
        return list(ex.map(_pack, [q[i] for i in range(q.shape[0])]))


def decompress_array_gzip(string_cells: str, device=None) -> torch.Tensor:
    """loader.py:105-129"""
    raw = gzip.decompress(base64.decodebytes(string_cells.encode('utf-8')))
    n = int.from_bytes(raw[0:4], 'little')
    vals = np.frombuffer(raw[4:4 + 4 * n], dtype='<i4')
    shape = [int.from_bytes(raw[i:i + 4], 'little') for i in range(4 + 4 * n, len(raw), 4)]
    t = torch.from_numpy(vals.astype(np.int32).reshape(shape))
    if device is not None:
        t = t.to(device)
    return (t / MAX_VAL).to(torch.float32)


def ch2val(c: str) -> int:
    """loader.py:147-174: two characters -> integer in [0, NB_CHARS**2)."""
    assert len(c) == 2

    def idx(ch):
        if ord(ch) >= ord('À'):
            return ord(ch) - ord('À') + (ord('Z') - ord('A')) + (ord('z') - ord('a'))
        if ord(ch) >= ord('a'):
            return ord(ch) - ord('a') + (ord('Z') - ord('A'))
        return ord(ch) - ord('A')

    return idx(c[0]) * NB_CHARS + idx(c[1])


def val2ch(v: int) -> str:
    """loader.py:177-203: integer -> two characters."""

    def ch(i):
        if ord('A') + i <= ord('Z'):
            return chr(ord('A') + i)
        if ord('a') + i - (ord('Z') - ord('A')) <= ord('z'):
            return chr(ord('a') + i - (ord('Z') - ord('A')))
        return chr(ord('À') + i - (ord('Z') - ord('A')) - (ord('z') - ord('a')))

    return ch(v // NB_CHARS) + ch(v % NB_CHARS)


def decompress_array(string_cells: str, nb_dims: int = 0, device=None) -> torch.Tensor:
    """loader.py:69-102: the gzip codec, then the two-character codec
    ``'<chars>::<d0;d1;...>'``."""
    try:
        return decompress_array_gzip(string_cells, device)
    except Exception:
        parts = string_cells.split('::')
        if len(parts) != 2 or len(parts[0]) % 2 != 0:
            raise ValueError('unsupported cell encoding (gzip and two-character codecs only)')
        shape = [int(c) for c in parts[-1].split(';')]
        vals = [ch2val(parts[0][i:i + 2]) for i in range(0, len(parts[0]), 2)]
        t = torch.tensor(vals, dtype=torch.int32).reshape(shape)
        if device is not None:
            t = t.to(device)
        return (t / MAX_VAL).to(torch.float32)
