"""Cell-state codec: the on-disk string format of found creatures.

Mirror of leniax ``loader.py`` (``make_array_compressible`` 16-30,
``compress_array`` 33-66, ``decompress_array`` 69-102,
``decompress_array_gzip`` 105-129, ``ch2val`` / ``val2ch`` 147-203,
``load_raw_cells`` 206-241, the run-length codec of the classic species
strings 246-350).
A state is quantised to int32 on the ``NB_CHARS**2 - 1`` grid, laid out as
``[count][values][shape]`` little-endian int32 words, gzip-compressed and
base64-encoded.

GB300 split: the quantisation of a whole batch of states runs on the device
with one copy of the int32 words to the host; the byte work (gzip, base64) is
host work by nature and runs on a thread pool (zlib releases the GIL).
``decompress_array`` tries the gzip codec, the two-character codec, an npz
archive (read without pickles) and the run-length codec; the base64-pickle
fallback is not supported (unpickling an untrusted string executes code), and
``last_frame.p`` files are read with an unpickler that admits numpy arrays
only.
"""
import base64
import codecs
import gzip
import io
import os
import pickle
from concurrent.futures import ThreadPoolExecutor
from typing import Dict, List

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


def _npz_decode(string_cells: str) -> np.ndarray:
    """An npz archive (latin-1 string) holding ``x`` as uint8, scaled to
    [0, 1] (loader.py:90-93); numpy reads it without pickles."""
    with np.load(io.BytesIO(string_cells.encode('latin1')), allow_pickle=False) as z:
        return z['x'] / 255.


def decompress_array(string_cells: str, nb_dims: int = 0, device=None) -> torch.Tensor:
    """loader.py:69-102: the gzip codec, the two-character codec
    ``'<chars>::<d0;d1;...>'``, an npz archive, then the run-length codec
    (``nb_dims`` axes, channel axis included)."""
    try:
        return decompress_array_gzip(string_cells, device)
    except Exception:
        pass
    parts = string_cells.split('::')
    if len(parts) == 2 and len(parts[0]) % 2 == 0:
        try:
            shape = [int(c) for c in parts[-1].split(';')]
            vals = [ch2val(parts[0][i:i + 2]) for i in range(0, len(parts[0]), 2)]
            t = torch.tensor(vals, dtype=torch.int32).reshape(shape)
            if device is not None:
                t = t.to(device)
            return (t / MAX_VAL).to(torch.float32)
        except Exception:
            pass
    try:
        arr = _npz_decode(string_cells)
    except Exception:
        arr = deprecated_decompress_array(string_cells, nb_dims)
    t = torch.from_numpy(np.asarray(arr, dtype=np.float32))
    return t.to(device) if device is not None else t


# ---------------------------------------------------------------- run-length codec
# Dimension delimiters of the run-length codec (loader.py:246): after the
# cells of a row, '$' closes the row, '%' a plane, '#' a volume, '@A'.. '@F'
# the higher blocks; a decimal count before a symbol repeats it.
RLE_DELIMS = ('', '$', '%', '#', '@A', '@B', '@C', '@D', '@E', '@F')


def rle_value(sym: str) -> int:
    """The 0..255 value of a run-length symbol (loader.py:287-296): '.' and
    'b' 0, 'o' 255, 'A'..'X' 1..24, two characters 'p'..'y' x 'A'..'X' from
    25 on."""
    if sym in ('.', 'b'):
        return 0
    if sym == 'o':
        return 255
    if len(sym) == 1:
        return ord(sym) - ord('A') + 1
    return 25 + 24 * (ord(sym[0]) - ord('p')) + ord(sym[1]) - ord('A')


def rle_symbol(v: int) -> str:
    """The run-length symbol of a 0..255 value (loader.py:298-304)."""
    if v == 0:
        return '.'
    if v < 25:
        return chr(ord('A') + v - 1)
    q, r = divmod(v - 25, 24)
    return chr(ord('p') + q) + chr(ord('A') + r)


# leniax's names of the two symbol helpers (loader.py:287-304)
char2val_deprecated = rle_value
val2char_deprecated = rle_symbol


def deprecated_compress_array(cells) -> str:
    """loader.py:307-320: values rounded to 0..255, runs of equal values per
    row as ``[count]symbol`` (count left out when 1), rows and blocks joined
    by their delimiters, ``'!'`` at the end."""
    q = np.rint(np.asarray(cells) * 255).astype(np.int64)

    def encode(a):
        if a.ndim == 1:
            out, i = [], 0
            while i < len(a):
                j = i
                while j < len(a) and a[j] == a[i]:
                    j += 1
                out.append((str(j - i) if j - i > 1 else '') + rle_symbol(int(a[i])))
                i = j
            return ''.join(out)
        return RLE_DELIMS[a.ndim - 1].join(encode(sub) for sub in a)

    return encode(q) + '!'


def deprecated_decompress_array(cells_code: str, nb_dims: int) -> np.ndarray:
    """loader.py:323-350: an ``nb_dims``-axis array from a run-length code.

    A value symbol with count n adds n cells to the open row; a delimiter of
    rank d with count n closes the open blocks of every rank below d, each
    followed by n - 1 empty ones.  Short rows and blocks are padded with
    zeros to the longest (float32, values / 255)."""
    if nb_dims < 1:
        raise ValueError('the run-length codec needs the number of axes (channel axis included)')
    open_blocks: List[list] = [[] for _ in range(nb_dims)]  # [0]: the open row; [r]: the open rank-r block
    count, prefix = '', ''
    for ch in cells_code.rstrip('!') + RLE_DELIMS[nb_dims - 1]:
        if ch.isdigit():
            count += ch
            continue
        if ch in 'pqrstuvwxy@':
            prefix = ch
            continue
        sym, prefix = prefix + ch, ''
        reps, count = (int(count) if count else 1), ''
        if sym in RLE_DELIMS:
            for r in range(RLE_DELIMS.index(sym)):
                open_blocks[r + 1].append(open_blocks[r])
                open_blocks[r + 1].extend([] for _ in range(reps - 1))
                open_blocks[r] = []
        else:
            open_blocks[0].extend([rle_value(sym) / 255] * reps)
    top = open_blocks[nb_dims - 1]
    lens = [0] * nb_dims

    def measure(node, depth):
        lens[depth] = max(lens[depth], len(node))
        if depth < nb_dims - 1:
            for sub in node:
                measure(sub, depth + 1)

    measure(top, 0)
    out = np.zeros(lens, dtype=np.float64)

    def place(node, index):
        if len(index) == nb_dims - 1:
            out[index + (slice(0, len(node)), )] = node
        else:
            for i, sub in enumerate(node):
                place(sub, index + (i, ))

    place(top, ())
    return out.astype(np.float32)


# ---------------------------------------------------------------- configurations
class _NumpyOnlyUnpickler(pickle.Unpickler):
    """Unpickles numpy arrays and nothing else (a saved ``last_frame.p``)."""
    ALLOWED = {('numpy', 'ndarray'), ('numpy', 'dtype'), ('numpy.core.multiarray', '_reconstruct'),
               ('numpy._core.multiarray', '_reconstruct'), ('numpy.core.multiarray', 'scalar'),
               ('numpy._core.multiarray', 'scalar')}

    def find_class(self, module, name):
        if (module, name) in self.ALLOWED:
            return super().find_class(module, name)
        raise pickle.UnpicklingError(f'refused to unpickle {module}.{name}: numpy arrays only')


def load_raw_cells(config: Dict, use_init_cells: bool = True, device=None) -> torch.Tensor:
    """loader.py:206-241: the cells of a leniax configuration
    (``run_params['init_cells']``, or ``['cells']``): an encoded string
    (:func:`decompress_array` with the channel axis), ``'MISSING'`` (empty),
    ``'last_frame.p'`` beside the configuration (``config['main_path']``), or
    nested lists; a single channel squeezed out is put back."""
    nb_dims = config['world_params']['nb_dims']
    rp = config['run_params']
    cells = rp.get('init_cells', rp.get('cells')) if use_init_cells else rp['cells']
    if isinstance(cells, str):
        if cells == 'MISSING':
            t = torch.zeros((0, ), dtype=torch.float32)
        elif cells == 'last_frame.p':
            with open(os.path.join(config['main_path'], 'last_frame.p'), 'rb') as f:
                t = torch.from_numpy(np.asarray(_NumpyOnlyUnpickler(f).load(), dtype=np.float32))
        else:
            t = decompress_array(cells, nb_dims + 1)
    else:
        t = torch.as_tensor(np.asarray(cells, dtype=np.float32))
    if t.dim() == nb_dims and config['world_params']['nb_channels'] == 1:
        t = t[None]
    return t.to(device) if device is not None else t
