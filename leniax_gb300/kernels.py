"""Kernel construction and mapping: the inputs of the Lenia hot path.

Mirror of leniax ``kernels.py`` (``KernelMapping`` 10-63,
``get_kernels_and_mapping`` 66-158, ``circle_2d`` 176-212, ``ellipse_2d`` /
``oriented_ellipse_2d`` 214-311, ``register`` 312-317) and
``kernel_functions.py`` (7-261).  This is the once-per-configuration boundary
preparation (host side, like the reference); the per-step hot path runs in the
CUDA engine.  The spectrum is returned as a CUDA complex64 tensor
``[1, C, max_k, *world]`` exactly as leniax returns it (fftshift then fftn of
the world-centred kernels, kernels.py:145-152).
"""
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from .constant import EPSILON


# ---------------------------------------------------------------- kernel functions
def poly_quad(params, X):
    """kernel_functions.py:7-37"""
    return (4 * X * (1 - X))**params[0]


def gauss_bump(params, X):
    """kernel_functions.py:40-69"""
    q = params[0]
    with np.errstate(over='ignore', under='ignore'):
        return np.exp(q * (q - 1 / (X * (1 - X) + X.dtype.type(EPSILON))))


def step(params, X):
    """kernel_functions.py:72-102"""
    q = params[0]
    return ((X >= q) * (X <= 1 - q)).astype(X.dtype)


def gauss(params, X):
    """kernel_functions.py:105-134"""
    q = params[0]
    out = ((X - q) / (X.dtype.type(0.3) * q))**2
    return np.exp(-out / 2)


def threshold(params, X):
    """kernel_functions.py:137-167"""
    return (X >= params[0]).astype(X.dtype)


def staircase(params, X):
    """kernel_functions.py:170-208"""
    m, s = params[0], params[1]
    out = 0.5 * (X >= m - s) * (X < m - s / 2)
    out = out + 1 * (X >= m - s / 2) * (X <= m + s / 2)
    out = out + 0.5 * (X > m + s / 2) * (X <= m + s)
    return out.astype(X.dtype)


def triangle(params, X):
    """kernel_functions.py:211-250"""
    m, s = params[0], params[1]
    left, right = m - s, m + s
    out = (X >= left) * (X < m) * (X - left) / (m - left)
    out = out + (X >= m) * (X <= right) * (X - right) / (m - right)
    return out.astype(X.dtype)


kf_register = {
    'poly_quad': poly_quad,
    'gauss_bump': gauss_bump,
    'gauss': gauss,
    'step': step,
    'threshold': threshold,
    'staircase': staircase,
    'triangle': triangle,
}


# ---------------------------------------------------------------- kernels
def circle_nd(R, k_params, kf_slug, kf_params, nb_dims=2) -> np.ndarray:
    """Ring kernel of leniax ``circle_2d`` (kernels.py:176-212), float32; for
    ``nb_dims == 3`` the distance runs over the three axes (this engine's
    extension: leniax builds 2D kernels only)."""
    f32 = np.float32
    r = k_params[0]
    bs = np.asarray(k_params[1], dtype=f32)
    k_radius_px = math.ceil(r * R)
    coords = np.indices([k_radius_px * 2] * nb_dims).astype(f32)
    centered = (coords - f32(k_radius_px)) / f32(r * R)
    distances = np.sqrt(np.sum(centered**2, axis=0))
    nb_b = bs.shape[0]
    B_dist = f32(nb_b) * distances
    bs_mat = bs[np.minimum(np.floor(B_dist).astype(np.int64), nb_b - 1)]
    raw_kernel = kf_register[kf_slug](np.asarray(kf_params, dtype=f32), np.mod(B_dist, f32(1)))
    kernel = (distances < 1) * raw_kernel * bs_mat
    kernel = (kernel / kernel.sum()).astype(f32)
    return kernel[np.newaxis]


def circle_2d(R, k_params, kf_slug, kf_params):
    """kernels.py:176-212"""
    return circle_nd(R, k_params, kf_slug, kf_params, 2)


def _ellipse_rings(R, k_params, kf_slug, kf_params):
    """The part leniax's ``ellipse_2d`` and ``oriented_ellipse_2d`` share
    (kernels.py:214-311), float32: ``k_params`` = [r, b, a, b_axis,
    theta / pi]; the grid of ``circle_2d`` rotated by theta, distances on an
    ellipse of semi-axes a and b_axis (in units of r R), rings as in
    ``circle_2d``.  Returns the rotated first coordinate and the
    unnormalised kernel."""
    f32 = np.float32
    r = k_params[0]
    bs = np.asarray(k_params[1], dtype=f32)
    a, b = f32(k_params[2]), f32(k_params[3])
    theta = f32(k_params[4] * math.pi)
    k_radius_px = math.ceil(r * R)
    coords = np.indices([k_radius_px * 2] * 2).astype(f32)
    centered = (coords - f32(k_radius_px)) / f32(r * R)
    cos, sin = np.cos(theta), np.sin(theta)
    rot0 = centered[0] * cos + centered[1] * sin
    rot1 = -centered[0] * sin + centered[1] * cos
    distances = np.sqrt((rot0 / a)**2 + (rot1 / b)**2)
    nb_b = bs.shape[0]
    B_dist = f32(nb_b) * distances
    bs_mat = bs[np.minimum(np.floor(B_dist).astype(np.int64), nb_b - 1)]
    raw_kernel = kf_register[kf_slug](np.asarray(kf_params, dtype=f32), np.mod(B_dist, f32(1)))
    return rot0, (distances < 1) * raw_kernel * bs_mat


def ellipse_2d(R, k_params, kf_slug, kf_params):
    """kernels.py:214-259: the elliptic rings normalised to sum 1, then
    signed by the rotated first coordinate (-1 below -0.01, +1 above 0.01,
    the coordinate itself in between)."""
    rot0, kernel = _ellipse_rings(R, k_params, kf_slug, kf_params)
    kernel = kernel / kernel.sum()
    sign = rot0.copy()
    sign[rot0 < -0.01] = -1
    sign[sign > 0.01] = 1
    return (kernel * sign).astype(np.float32)[np.newaxis]


def oriented_ellipse_2d(R, k_params, kf_slug, kf_params):
    """kernels.py:262-307: the elliptic rings times the rotated first
    coordinate, normalised to an absolute sum of 1."""
    rot0, kernel = _ellipse_rings(R, k_params, kf_slug, kf_params)
    kernel = kernel * rot0
    return (kernel / np.abs(kernel).sum()).astype(np.float32)[np.newaxis]


def raw(R, k_params, kf_slug, kf_params):
    """kernels.py:161-173"""
    return np.asarray(k_params, dtype=np.float32)


register = {'raw': raw, 'circle_2d': circle_2d, 'ellipse_2d': ellipse_2d, 'oriented_ellipse_2d': oriented_ellipse_2d}


class KernelMapping:
    """kernels.py:10-63: explicit description of the kernel graph."""

    def __init__(self, nb_channels: int, nb_kernels: int):
        self.cin_kernels: List[List[int]] = [[] for _ in range(nb_channels)]
        self.cin_k_params: List[List] = [[] for _ in range(nb_channels)]
        self.cin_kfs: List[List[str]] = [[] for _ in range(nb_channels)]
        self.cin_gfs: List[List[str]] = [[] for _ in range(nb_channels)]
        self.cin_gf_params: List[List] = [[] for _ in range(nb_channels)]
        self.kernels_weight_per_channel = [[0.] * nb_kernels for _ in range(nb_channels)]
        self.true_channels: Optional[List[bool]] = None

    def get_k_params(self):
        return [item for sub in self.cin_k_params for item in sub]

    def get_gf_params(self, device=None) -> torch.Tensor:
        flat = [item for sub in self.cin_gf_params for item in sub]
        return torch.tensor(flat, dtype=torch.float32, device=device)

    def get_kernels_weight_per_channel(self, device=None) -> torch.Tensor:
        return torch.tensor(self.kernels_weight_per_channel, dtype=torch.float32, device=device)

    # engine view -------------------------------------------------------------
    def kernel_table(self) -> Tuple[List[int], List[int], List[str], int]:
        """(c_in, slot, growth slug) of every true kernel in leniax's flattened
        order, and max_k (kernels.py:122-143; helpers.py:452-458)."""
        max_k = max(map(len, self.cin_kernels))
        cin, slot, gfs = [], [], []
        for c, (lst, gl) in enumerate(zip(self.cin_kernels, self.cin_gfs)):
            for j, _ in enumerate(lst):
                cin.append(c)
                slot.append(j)
                gfs.append(gl[j])
        return cin, slot, gfs, max_k


def crop_zero(kernels: np.ndarray) -> np.ndarray:
    """utils.py:296-317: drop every index of each world axis at which all
    kernels are zero (the masks are taken on the uncropped array)."""
    nz = kernels != 0
    keep = []
    for ax in range(1, kernels.ndim):
        others = tuple(a for a in range(kernels.ndim) if a != ax)
        keep.append(np.nonzero(np.any(nz, axis=others))[0])
    return kernels[np.ix_(np.arange(kernels.shape[0]), *keep)]


def get_kernels_and_mapping(kernels_params: List[Dict], world_size: Sequence[int], nb_channels: int, R: float,
                            fft: bool = True, device=None) -> Tuple[torch.Tensor, KernelMapping]:
    """kernels.py:66-158.  Returns the spectrum ``[1, C, max_k, *world]``
    complex64 (``fft=True``), or the cropped real kernels ``[C*max_k, 1,
    *kernel_dims]`` of the direct-convolution path (``fft=False``), on
    ``device`` (default: current CUDA device)."""
    if device is None:
        device = torch.device('cuda', torch.cuda.current_device()) if torch.cuda.is_available() else 'cpu'
    nb_dims = len(world_size)
    kernels_params.sort(key=lambda d: d['c_in'])  # kernels.py:90 (stable, in place as in leniax)
    mapping = KernelMapping(nb_channels, len(kernels_params))
    padded = []
    for kernel_idx, p in enumerate(kernels_params):
        slug = p.get('k_slug', 'circle_2d')
        if slug == 'circle_2d':
            k = circle_nd(R, p['k_params'], p['kf_slug'], p['kf_params'], nb_dims)
        else:
            k = register[slug](R, p['k_params'], p['kf_slug'], p['kf_params'])
        pads = [(0, 0)]
        for ws, ks in zip(world_size, k.shape[1:]):
            need = ws - ks
            pads.append(((need // 2), need // 2 + (need % 2)))
        padded.append(np.pad(k, pads))
        c_in = p['c_in']
        mapping.cin_kernels[c_in].append(kernel_idx)
        mapping.cin_gfs[c_in].append(p['gf_slug'])
        mapping.cin_gf_params[c_in].append(p['gf_params'])
        mapping.cin_kfs[c_in].append(p['kf_slug'])
        mapping.cin_k_params[c_in].append(p['k_params'])
        mapping.kernels_weight_per_channel[p['c_out']][kernel_idx] = p['h']
    kernels = np.concatenate(padded, axis=0).astype(np.float32)
    if not fft:
        kernels = crop_zero(kernels)  # kernels.py:118-119
    kshape = kernels.shape[1:]
    max_k = max(map(len, mapping.cin_kernels))
    per_channel, true_channels = [], []
    for lst in mapping.cin_kernels:
        K_tmp = kernels[np.array(lst, dtype=np.int64)] if lst else np.zeros((0, ) + kshape, np.float32)
        missing = max_k - K_tmp.shape[0]
        true_channels += [True] * K_tmp.shape[0] + [False] * missing
        if missing:
            K_tmp = np.concatenate([K_tmp, np.zeros((missing, ) + kshape, np.float32)])
        per_channel.append(K_tmp)
    mapping.true_channels = None if all(true_channels) else true_channels
    if not fft:
        return torch.from_numpy(np.concatenate(per_channel)[:, np.newaxis]).to(device), mapping
    axes = tuple(range(-1, -nb_dims - 1, -1))
    K = np.stack(per_channel)[np.newaxis]  # [1, C, max_k, *ws]
    K = np.fft.fftshift(K, axes=axes)
    K = np.fft.fftn(K.astype(np.complex64), axes=axes).astype(np.complex64)
    return torch.from_numpy(np.ascontiguousarray(K)).to(device), mapping


# ---------------------------------------------------------------- device builder
KF_IDS = {'poly_quad': 0, 'gauss_bump': 1, 'step': 2, 'gauss': 3, 'threshold': 4, 'staircase': 5, 'triangle': 6}


class RingBatchC:
    """ctypes mirror of ``lgx_ring_batch`` (built lazily with the library)."""
    _cls = None

    @classmethod
    def get(cls):
        if cls._cls is None:
            import ctypes

            class _C(ctypes.Structure):
                _fields_ = [('nb_dims', ctypes.c_int), ('size', ctypes.c_int), ('n', ctypes.c_int),
                            ('kf_id', ctypes.c_int), ('nb_max', ctypes.c_int), ('R', ctypes.c_void_p),
                            ('r', ctypes.c_void_p), ('b', ctypes.c_void_p), ('nb', ctypes.c_void_p),
                            ('kf_params', ctypes.c_void_p), ('kernel_out', ctypes.c_void_p),
                            ('k_half', ctypes.c_void_p), ('status', ctypes.c_void_p)]

            cls._cls = _C
        return cls._cls


def ring_kernels(world: Sequence[int], R, r, b, kf_slug: str, kf_params, spectrum: bool = True, device=None):
    """Ring kernels of ``circle_2d`` (kernels.py:176-212) built on the GPU for
    a batch of worlds, each with its own radius ``R[i]``, relative radius
    ``r[i]``, ring weights ``b[i]`` (list) and kernel-function parameters
    ``kf_params[i]``; placed and fftshifted on the world grid as
    ``get_kernels_and_mapping`` does.  Returns ``(kernels [n, *world] float32,
    K_half [n, *world[:-1], W//2+1] complex64 or None)``.  Square 2D and
    cubic 3D worlds of any side the N-D engine takes (odd and prime sides
    included: fftshift rolls by side // 2)."""
    import ctypes
    from . import _lib
    world = [int(w) for w in world]
    n = len(R)
    if device is None:
        device = torch.device('cuda', torch.cuda.current_device())
    if kf_slug not in KF_IDS:
        raise ValueError(f'unknown kernel function slug {kf_slug!r}')
    if len(set(world)) != 1:
        raise ValueError(f'world {world} must be square / cubic')
    rr = [float(x) for x in (r if hasattr(r, '__len__') else [r] * n)]
    bl = [list(map(float, x)) for x in b]
    if len(bl) == 1 and n > 1:
        bl = bl * n
    nb_max = max(len(x) for x in bl)
    bm = np.zeros((n, nb_max), np.float32)
    for i, x in enumerate(bl):
        bm[i, :len(x)] = x
    kfp = np.zeros((n, 2), np.float32)
    kf_rows = kf_params if (len(kf_params) == n and hasattr(kf_params[0], '__len__')) else [kf_params] * n
    for i, x in enumerate(kf_rows):
        x = list(x)
        kfp[i, :len(x)] = x
    t = lambda a, dt=torch.float32: torch.as_tensor(np.asarray(a), dtype=dt).to(device)
    Rt, rt, bt = t(np.asarray(R, np.float32)), t(np.asarray(rr, np.float32)), t(bm)
    nbt, kft = t(np.array([len(x) for x in bl], np.int32), torch.int32), t(kfp)
    out = torch.empty([n] + world, dtype=torch.float32, device=device)
    kh = torch.empty([n] + world[:-1] + [world[-1] // 2 + 1], dtype=torch.complex64, device=device) if spectrum else None
    status = torch.zeros(1, dtype=torch.int32, device=device)
    job = RingBatchC.get()()
    job.nb_dims, job.size, job.n, job.kf_id, job.nb_max = len(world), world[0], n, KF_IDS[kf_slug], nb_max
    job.R, job.r, job.b, job.nb, job.kf_params = (x.data_ptr() for x in (Rt, rt, bt, nbt, kft))
    job.kernel_out = out.data_ptr()
    job.k_half = kh.data_ptr() if kh is not None else None
    job.status = status.data_ptr()
    lib = _lib.load()
    if not getattr(lib, '_lgx_ring_bound', False):
        lib.lgx_ring_kernels_workspace_bytes.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]
        lib.lgx_ring_kernels_workspace_bytes.restype = ctypes.c_int
        lib.lgx_ring_kernels.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
        lib.lgx_ring_kernels.restype = ctypes.c_int
        lib._lgx_ring_bound = True
    nbytes = ctypes.c_size_t(0)
    _lib.check(lib.lgx_ring_kernels_workspace_bytes(ctypes.byref(job), ctypes.byref(nbytes)))
    ws = torch.empty(max(int(nbytes.value), 256), dtype=torch.uint8, device=device)
    _lib.check(lib.lgx_ring_kernels(ctypes.byref(job), ws.data_ptr(), ws.numel(),
                                    torch.cuda.current_stream(device).cuda_stream))
    if int(status.item()) != 0:
        raise ValueError('a kernel box (2*ceil(r*R) cells) exceeds the world, or a ring list is empty')
    return out, kh
