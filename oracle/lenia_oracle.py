"""CPU oracle for the Lenia hot path (numpy) -- TEST INFRASTRUCTURE ONLY.

This module restates, in plain numpy, the arithmetic of leniax's Lenia step and
scan drivers.  It is the checker of the CUDA engine in ``leniax_gb300``: only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import it.  The product path never calls it and has no CPU fallback.

leniax itself is JAX code (``jax>=0.3.4``/``jaxlib>=0.3.2``, pinned in the
reference ``setup.py:13-21``); neither is installed here, so the published
algorithms behind its call sites (``jnp.fft.fftn``/``ifftn``, ``jnp.matmul``,
``jnp.exp``, ``lax.conv_general_dilated``) are restated with numpy/scipy.

Two precisions:

* ``np.float64`` -- the FP64 oracle (complex128 FFTs).
* ``np.float32`` -- mirrors leniax's FP32 op order (complex64 full ``fftn``,
  float32 elementwise ops in the same order as the reference source).

Pinning: the FP32 mode reproduces leniax's own golden frames
``tests/fixtures/{orbium-test_last_frame,orbium-scutium-test_last_frame2,
aquarium-test_last_frame}.p`` at the reference tests' tolerances
(``tests/test_pipeline.py:35,92,111``) plus the KATs of ``tests/test_core.py``
and ``tests/test_statistics.py``; see ``tests/test_oracle_golden.py``.

Reference files cited below are paths inside the leniax project.
"""
from __future__ import annotations

import base64
import gzip
import math
from fractions import Fraction
from typing import Dict, List, Sequence

import numpy as np

try:  # scipy.fft keeps single precision; numpy.fft is the fallback
    import scipy.fft as _fft

    def _fftn(x, axes, workers=None):
        return _fft.fftn(x, axes=axes, workers=workers)

    def _ifftn(x, axes, workers=None):
        return _fft.ifftn(x, axes=axes, workers=workers)
except Exception:  # pragma: no cover
    def _fftn(x, axes, workers=None):
        return np.fft.fftn(x, axes=axes)

    def _ifftn(x, axes, workers=None):
        return np.fft.ifftn(x, axes=axes)

# leniax/constant.py:7,9
EPSILON = 1e-7
START_CHECK_STOP = 10
# leniax/statistics.py:284,313-314
MONOTONIC_STOP_STEP = 128
MASS_VOLUME_THRESHOLD = 10.
MASS_VOLUME_STOP_STEP = 128
# leniax/constant.py:13
NB_CHARS = (ord('Z') - ord('A')) + (ord('z') - ord('a')) + (ord('þ') - ord('À'))

# Order of the scalar statistics in leniax's stats dict (statistics.py:102-115).
STAT_KEYS = (
    'channel_mass', 'mass', 'mass_volume', 'mass_density', 'growth', 'growth_volume', 'growth_density',
    'mass_speed', 'mass_angle_speed', 'mass_growth_dist', 'inertia', 'potential_volume'
)


def _c(dtype):
    return np.complex64 if np.dtype(dtype) == np.float32 else np.complex128


# ---------------------------------------------------------------------------
# Kernel shell functions -- leniax/kernel_functions.py
# ---------------------------------------------------------------------------
def kf_poly_quad(params, X):
    """kernel_functions.py:7-37: (4 X (1-X))**q"""
    q = params[0]
    return (4 * X * (1 - X))**q


def kf_gauss_bump(params, X):
    """kernel_functions.py:40-69: exp(q (q - 1/(X(1-X) + EPSILON)))"""
    q = params[0]
    with np.errstate(over='ignore', under='ignore'):
        return np.exp(q * (q - 1 / (X * (1 - X) + X.dtype.type(EPSILON))))


def kf_step(params, X):
    """kernel_functions.py:72-102"""
    q = params[0]
    return ((X >= q) * (X <= 1 - q)).astype(X.dtype)


def kf_gauss(params, X):
    """kernel_functions.py:105-134: exp(-((X-q)/(0.3 q))**2 / 2)"""
    q = params[0]
    out = ((X - q) / (X.dtype.type(0.3) * q))**2
    return np.exp(-out / 2)


def kf_threshold(params, X):
    """kernel_functions.py:137-167"""
    return (X >= params[0]).astype(X.dtype)


def kf_staircase(params, X):
    """kernel_functions.py:170-208"""
    m, s = params[0], params[1]
    out = 0.5 * (X >= m - s) * (X < m - s / 2)
    out = out + 1 * (X >= m - s / 2) * (X <= m + s / 2)
    out = out + 0.5 * (X > m + s / 2) * (X <= m + s)
    return out.astype(X.dtype)


def kf_triangle(params, X):
    """kernel_functions.py:211-250"""
    m, s = params[0], params[1]
    left, right = m - s, m + s
    out = (X >= left) * (X < m) * (X - left) / (m - left)
    out = out + (X >= m) * (X <= right) * (X - right) / (m - right)
    return out.astype(X.dtype)


KF_REGISTER = {
    'poly_quad': kf_poly_quad,
    'gauss_bump': kf_gauss_bump,
    'gauss': kf_gauss,
    'step': kf_step,
    'threshold': kf_threshold,
    'staircase': kf_staircase,
    'triangle': kf_triangle,
}


# ---------------------------------------------------------------------------
# Growth functions -- leniax/growth_functions.py
# ---------------------------------------------------------------------------
def gf_poly_quad4(params, X):
    """growth_functions.py:6-45: 2 max(0, 1-(X-m)^2/(9 s^2))^4 - 1"""
    m, s = params[0], params[1]
    out = 1 - (X - m)**2 / (9 * s**2)
    out = np.maximum(0, out)
    out = out**4
    return 2 * out - 1


def gf_gaussian(params, X):
    """growth_functions.py:48-82: 2 exp(-((X-m)/s)^2/2) - 1"""
    m, s = params[0], params[1]
    out = ((X - m) / s)**2
    out = np.exp(-out / 2)
    return 2 * out - 1


def gf_gaussian_target(params, X):
    """growth_functions.py:85-119"""
    m, s = params[0], params[1]
    out = ((X - m) / s)**2
    return np.exp(-out / 2)


def gf_step(params, X):
    """growth_functions.py:122-160"""
    m, s = params[0], params[1]
    out = (np.abs(X - m) <= s)
    return (2 * out - 1).astype(X.dtype)


def gf_staircase(params, X):
    """growth_functions.py:163-201"""
    m, s = params[0], params[1]
    out = 0.5 * (X >= m - s) * (X < m - s / 2)
    out = out + 1 * (X >= m - s / 2) * (X <= m + s / 2)
    out = out + 0.5 * (X > m + s / 2) * (X <= m + s)
    return (2 * out - 1).astype(X.dtype)


def gf_triangle(params, X):
    """growth_functions.py:204-243"""
    m, s = params[0], params[1]
    left, right = m - s, m + s
    out = (X >= left) * (X < m) * (X - left) / (m - left)
    out = out + (X >= m) * (X <= right) * (X - right) / (m - right)
    return (2 * out - 1).astype(X.dtype)


def gf_identity(params, X):
    """growth_functions.py:246-253"""
    return X


GF_REGISTER = {
    'poly_quad4': gf_poly_quad4,
    'gaussian': gf_gaussian,
    'gaussian_target': gf_gaussian_target,
    'step': gf_step,
    'staircase': gf_staircase,
    'triangle': gf_triangle,
    'identity': gf_identity,
}


# ---------------------------------------------------------------------------
# Kernels -- leniax/kernels.py
# ---------------------------------------------------------------------------
def circle_kernel(R, k_params, kf_slug, kf_params, nb_dims=2, dtype=np.float32, normalize=True):
    """Radial ring kernel, kernels.py:176-212 (``circle_2d``), generalised to
    ``nb_dims`` axes (distance over all axes).  For ``nb_dims == 2`` it is the
    reference's ``circle_2d``; the D-dimensional form is this project's
    extension (leniax builds only 2D kernels, kernels.py:192-197).
    ``normalize=False`` skips the division by the sum (kernels.py:207-208):
    with a one-hot ``b`` it gives one ring of the kernel, so a test can form
    the kernel as a differentiable function of the ring weights."""
    dtype = np.dtype(dtype).type
    r = k_params[0]
    bs = np.asarray(k_params[1], dtype=dtype)
    k_radius_px = math.ceil(r * R)
    coords = np.indices([k_radius_px * 2] * nb_dims).astype(dtype)
    centered = (coords - dtype(k_radius_px)) / dtype(r * R)
    distances = np.sqrt(np.sum(centered**2, axis=0))
    nb_b = bs.shape[0]
    B_dist = dtype(nb_b) * distances
    bs_mat = bs[np.minimum(np.floor(B_dist).astype(np.int64), nb_b - 1)]
    kfp = np.asarray(kf_params, dtype=dtype)
    raw_kernel = KF_REGISTER[kf_slug](kfp, np.mod(B_dist, dtype(1)))
    kernel = (distances < 1) * raw_kernel * bs_mat
    if normalize:
        kernel = kernel / kernel.sum()
    return kernel.astype(dtype)[np.newaxis, ...]


def world_kernel(R, k_params, kf_slug, kf_params, world_size, dtype=np.float64, normalize=True):
    """The world-sized, fftshifted real kernel whose ``fftn`` is leniax's
    spectrum: ``circle_kernel`` centred by ``_pad_kernel`` (kernels.py:93-101)
    and shifted by ``fftshift`` (kernels.py:148).  ``[*world_size]``."""
    k = circle_kernel(R, k_params, kf_slug, kf_params, len(world_size), dtype, normalize)
    return np.fft.fftshift(_pad_kernel(k, world_size)[0])


def _pad_kernel(k, world_size):
    """kernels.py:93-101: centre the kernel in a world-sized array."""
    padding = [(0, 0)]
    for ws, ks in zip(world_size, k.shape[1:]):
        pad_needed = ws - ks
        if pad_needed % 2 == 0:
            padding.append(((ws - ks) // 2, (ws - ks) // 2))
        else:
            padding.append(((ws - ks) // 2, (ws - ks) // 2 + 1))
    return np.pad(k, padding)


def crop_zero(kernels):
    """utils.py:296-317: remove, along each world axis, every index where
    all kernels are zero (interior ones included); the zero masks are those
    of the uncropped array."""
    where_zero = kernels == 0
    out = kernels
    for ax in range(1, kernels.ndim):
        others = tuple(a for a in range(kernels.ndim) if a != ax)
        keep = ~np.all(where_zero, axis=others)
        out = np.compress(keep, out, axis=ax)
    return out


def get_kernels_and_mapping(kernels_params: List[Dict], world_size: Sequence[int], nb_channels: int, R: float,
                            fft: bool = True, dtype=np.float32):
    """kernels.py:66-158.

    Returns ``(K, mapping)``: for ``fft=True`` K is the full complex spectrum
    ``[1, C, max_k, *world_size]`` (fftshift then fftn over the world axes,
    kernels.py:145-152); for ``fft=False`` K is ``[C*max_k, 1, kh, kw]`` real.
    ``mapping`` is a dict with ``cin_kernels``, ``cin_gfs``, ``gf_params``
    ``[K, 2]``, ``weights`` ``[C, K]`` and ``true_channels`` (None if all true).
    """
    nb_dims = len(world_size)
    kernels_params = sorted(kernels_params, key=lambda d: d['c_in'])  # kernels.py:90 (stable)
    nbk = len(kernels_params)
    cin_kernels = [[] for _ in range(nb_channels)]
    cin_gfs = [[] for _ in range(nb_channels)]
    cin_gf_params = [[] for _ in range(nb_channels)]
    weights = np.zeros([nb_channels, nbk], dtype=dtype)
    kernels_list = []
    for kernel_idx, p in enumerate(kernels_params):
        assert p.get('k_slug', 'circle_2d') == 'circle_2d', 'only circle_2d kernels are restated'
        k = circle_kernel(R, p['k_params'], p['kf_slug'], p['kf_params'], nb_dims, dtype)
        kernels_list.append(_pad_kernel(k, world_size))
        cin_kernels[p['c_in']].append(kernel_idx)
        cin_gfs[p['c_in']].append(p['gf_slug'])
        cin_gf_params[p['c_in']].append(p['gf_params'])
        weights[p['c_out'], kernel_idx] = p['h']
    kernels = np.concatenate(kernels_list, axis=0)
    if not fft:
        kernels = crop_zero(kernels)
    kshape = kernels.shape[1:]
    max_k = max(map(len, cin_kernels))
    per_channel = []
    true_channels = []
    for lst in cin_kernels:
        K_tmp = kernels[np.array(lst, dtype=np.int64)] if len(lst) else np.zeros((0, ) + kshape, dtype=dtype)
        nb_missing = max_k - K_tmp.shape[0]
        true_channels += [True] * K_tmp.shape[0] + [False] * nb_missing
        if nb_missing > 0:
            K_tmp = np.concatenate([K_tmp, np.zeros((nb_missing, ) + kshape, dtype=dtype)], axis=0)
        per_channel.append(K_tmp[:, np.newaxis])
    if fft:
        axes = tuple(range(-1, -nb_dims - 1, -1))
        K = np.stack(per_channel)[np.newaxis, :, :, 0]  # [1, C, max_k, *ws]
        K = np.fft.fftshift(K, axes=axes)
        K = _fftn(K.astype(_c(dtype)), axes=axes).astype(_c(dtype))
    else:
        K = np.concatenate(per_channel, axis=0)  # [C*max_k, 1, kh, kw]
    gf_params = np.array([gp for lst in cin_gf_params for gp in lst], dtype=dtype)
    mapping = {
        'cin_kernels': cin_kernels,
        'cin_gfs': cin_gfs,
        'gf_slugs': [g for lst in cin_gfs for g in lst],
        'gf_params': gf_params,
        'weights': weights,
        'true_channels': None if all(true_channels) else true_channels,
        'max_k': max_k,
    }
    return K, mapping


def tc_indices_of(true_channels):
    """helpers.py:452-458"""
    if true_channels is None:
        return None
    return tuple(i for i, t in enumerate(true_channels) if t)


# ---------------------------------------------------------------------------
# Step -- leniax/core.py
# ---------------------------------------------------------------------------
def get_potential_fft(state, K, tc_indices=None, workers=None):
    """core.py:52-102: real(ifftn(fftn(state)[:, :, None] * K)), reshape, take."""
    dtype = state.dtype
    nd = state.ndim - 2
    axes = tuple(range(-1, -nd - 1, -1))
    fft_cells = _fftn(state.astype(_c(dtype)), axes=axes, workers=workers).astype(_c(dtype))
    fft_out = fft_cells[:, :, np.newaxis] * K
    conv = np.real(_ifftn(fft_out, axes=axes, workers=workers)).astype(dtype)
    C = state.shape[1]
    conv = conv.reshape((-1, K.shape[2] * C) + state.shape[2:])
    if tc_indices is not None:
        conv = np.take(conv, np.array(tc_indices), axis=1)
    return conv


def get_potential_conv(state, K, padding, tc_indices=None):
    """core.py:105-146: wrap-pad then depthwise VALID cross-correlation
    (``lax.conv_general_dilated`` with ``feature_group_count=C``), over the
    2 or 3 world axes."""
    C = state.shape[1]
    padded = np.pad(state, padding, mode='wrap')
    O = K.shape[0]
    per_group = O // C
    kd = K.shape[2:]
    out_dims = tuple(padded.shape[2 + i] - kd[i] + 1 for i in range(len(kd)))
    out = np.zeros((state.shape[0], O) + out_dims, dtype=state.dtype)
    for o in range(O):
        c = o // per_group
        for tap in np.ndindex(*kd):
            window = tuple(slice(t, t + n) for t, n in zip(tap, out_dims))
            out[:, o] += K[(o, 0) + tap] * padded[(slice(None), c) + window]
    if tc_indices is not None:
        out = np.take(out, np.array(tc_indices), axis=1)
    return out


def update_conv(state, K, gf_params, weights, dt, model):
    """core.py:13-49 with the direct-convolution potential (fft=False):
    ``K`` ``[C*max_k, 1, *kernel_dims]`` with the padding of
    helpers.py:465-481."""
    potential = get_potential_conv(state, K, conv_padding(K.shape), model.tc_indices)
    field = get_field(potential, gf_params, weights, model.gf_slugs, model.average)
    new_state = STATE_REGISTER[model.state_slug](state, field, dt)
    return new_state, field, potential


def conv_padding(kernel_shape):
    """helpers.py:470-478: wrap padding used by the direct-conv potential."""
    pad = [(0, 0), (0, 0)]
    for d in kernel_shape[2:]:
        pad.append((d // 2, d // 2 - 1) if d % 2 == 0 else (d // 2, d // 2))
    return tuple(pad)


def weighted_sum(fields, weights):
    """core.py:202-225: w[C,K] @ fields[K, N*|W|]."""
    N, nbk = fields.shape[:2]
    wd = list(fields.shape[2:])
    C = weights.shape[0]
    f = np.swapaxes(fields, 0, 1).reshape(nbk, -1)
    out = np.matmul(weights, f).reshape([C, N] + wd)
    return np.swapaxes(out, 0, 1)


def weighted_mean(fields, weights):
    """core.py:228-242"""
    out = weighted_sum(fields, weights)
    div = weights.sum(axis=1)
    return out / div.reshape((1, -1) + (1, ) * (fields.ndim - 2))


def get_field(potential, gf_params, weights, gf_slugs, average=True):
    """core.py:163-199"""
    fields = []
    for i, slug in enumerate(gf_slugs):
        fields.append(GF_REGISTER[slug](gf_params[i], potential[:, i]))
    f = np.stack(fields, axis=1)
    return weighted_mean(f, weights) if average else weighted_sum(f, weights)


def _bdt(dt, state):
    dt = np.asarray(dt, dtype=state.dtype)
    if dt.ndim == 1 and dt.shape[0] == state.shape[0] and state.shape[0] != 1:
        dt = dt.reshape((-1, ) + (1, ) * (state.ndim - 1))
    return dt


def get_state_v1(state, field, dt):
    """core.py:245-272: clip(state + dt*field, 0, 1) (straight-through grad)."""
    return np.clip(state + _bdt(dt, state) * field, 0., 1.).astype(state.dtype)


def get_state_v2(state, field, dt):
    """core.py:275-297: state (1-dt) + dt field."""
    dt = _bdt(dt, state)
    return (state * (1 - dt) + dt * field).astype(state.dtype)


def get_state_simple(state, field, dt):
    """core.py:300-319: state + dt field."""
    return (state + _bdt(dt, state) * field).astype(state.dtype)


STATE_REGISTER = {'v1': get_state_v1, 'v2': get_state_v2, 'simple': get_state_simple}


class Model:
    """Bundle of the static arguments that ``helpers.build_update_fn``
    (helpers.py:401-427) closes over."""

    def __init__(self, mapping, state_slug='v1', average=True):
        self.tc_indices = tc_indices_of(mapping['true_channels'])
        self.gf_slugs = list(mapping['gf_slugs'])
        self.state_slug = state_slug
        self.average = average


def update(state, K, gf_params, weights, dt, model: Model, workers=None):
    """core.py:13-49 with the FFT potential."""
    potential = get_potential_fft(state, K, model.tc_indices, workers=workers)
    field = get_field(potential, gf_params, weights, model.gf_slugs, model.average)
    new_state = STATE_REGISTER[model.state_slug](state, field, dt)
    return new_state, field, potential


# ---------------------------------------------------------------------------
# Statistics -- leniax/statistics.py, utils.center_world
# ---------------------------------------------------------------------------
def center_world(x, shift_idx):
    """utils.py:269-293: per-world ``roll(x, -shift, world axes)``."""
    out = np.empty_like(x)
    nd = shift_idx.shape[1]
    axes = tuple(range(-nd, 0))
    for n in range(x.shape[0]):
        out[n] = np.roll(x[n], tuple(-int(s) for s in shift_idx[n]), axes)
    return out


def compute_stats(cells, field, potential, prev_shift, prev_centroid, prev_angle, R, T_static):
    """statistics.py:36-126.  ``R``/``T_static`` are the static world params
    the reference closes over (statistics.py:22-24)."""
    dtype = cells.dtype.type
    ws = cells.shape[2:]
    nd = len(ws)
    dt = dtype(1. / T_static)
    R = dtype(R)
    R2 = dtype(R * R)
    eps = dtype(EPSILON)
    non_batch = tuple(range(-(1 + nd), 0))
    world_axes = tuple(range(-nd, 0))
    coords = np.indices(ws)
    mid = np.array([s // 2 for s in ws]).reshape((-1, ) + (1, ) * nd)
    cc = (coords - mid).astype(dtype)[:, np.newaxis, np.newaxis]  # [nd,1,1,*ws]

    ccells = center_world(cells, prev_shift)
    cfield = center_world(field, prev_shift)
    pos_field = np.maximum(cfield, 0)
    m_00 = ccells.sum(axis=non_batch)
    g_00 = pos_field.sum(axis=non_batch)
    potential_volume = (potential > eps).sum(axis=non_batch).astype(dtype) / R2
    channel_mass = ccells.sum(axis=world_axes) / R2
    mass = m_00 / R2
    mass_volume = (ccells > eps).sum(axis=non_batch).astype(dtype) / R2
    mass_density = mass / (mass_volume + eps)
    growth = g_00 / R2
    growth_volume = (pos_field > eps).sum(axis=non_batch).astype(dtype) / R2
    growth_density = growth / (growth_volume + eps)
    AX = ccells[np.newaxis] * cc
    MX = AX.sum(axis=non_batch)  # [nd, N]
    mass_centroid = MX / (m_00 + eps)
    delta = mass_centroid - prev_centroid
    dist_m = np.sqrt((delta**2).sum(axis=0))
    mass_speed = dist_m / R / dt
    if nd >= 2:
        ang = np.degrees(np.arctan2(delta[1], delta[0])).astype(dtype)
    else:
        ang = np.zeros_like(dist_m)
    mass_angle = ang * (dist_m / R > dtype(0.001))
    mass_angle_speed = (np.mod(mass_angle - prev_angle + dtype(540), dtype(360)) - dtype(180)) / dt
    GX = (pos_field[np.newaxis] * cc).sum(axis=non_batch)
    growth_centroid = GX / (g_00 + eps)
    mass_growth_dist = np.sqrt(((growth_centroid - mass_centroid)**2).sum(axis=0)) / R
    MX2 = (AX * cc).sum(axis=non_batch)
    MuX2 = MX2 - mass_centroid * MX
    mass2_centroid = MuX2 / (m_00**2 + eps)
    inertia = mass2_centroid.sum(axis=0)
    stats = {
        'channel_mass': channel_mass,
        'mass': mass,
        'mass_volume': mass_volume,
        'mass_density': mass_density,
        'growth': growth,
        'growth_volume': growth_volume,
        'growth_density': growth_density,
        'mass_speed': mass_speed,
        'mass_angle_speed': mass_angle_speed,
        'mass_growth_dist': mass_growth_dist,
        'inertia': inertia,
        'potential_volume': potential_volume,
    }
    stats = {k: np.asarray(v, dtype=dtype) for k, v in stats.items()}
    # absolute torus position of the centroid (this project's extra output):
    # centred-frame centroid + size//2 + carried shift, wrapped to [0, size)
    sizes = np.array(ws, dtype=np.float64).reshape(-1, 1)
    stats['mass_centroid'] = np.mod(mass_centroid + (sizes // 2) + prev_shift.T, sizes).T.astype(dtype)
    shift_idx = np.trunc(mass_centroid).astype(np.int64).T
    total_shift = np.mod(prev_shift + shift_idx, np.array(ws, dtype=np.int64)).astype(np.int32)
    frac = (mass_centroid - np.trunc(mass_centroid)).astype(dtype)
    return stats, total_shift, frac, mass_angle.astype(dtype)


def min_channel_mass_heuristic(epsilon, channel_mass):
    """statistics.py:224-236"""
    return (channel_mass >= epsilon).all(axis=1)


def max_channel_mass_heuristic(init_channel_mass, channel_mass):
    """statistics.py:239-251"""
    return (channel_mass <= 3 * init_channel_mass).all(axis=1)


def min_mass_heuristic(epsilon, mass):
    """statistics.py:254-266"""
    return mass >= epsilon


def max_mass_heuristic(init_mass, mass):
    """statistics.py:269-281"""
    return mass <= 3 * init_mass


def monotonic_heuristic(sign, previous_sign, monotone_counter):
    """statistics.py:287-306"""
    sign_cond = (sign == previous_sign)
    monotone_counter = monotone_counter * sign_cond + 1
    return monotone_counter <= MONOTONIC_STOP_STEP, monotone_counter


def mass_volume_heuristic(mass_volume, mass_volume_counter):
    """statistics.py:317-333"""
    volume_cond = mass_volume > MASS_VOLUME_THRESHOLD
    mass_volume_counter = mass_volume_counter * volume_cond + 1
    return mass_volume_counter <= MASS_VOLUME_STOP_STEP, mass_volume_counter


def check_heuristics(stats: Dict[str, np.ndarray]) -> np.ndarray:
    """statistics.py:134-205: sequential scan over T; returns
    ``continue_stat`` ``[T, N]`` (float, cumulative product)."""
    mass = stats['mass']
    cm = stats['channel_mass']
    T, N = mass.shape
    dtype = mass.dtype.type
    should_continue = np.ones(N, dtype=dtype)
    init_cm = cm[0]
    previous_mass = mass[0]
    previous_sign = np.zeros(N, dtype=dtype)
    c_mono = np.zeros(N, dtype=np.int32)
    c_vol = np.zeros(N, dtype=np.int32)
    out = np.zeros((T, N), dtype=dtype)
    for t in range(T):
        cond = min_channel_mass_heuristic(dtype(EPSILON), cm[t])
        cond = cond & max_channel_mass_heuristic(init_cm, cm[t])
        sign = np.sign(mass[t] - previous_mass).astype(dtype)
        c1, c_mono = monotonic_heuristic(sign, previous_sign, c_mono)
        c2, c_vol = mass_volume_heuristic(stats['mass_volume'][t], c_vol)
        cond = cond & c1 & c2
        should_continue = should_continue * cond
        out[t] = should_continue
        previous_mass = mass[t]
        previous_sign = sign
    return out


# Search-batch stop set (the search workload's stop conditions): a world stops at the first
# step whose pre-update state has raw mass below 1e-3, raw mass above
# 0.9 * area, or a live cell (> EPSILON) on the outer rows/columns of the
# un-centred torus.  This is this project's own stop set, not leniax's.
BOX_MIN_MASS = 1e-3
BOX_MAX_FRAC = 0.9


def box_stop_flags(cells):
    """Per-world boolean ``continue`` flag of the box stop set for one step."""
    nd = cells.ndim - 2
    area = float(np.prod(cells.shape[1:]))  # channels x world cells
    raw = cells.reshape(cells.shape[0], -1).sum(axis=1)
    alive = cells > EPSILON
    touch = np.zeros(cells.shape[0], dtype=bool)
    for ax in range(2, 2 + nd):
        first = np.take(alive, 0, axis=ax)
        last = np.take(alive, cells.shape[ax] - 1, axis=ax)
        touch |= first.reshape(cells.shape[0], -1).any(axis=1)
        touch |= last.reshape(cells.shape[0], -1).any(axis=1)
    return (raw >= BOX_MIN_MASS) & (raw <= BOX_MAX_FRAC * area) & (~touch)


# ---------------------------------------------------------------------------
# Scan drivers -- leniax/runner.py
# ---------------------------------------------------------------------------
def run_scan(cells0, K, gf_params, weights, T, max_run_iter, R, model: Model, T_static=None,
             keep_intermediary=True, workers=None, with_box=False):
    """runner.py:119-164 (``keep_intermediary=True``) and the per-solution body
    of runner.py:167-215 (``keep_intermediary=False``).

    Returns ``(cells[T], field[T], potential[T], stats)`` or, without the
    intermediaries, ``(stats, final_cells)``.  ``stats`` values are ``[T, N]``
    (``channel_mass`` ``[T, N, C]``) plus ``N`` (float count).
    """
    dtype = cells0.dtype.type
    T_static = float(T) if T_static is None else T_static
    Tarr = np.asarray(T, dtype=dtype)
    dt = dtype(1) / Tarr
    nd = cells0.ndim - 2
    N = cells0.shape[0]
    shift = np.zeros((N, nd), dtype=np.int32)
    centroid = np.zeros((nd, N), dtype=dtype)
    angle = np.zeros(N, dtype=dtype)
    cells = cells0
    all_stats = {k: [] for k in STAT_KEYS + ('mass_centroid', )}
    ys_cells, ys_field, ys_pot = [], [], []
    box = []
    for _ in range(max_run_iter):
        new_cells, field, potential = update(cells, K, gf_params, weights, dt, model, workers)
        st, shift, centroid, angle = compute_stats(cells, field, potential, shift, centroid, angle, R, T_static)
        for k in all_stats:
            all_stats[k].append(st[k])
        if with_box:
            box.append(box_stop_flags(cells))
        if keep_intermediary:
            ys_cells.append(cells)
            ys_field.append(field)
            ys_pot.append(potential)
        cells = new_cells
    stats = {k: np.stack(v) for k, v in all_stats.items()}
    cont = check_heuristics(stats)
    stats['N'] = cont.sum(axis=0)
    if with_box:
        b = np.stack(box)  # [T, N] continue flags
        stats['N_box'] = np.cumprod(b, axis=0).sum(axis=0).astype(np.int32)
    if keep_intermediary:
        return np.stack(ys_cells), np.stack(ys_field), np.stack(ys_pot), stats
    return stats, cells


def run_scan_mem_optimized(cells0, K, gf_params, weights, T, max_run_iter, R, model: Model, T_static=None,
                           workers=None, with_box=False):
    """runner.py:167-215: vmap over solutions (a loop here).  Stats come back
    ``[Ns, T, Ni]`` and ``N`` ``[Ns, Ni]``, as the reference's vmap stacks them."""
    out_stats = []
    finals = []
    for s in range(cells0.shape[0]):
        st, fin = run_scan(cells0[s], K[s], gf_params[s], weights[s], T[s], max_run_iter, R, model, T_static,
                           keep_intermediary=False, workers=workers, with_box=with_box)
        out_stats.append(st)
        finals.append(fin)
    stats = {k: np.stack([st[k] for st in out_stats]) for k in out_stats[0]}
    return stats, np.stack(finals)


def run_eager(cells, K, gf_params, weights, T, max_run_iter, R, model: Model, stat_trunc=False, T_static=None):
    """runner.py:16-116: Python loop with the total-mass heuristics."""
    dtype = cells.dtype.type
    T_static = float(T) if T_static is None else T_static
    dt = dtype(1) / np.asarray(T, dtype=dtype)
    nd = cells.ndim - 2
    N = 1
    all_cells = [cells]
    all_fields, all_pots, all_stats = [], [], []
    init_mass = cells.sum()
    previous_mass = init_mass
    previous_sign = np.zeros(N, dtype=np.int32)
    c_mono = np.zeros(N, dtype=np.int32)
    c_vol = np.zeros(N, dtype=np.int32)
    should_continue = np.ones(N, dtype=np.int32)
    shift = np.zeros((N, nd), dtype=np.int32)
    centroid = np.zeros((nd, N), dtype=dtype)
    angle = np.zeros(N, dtype=dtype)
    current_iter = 0
    for current_iter in range(max_run_iter):
        new_cells, field, potential = update(cells, K, gf_params, weights, dt, model)
        st, shift, centroid, angle = compute_stats(cells, field, potential, shift, centroid, angle, R, T_static)
        cells = new_cells
        all_cells.append(cells)
        all_fields.append(field)
        all_pots.append(potential)
        all_stats.append(st)
        mass = st['mass']
        cond = min_mass_heuristic(EPSILON, mass) & max_mass_heuristic(init_mass, mass)
        sign = np.sign(mass - previous_mass)
        c1, c_mono = monotonic_heuristic(sign, previous_sign, c_mono)
        c2, c_vol = mass_volume_heuristic(st['mass_volume'], c_vol)
        should_continue = should_continue * (cond & c1 & c2)
        previous_mass = mass
        previous_sign = sign
        if stat_trunc and current_iter >= START_CHECK_STOP and int(should_continue[0]) == 0:
            break
    all_cells.pop()
    stats = {k: np.stack([s[k] for s in all_stats]) for k in all_stats[0]} if all_stats else {}
    stats['N'] = np.array(current_iter)
    return np.stack(all_cells), np.stack(all_fields), np.stack(all_pots), stats


# ---------------------------------------------------------------------------
# Cell-state codecs and config helpers (fixture decoding)
# ---------------------------------------------------------------------------
_DIM_DELIM = {0: '', 1: '$', 2: '%', 3: '#', 4: '@A', 5: '@B', 6: '@C', 7: '@D', 8: '@E', 9: '@F'}


def _char2val_deprecated(ch: str) -> int:
    """loader.py:273-281"""
    if ch in '.b':
        return 0
    if ch == 'o':
        return 255
    if len(ch) == 1:
        return ord(ch) - ord('A') + 1
    return (ord(ch[0]) - ord('p')) * 24 + (ord(ch[1]) - ord('A') + 25)


def _append_stack(lst, elem, count, is_repeat=False):
    lst.append(elem)
    if count != '':
        repeated = elem if is_repeat else []
        lst.extend([repeated] * (int(count) - 1))


def _max_lens(dim, lst, max_lens, nb_dims):
    max_lens[dim] = max(max_lens[dim], len(lst))
    if dim < nb_dims - 1:
        for sub in lst:
            _max_lens(dim + 1, sub, max_lens, nb_dims)


def _cubify(dim, lst, max_lens, nb_dims):
    more = max_lens[dim] - len(lst)
    if dim < nb_dims - 1:
        lst.extend([[]] * more)
        for sub in lst:
            _cubify(dim + 1, sub, max_lens, nb_dims)
    else:
        lst.extend([0] * more)


def rle_decode(cells_code: str, nb_dims: int) -> np.ndarray:
    """Deprecated run-length cell codec, loader.py:323-350."""
    stacks: List[List] = [[] for _ in range(nb_dims)]
    last, count = '', ''
    delims = list(_DIM_DELIM.values())
    st = cells_code.rstrip('!') + _DIM_DELIM[nb_dims - 1]
    for ch in st:
        if ch.isdigit():
            count += ch
        elif ch in 'pqrstuvwxy@':
            last = ch
        else:
            if last + ch not in delims:
                _append_stack(stacks[0], _char2val_deprecated(last + ch) / 255, count, is_repeat=True)
            else:
                dim = delims.index(last + ch)
                for d in range(dim):
                    _append_stack(stacks[d + 1], stacks[d], count, is_repeat=False)
                    stacks[d] = []
            last, count = '', ''
    cells_l = stacks[nb_dims - 1]
    max_lens = [0] * nb_dims
    _max_lens(0, cells_l, max_lens, nb_dims)
    _cubify(0, cells_l, max_lens, nb_dims)
    return np.array(cells_l, dtype=np.float32)


def gzip_decode(string_cells: str) -> np.ndarray:
    """gzip+base64 int32 codec, loader.py:105-129."""
    raw = gzip.decompress(base64.decodebytes(string_cells.encode('utf-8')))
    max_val = NB_CHARS**2 - 1
    n = int.from_bytes(raw[0:4], 'little')
    vals = np.frombuffer(raw[4:4 + 4 * n], dtype='<i4').astype(np.int64)
    shape = [int.from_bytes(raw[i:i + 4], 'little') for i in range(4 + 4 * n, len(raw), 4)]
    return (vals.reshape(shape) / max_val).astype(np.float32)


def decode_cells(code, nb_dims_with_channel: int) -> np.ndarray:
    """Subset of loader.decompress_array (loader.py:69-102): gzip, then the
    deprecated RLE (the pickle-based fallbacks are not restated)."""
    if isinstance(code, (list, tuple)):
        return np.array(code, dtype=np.float32)
    try:
        return gzip_decode(code)
    except Exception:
        return rle_decode(code, nb_dims_with_channel)


def st2fracs2float(st: str) -> List[float]:
    """utils.py:214-225"""
    return [float(Fraction(s)) for s in st.split(',')]


_OLD_GF = {0: 'poly_quad4', 1: 'gaussian', 2: 'gaussian_target', 3: 'step'}
_OLD_K = {0: 'poly_quad', 1: 'gauss_bump', 2: 'step', 3: 'staircase', 4: 'gauss'}


def kernels_v1_to_v2(k_list: List[Dict]) -> List[Dict]:
    """utils.py:91-124: v1 kernel entries to v2 kernel params."""
    out = []
    for kp in k_list:
        bs = st2fracs2float(kp['b']) if isinstance(kp['b'], str) else kp['b']
        out.append({
            'k_slug': 'circle_2d',
            'k_params': [kp.get('r', 1.), bs],
            'kf_slug': _OLD_K[kp['k_id']],
            'kf_params': [kp['q']],
            'gf_slug': _OLD_GF[kp['gf_id']],
            'gf_params': [kp['m'], kp['s']],
            'h': kp['h'],
            'c_in': kp['c_in'],
            'c_out': kp['c_out'],
        })
    return out


def merge_cells(cells, other, offset=None):
    """utils.py:231-263 (centred additive merge)."""
    assert cells.ndim == other.ndim and cells.shape[0] == other.shape[0]
    offset = offset or [0] * cells.ndim
    pads = []
    for i in range(cells.ndim):
        ps = int(max((cells.shape[i] - other.shape[i]) // 2 + offset[i], 0))
        pads.append((ps, int(cells.shape[i] - other.shape[i] - ps)))
    return cells + np.pad(other, pads)


def create_init_cells(world_size, nb_channels, raw_cells):
    """helpers.py:91-128 for the list-of-patterns form."""
    cells = np.zeros([nb_channels] + list(world_size), dtype=np.float32)
    for c in raw_cells:
        if len(c) != 0:
            cells = merge_cells(cells, c)
    return cells[np.newaxis]


# ---------------------------------------------------------------------------
# Initial states -- leniax/perlin.py, leniax/initializations.py, loader.py
# ---------------------------------------------------------------------------
def perlin_interpolant(t):
    """perlin.py:12-13: 6t^5 - 15t^4 + 10t^3."""
    return t * t * t * (t * (t * 6 - 15) + 10)


def perlin_noise_2d(angles, shape, res):
    """perlin.py:16-71 (generate_perlin_noise_2d): 2D Perlin noise of
    ``angles.shape[0]`` states from the gradient angles ``[n, res0, res1]``.
    The gradients at the lattice points are (cos a, sin a), wrapped by one
    period, repeated ``shape // res`` times along each axis and sliced at the
    four corners; ramps are the fractional grid coordinates (taken here as
    ``arange(shape) * (res / shape) % 1``); the quintic interpolant blends the
    four corner dot products; the result is scaled by sqrt(2)."""
    angles = np.asarray(angles, dtype=np.float64)
    grads = np.stack([np.cos(angles), np.sin(angles)], axis=-1)  # [n, r0, r1, 2]
    grads = np.pad(grads, [(0, 0), (0, 1), (0, 1), (0, 0)], mode='wrap')
    d = (shape[0] // res[0], shape[1] // res[1])
    grads = grads.repeat(d[0], 1).repeat(d[1], 2)
    diff = [grads.shape[1] - shape[0], grads.shape[2] - shape[1]]
    g00 = grads[:, :-diff[0], :-diff[1]]
    g10 = grads[:, diff[0]:, :-diff[1]]
    g01 = grads[:, :-diff[0], diff[1]:]
    g11 = grads[:, diff[0]:, diff[1]:]
    gy = (np.arange(shape[0]) * (res[0] / shape[0])) % 1
    gx = (np.arange(shape[1]) * (res[1] / shape[1])) % 1
    grid = np.stack(np.meshgrid(gy, gx, indexing='ij'), axis=-1)[np.newaxis]  # [1, H, W, 2]
    n00 = (np.stack([grid[..., 0], grid[..., 1]], -1) * g00).sum(3)
    n10 = (np.stack([grid[..., 0] - 1, grid[..., 1]], -1) * g10).sum(3)
    n01 = (np.stack([grid[..., 0], grid[..., 1] - 1], -1) * g01).sum(3)
    n11 = (np.stack([grid[..., 0] - 1, grid[..., 1] - 1], -1) * g11).sum(3)
    t = perlin_interpolant(grid)
    n0 = n00 * (1 - t[..., 0]) + t[..., 0] * n10
    n1 = n01 * (1 - t[..., 0]) + t[..., 0] * n11
    return np.sqrt(2) * ((1 - t[..., 1]) * n0 + t[..., 1] * n1)


def perlin_res(world_size, R):
    """initializations.py:57-58: Perlin periods of a world."""
    kr = math.ceil(R)
    return [world_size[0] // (kr * 3), world_size[1] // (kr * 2)]


def make_array_compressible(cells):
    """loader.py:16-30: round to the NB_CHARS**2 - 1 grid (numpy's round is
    half to even, as jnp.round)."""
    max_val = NB_CHARS**2 - 1
    return (np.round(cells * max_val).astype(np.int32) / max_val).astype(np.float32)


def perlin_init(angles, world_size, R, m, compressible=True):
    """initializations.py:35-77 given the gradient angles ``[nb_init, *res]``:
    noise normalised per state to [0, 1], scaled by m + i / nb_init *
    (min(1, 3 m) - m), made compressible.  -> ``[nb_init, 1, *world]``."""
    nb_init = angles.shape[0]
    cells = perlin_noise_2d(angles, tuple(world_size), tuple(perlin_res(world_size, R)))
    cells = cells - cells.min(axis=(1, 2), keepdims=True)
    cells = cells / cells.max(axis=(1, 2), keepdims=True)
    hi = min(1, 3 * m)
    scaling = np.array([m + i / nb_init * (hi - m) for i in range(nb_init)])[:, None, None]
    cells = (cells * scaling)[:, np.newaxis]
    return make_array_compressible(cells) if compressible else cells.astype(np.float32)


def cropped_perlin_init(angles, world_size, R, m, compressible=True):
    """initializations.py:80-116: the Perlin state's 2 ceil(R) square at rows
    and columns [24, 24 + 2 ceil(R)) centred on a zero 128 x 128 world."""
    cells = perlin_init(angles, world_size, R, m, compressible)
    size = math.ceil(R) * 2
    pad_left = (128 - size) // 2
    pad_right = pad_left + 1 if pad_left * 2 + size != 128 else pad_left
    out = np.pad(cells[:, :, 24:24 + size, 24:24 + size], ((0, 0), (0, 0), (pad_left, pad_right),
                                                           (pad_left, pad_right)))
    return make_array_compressible(out) if compressible else out
