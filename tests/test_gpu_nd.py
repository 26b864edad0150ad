"""General N-D engine (odd, non-square and 3D worlds of any side factoring
into 2, 3, 5, 7; any channels and kernels) and the general adjoint, against
the oracle (forward, core.py:13-49 / runner.py:119-215) and float64 autograd of
leniax's graph (the jax.grad stand-in, runner.py:363-448)."""
import numpy as np
import pytest
import torch

from leniax_gb300 import _lib
from leniax_gb300 import grad as lgrad
from leniax_gb300 import helpers, kernels, runner, statistics
from oracle import lenia_grad_oracle as GO
from oracle import lenia_oracle as O
from tests.cases import bump_kernel_params, golden_case, golden_world, random_multichannel_params

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-5
REL = 1e-3


def relerr(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-30))


def _cells(n, C, world, seed, frac=3):
    rng = np.random.Generator(np.random.PCG64(seed))
    cells = np.zeros((n, C) + tuple(world), np.float32)
    sl = tuple(slice((w - w // frac) // 2, (w - w // frac) // 2 + w // frac) for w in world)
    cells[(slice(None), slice(None)) + sl] = rng.random((n, C) + tuple(w // frac for w in world), dtype=np.float32)
    return cells


# (world, C, per_channel kernels, R, mean): odd, non-square, 3D multi-channel, 48^3
CASES = [
    ([45, 45], 1, 1, 8.0, True),
    ([100, 128], 2, 2, 12.0, True),
    ([48, 80], 2, 1, 8.0, False),
    ([48, 48, 48], 1, 1, 8.0, True),
    ([24, 40, 36], 2, 2, 5.0, False),
    ([32, 32, 32], 3, 1, 6.0, True),
]


def _model(world, C, per, R, mean, seed=1):
    if C == 1 and per == 1:
        kp = bump_kernel_params(s=0.03)
    else:
        kp = random_multichannel_params(C, per, seed=seed, R_range=(0.5 * R, R), world_R=R)
    return kp


@pytest.mark.parametrize('world,C,per,R,mean', CASES)
def test_nd_single_step_matches_oracle(cuda, world, C, per, R, mean):
    dev = cuda
    kp = _model(world, C, per, R, mean)
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], list(world), C, R, True, dev)
    upd = helpers.build_update_fn(K.shape, mp, 'v1', mean)
    assert _lib.load().lgx_select_engine(upd.model.plan.handle, 1, 3, 0) == _lib.ENGINES['nd']
    Ko, mpo = O.get_kernels_and_mapping([dict(p) for p in kp], list(world), C, R, True, np.float32)
    cells = _cells(3, C, world, seed=sum(world))
    dt = np.float32(1) / np.float32(5)
    so, fo, po = O.update(cells, Ko, mpo['gf_params'], mpo['weights'], dt, O.Model(mpo, 'v1', mean))
    s, f, p = upd(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev),
                  mp.get_kernels_weight_per_channel(dev), torch.tensor(dt, device=dev))
    tol_p = 5e-6 if len(world) == 3 else 2e-6
    assert np.abs(p.cpu().numpy() - po).max() < tol_p
    assert np.abs(s.cpu().numpy() - so).max() <= STEP_TOL
    assert np.abs(f.cpu().numpy() - fo).max() < 2e-4
    # per-world dt
    dts = np.array([0.1, 0.2, 0.05], np.float32)
    s2, _, _ = upd(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev),
                   mp.get_kernels_weight_per_channel(dev), torch.from_numpy(dts).to(dev))
    for i in range(3):
        so_i, _, _ = O.update(cells[i:i + 1], Ko, mpo['gf_params'], mpo['weights'], dts[i], O.Model(mpo, 'v1', mean))
        assert np.abs(s2[i:i + 1].cpu().numpy() - so_i).max() <= STEP_TOL


@pytest.mark.parametrize('world,C,per,R,mean', [CASES[1], CASES[4]])
def test_nd_run_scan_trajectories_and_stats(cuda, world, C, per, R, mean):
    # run_scan (runner.py:119-164) on the N-D engine: per-step cells, field,
    # potential, the 12 statistics and N against the oracle.  Statistics are
    # held to 1e-4 or to 8x the oracle's own FP32-vs-FP64 spread, whichever is
    # larger: mass_angle_speed is the angle of a centroid displacement, ill
    # conditioned when the centroid barely moves
    dev = cuda
    kp = _model(world, C, per, R, mean, seed=4)
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], list(world), C, R, True, dev)
    upd = helpers.build_update_fn(K.shape, mp, 'v1', mean)
    Ko, mpo = O.get_kernels_and_mapping([dict(p) for p in kp], list(world), C, R, True, np.float32)
    cells = _cells(2, C, world, seed=7)
    steps = 6
    cs_o, fs_o, ps_o, st_o = O.run_scan(cells, Ko, mpo['gf_params'], mpo['weights'], 5, steps, R,
                                        O.Model(mpo, 'v1', mean))
    cs, fs, ps, st = runner.run_scan(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev),
                                     mp.get_kernels_weight_per_channel(dev), torch.tensor(5.), steps, R, upd,
                                     statistics.ComputeStatsFn(list(world), R, 5))
    assert np.abs(cs.cpu().numpy() - cs_o).max() < 2e-5
    assert np.abs(ps.cpu().numpy() - ps_o).max() < 5e-6
    assert np.abs(fs.cpu().numpy() - fs_o).max() < 5e-4
    Ko64, mpo64 = O.get_kernels_and_mapping([dict(p) for p in kp], list(world), C, R, True, np.float64)
    *_, st64 = O.run_scan(cells.astype(np.float64), Ko64, mpo64['gf_params'], mpo64['weights'], 5, steps, R,
                          O.Model(mpo64, 'v1', mean))
    for k in statistics.STAT_KEYS:
        a, b, b32 = st[k].cpu().numpy(), st64[k], st_o[k]
        atol = 8 / R**2 if k.endswith('volume') or k.endswith('density') else 1e-4
        tol = np.maximum(atol + 1e-4 * np.abs(b), 8 * np.abs(b32 - b))
        assert (np.abs(a - b) <= tol).all(), (k, np.abs(a - b).max())
    assert np.abs(st['N'].cpu().numpy() - st_o['N']).max() == 0


def test_nd_48cube_rollout_matches_fp64_oracle(cuda):
    # the 48^3 world of the differentiation workload through lgx_run: final
    # cells within a few times the oracle's FP32-vs-FP64 spread, identical N
    # and N_box, mass close, centroid close while alive
    dev = cuda
    size, R, steps, Ns, Ni = 48, 8.0, 24, 2, 2
    kp_m = [(0.15, 0.03), (0.2, 0.04)]
    cells = np.stack([_cells(Ni, 1, [size] * 3, seed=20 + s) for s in range(Ns)])
    Ks, gfs, ws = [], [], []
    upd = None
    for m, s in kp_m:
        K, mp = kernels.get_kernels_and_mapping(bump_kernel_params(m=m, s=s), [size] * 3, 1, R, True, dev)
        upd = upd or helpers.build_update_fn(K.shape, mp)
        Ks.append(K)
        gfs.append(mp.get_gf_params(dev))
        ws.append(mp.get_kernels_weight_per_channel(dev))
    Ts = torch.tensor([10., 5.])
    sd, fin = runner.run_scan_mem_optimized(None, torch.from_numpy(cells).to(dev), torch.stack(Ks), torch.stack(gfs),
                                            torch.stack(ws), Ts, steps, R, upd,
                                            statistics.ComputeStatsFn([size] * 3, R, 10), with_box=True,
                                            with_centroid=True)
    for s, (m, sg) in enumerate(kp_m):
        res = {}
        for dt in (np.float32, np.float64):
            Ko, mpo = O.get_kernels_and_mapping(bump_kernel_params(m=m, s=sg), [size] * 3, 1, R, True, dt)
            res[dt] = O.run_scan(cells[s].astype(dt), Ko, mpo['gf_params'], mpo['weights'], Ts[s].item(), steps, R,
                                 O.Model(mpo), T_static=10, keep_intermediary=False, with_box=True)
        st, f64 = res[np.float64]
        spread = np.abs(res[np.float32][1] - f64).max()
        assert np.abs(fin[s].cpu().numpy() - f64).max() <= max(2e-4, 8 * spread)
        np.testing.assert_array_equal(sd['N'][s].cpu().numpy(), st['N'])
        np.testing.assert_array_equal(sd['N_box'][s].cpu().numpy(), st['N_box'])
        mass, m64, m32 = sd['mass'][s].cpu().numpy(), st['mass'], res[np.float32][0]['mass']
        assert (np.abs(mass - m64) <= np.maximum(1e-4 * np.abs(m64), 8 * np.abs(m32 - m64)) + 1e-7).all()
        d = np.abs(sd['mass_centroid'][s].cpu().numpy() - st['mass_centroid'])
        d = np.minimum(d, size - d)
        assert (d[m64 > 1e-3] <= 1e-3 * size).all()


# ------------------------------------------------------------------ adjoint
def _kernel_table(mp):
    cin = [c for c, lst in enumerate(mp['cin_kernels']) for _ in lst]
    return cin, mp['gf_slugs']


def _engine_vs_autograd(dev, kp, world, C, R, mean, cells, steps, ckpt, dt, clip='ste', n_init=1):
    """Engine gradients of sum_sol MSE(final_sol, target_sol) with respect to
    (cells0, per-kernel real kernels, gf_params, weights) vs float64 autograd
    of the same graph; each solution takes n_init inits."""
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], list(world), C, R, True, dev)
    upd = helpers.build_update_fn(K.shape, mp, 'v1', mean)
    Ko, mpo = O.get_kernels_and_mapping([dict(p) for p in kp], list(world), C, R, True, np.float64)
    cin, slugs = _kernel_table(mpo)
    axes = tuple(range(-len(world), 0))
    ks = np.stack([np.real(np.fft.ifftn(Ko[0, c, j], axes=axes)) for c, lst in enumerate(mpo['cin_kernels'])
                   for j, _ in enumerate(lst)])  # [K, *world] float64 world-sized fftshifted kernels
    Ns = cells.shape[0] // n_init
    cells = cells.reshape((Ns, n_init, C) + tuple(world))
    target = (cells * 0.5).astype(np.float32)
    nK = len(cin)
    c0 = torch.from_numpy(cells).to(dev).requires_grad_(True)
    kr = torch.from_numpy(np.stack([ks.astype(np.float32)] * Ns)).to(dev).requires_grad_(True)
    gf = torch.from_numpy(np.stack([mpo['gf_params'].astype(np.float32)] * Ns)).to(dev).requires_grad_(True)
    ww = torch.from_numpy(np.stack([mpo['weights'].astype(np.float32)] * Ns)).to(dev).requires_grad_(True)
    fin = lgrad.rollout(c0, kr, gf, ww, torch.full((Ns, ), 1 / dt), upd, steps, ckpt, clip)
    loss = ((fin - torch.from_numpy(target).to(dev))**2).mean(dim=tuple(range(1, fin.dim()))).sum()
    loss.backward()
    got = [c0.grad.cpu().numpy(), kr.grad.cpu().numpy(), gf.grad.cpu().numpy(), ww.grad.cpu().numpy()]
    out = []
    for s in range(Ns):
        L, ref = GO.loss_and_grads_general(cells[s].astype(np.float64), ks, mpo['gf_params'].astype(np.float64),
                                           mpo['weights'].astype(np.float64), np.float64(dt), steps,
                                           target[s].astype(np.float64), cin, slugs, clip=clip, mean=mean)
        out.append([(got[i][s], ref[i]) for i in range(4)])
    assert nK == mpo['gf_params'].shape[0]
    return out


@pytest.mark.parametrize('mean', [True, False])
def test_nd_adjoint_two_channels(cuda, mean):
    # C = 2, K = 4 (two kernels per channel, random target channels): every
    # gradient -- initial cells, each kernel, (m, s) of each kernel and the
    # full [C, K] weight matrix -- within 1e-3 of float64 autograd
    kp = random_multichannel_params(2, 2, seed=5, R_range=(6, 10), world_R=10)
    cells = _cells(4, 2, [64, 64], seed=7, frac=2)
    res = _engine_vs_autograd(cuda, kp, [64, 64], 2, 10.0, mean, cells, 6, 3, 0.2, n_init=2)
    for s in range(2):
        for name, (g, r) in zip(('cells', 'kernel', 'gf', 'weights'), res[s]):
            assert relerr(g, r) <= REL, (mean, s, name, relerr(g, r))


def test_nd_adjoint_aquarium_topology(cuda):
    # leniax's aquarium fixture: C = 3, K = 15 (five per input channel),
    # weighted_sum, gauss kernel function, gaussian growth, dt = 1/2
    cfg, init, _ = golden_case('aquarium')
    cells, _, _ = golden_world(cfg, init)
    res = _engine_vs_autograd(cuda, cfg['kernels_params'], cfg['world_size'], 3, cfg['R'], cfg['weighted_average'],
                              cells, 4, 2, 1 / cfg['T'])
    for name, (g, r) in zip(('cells', 'kernel', 'gf', 'weights'), res[0]):
        assert relerr(g, r) <= REL, (name, relerr(g, r))


@pytest.mark.parametrize('clip', ['ste', 'mask'])
def test_nd_adjoint_48cube_single_world(cuda, clip):
    # the differentiation workload's 3D variant: one 48^3 world, checkpoints
    # every 4 steps over 8; dL/dw is identically zero (weighted_mean, one kernel)
    cells = _cells(1, 1, [48, 48, 48], seed=1)
    res = _engine_vs_autograd(cuda, bump_kernel_params(s=0.03), [48, 48, 48], 1, 8.0, True, cells, 8, 4, 0.1, clip)
    for name, (g, r) in zip(('cells', 'kernel', 'gf'), res[0][:3]):
        assert relerr(g, r) <= REL, (clip, name, relerr(g, r))
    g, r = res[0][3]
    assert np.abs(g).max() <= 1e-6 and np.abs(r).max() <= 1e-9


def test_nd_adjoint_ring_weights_through_the_kernel_builder(cuda):
    # dL/db of every kernel's ring weights: the torch ring builder chained to
    # the engine's kernel gradients, vs float64 autograd through the oracle's
    # rings (circle_2d, kernels.py:176-212), C = 2, K = 2, two rings each
    dev = cuda
    world, R, steps, dt = [64, 64], 10.0, 6, 0.2
    base = dict(k_slug='circle_2d', kf_slug='gauss_bump', kf_params=[1.0], gf_slug='gaussian')
    kp = [dict(base, k_params=[0.9, [0.5, 1.0]], gf_params=[0.15, 0.02], h=0.7, c_in=0, c_out=1),
          dict(base, k_params=[0.7, [1.0, 0.4]], gf_params=[0.25, 0.03], h=0.4, c_in=1, c_out=0)]
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], world, 2, R, True, dev)
    upd = helpers.build_update_fn(K.shape, mp, 'v1', False)
    cells = _cells(1, 2, world, seed=3, frac=2)
    target = cells * 0.5
    bs = [torch.tensor(p['k_params'][1], device=dev, requires_grad=True) for p in kp]
    kr = torch.stack([lgrad.ring_kernel(R, p['k_params'][0], b, 'gauss_bump', [1.0], world) for p, b in zip(kp, bs)])
    gf = torch.tensor([p['gf_params'] for p in kp], device=dev)[None]
    w = mp.get_kernels_weight_per_channel(dev)[None]
    fin = lgrad.rollout(torch.from_numpy(cells[None]).to(dev), kr[None], gf, w, torch.tensor([1 / dt]), upd, steps, 3)
    loss = ((fin - torch.from_numpy(target[None]).to(dev))**2).mean()
    gb = torch.autograd.grad(loss, bs)
    # float64: kernel k = sum_j b_kj ring_kj / sum_j b_kj sum(ring_kj), rings from the oracle
    b64 = [torch.tensor(p['k_params'][1], dtype=torch.float64, requires_grad=True) for p in kp]
    ks = []
    for p, b in zip(kp, b64):
        nb = len(p['k_params'][1])
        rings = torch.from_numpy(np.stack([O.world_kernel(R, [p['k_params'][0], list(np.eye(nb)[j])], 'gauss_bump',
                                                           [1.0], world, normalize=False) for j in range(nb)]))
        ks.append((b[:, None, None] * rings).sum(0) / (b * rings.sum(dim=(1, 2))).sum())
    fin64 = GO.rollout_general(torch.from_numpy(cells.astype(np.float64)), torch.stack(ks),
                               torch.tensor([p['gf_params'] for p in kp], dtype=torch.float64),
                               torch.from_numpy(mp.get_kernels_weight_per_channel().numpy().astype(np.float64)), dt,
                               steps, [0, 1], ['gaussian', 'gaussian'], mean=False)
    l64 = ((fin64 - torch.from_numpy(target.astype(np.float64)))**2).mean()
    gb64 = torch.autograd.grad(l64, b64)
    for a, b in zip(gb, gb64):
        assert relerr(a.cpu().numpy(), b.numpy()) <= REL
