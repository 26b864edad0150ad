"""Parity at the benchmark's own workloads, through the benchmark's own input
generators (``bench.make_inputs``, ``workloads.multichannel_params`` /
``multichannel_cells``, ``workloads.build_classes``).

Noise worlds are chaotic.  Over hundreds of steps two FP32 implementations of
the same step -- or leniax's FP32 op order and the FP64 oracle -- separate
exponentially, and for some worlds the stop step itself moves (16 worlds of the
128x128 search batch, 1024 steps: the FP32 oracle's ``N`` differs from the FP64
oracle's for 3 of them, e.g. 192 vs 243).  The tests therefore measure, per
world, the *predictable horizon* h: the first step at which the FP32 oracle's
mass departs from the FP64 oracle's by more than 1e-3 (relative), and require

* while t < h, the engine's mass (and centroid) within max(1e-4 relative,
  16x the FP32 oracle's own running error) of FP64 -- the engine is an FP32
  implementation of leniax's step as accurate as leniax's op order, up to a
  constant factor (two FP32 roundings of a chaotic map project differently
  onto its unstable direction, so their errors differ by a bounded factor);
* identical ``N`` / ``N_box`` to the FP64 oracle for every world whose stop
  step falls inside its predictable horizon (a stop decided while FP32
  arithmetic still tracks FP64), and that most worlds are of that kind;
* the final state within 16x the FP32-vs-FP64 spread for worlds that never
  leave their horizon.

Reference semantics: ``runner.py:167-215`` (batch rollout),
``statistics.py:11-205`` (stats and ``check_heuristics``), ``core.py:13-49``.
"""
import os

import numpy as np
import pytest
import torch

import bench
from leniax_gb300 import batch as lbatch
from leniax_gb300 import grad as lgrad
from leniax_gb300 import helpers, kernels, runner, statistics, workloads
from oracle import lenia_grad_oracle as GO
from oracle import lenia_oracle as O
from tests.cases import bump_kernel_params

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-5
REL = 1e-3  # gradient bound vs float64 autograd
ENVELOPE = 16  # engine error / FP32-oracle error bound on chaotic rollouts


def _workers():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def _horizon(m32, m64, tol=1e-3):
    """[T, n] masses -> per-world first step where the FP32 oracle departs
    from FP64 by more than tol (relative, floor 1e-3), T if never."""
    rel = np.abs(m32 - m64) / np.maximum(np.abs(m64), 1e-3)
    T = rel.shape[0]
    bad = rel > tol
    return np.where(bad.any(axis=0), bad.argmax(axis=0), T)


def _check_chaotic_batch(tag, mass_e, N_e, Nbox_e, fin_e, st32, st64, fin32, fin64, min_decided):
    """Chaos-aware comparison of an engine rollout with the FP32 / FP64
    oracles (arrays [T, n] for masses, [n] for stop counts, [n, ...] finals)."""
    m32, m64 = st32['mass'], st64['mass']
    T, n = m64.shape
    h = _horizon(m32, m64)
    env = np.maximum.accumulate(np.abs(m32 - m64), axis=0)  # FP32 oracle's running error
    tol = np.maximum(1e-4 * np.abs(m64), ENVELOPE * env) + 1e-7
    decided_n = decided_box = 0
    for w in range(n):
        t = slice(0, int(h[w]))
        err = np.abs(mass_e[t, w] - m64[t, w])
        assert (err <= tol[t, w]).all(), (tag, w, int(h[w]), float((err / tol[t, w]).max()))
        if st64['N'][w] < h[w] or h[w] == T:
            decided_n += 1
            assert int(N_e[w]) == int(st64['N'][w]), (tag, w, 'N', int(N_e[w]), int(st64['N'][w]), int(h[w]))
        if st64['N_box'][w] < h[w] or h[w] == T:
            decided_box += 1
            assert int(Nbox_e[w]) == int(st64['N_box'][w]), (tag, w, 'N_box', int(Nbox_e[w]),
                                                               int(st64['N_box'][w]), int(h[w]))
        if h[w] == T:
            spread = np.abs(fin32[w] - fin64[w]).max()
            assert np.abs(fin_e[w] - fin64[w]).max() <= max(2e-4, ENVELOPE * spread), (tag, w, spread)
    assert decided_n >= min_decided and decided_box >= min_decided, (tag, decided_n, decided_box)
    return h


def test_search_batch_128_1024_steps(cuda):
    """The search-batch workload (16 of the bench's 1024 worlds of 128x128:
    48x48 patches scaled by U[0.5, 1], bump kernel R=13, gaussian growth
    m=0.15 s=0.015, dt=0.1), 1024 steps on the resident engine with leniax's
    statistics, check_heuristics N and the box stop set."""
    dev = cuda
    n, steps = 16, bench.STEPS_EULER
    cells = bench.make_inputs(bench.N_WORLDS, seed=1)[:, :n].copy()  # the bench's first 16 worlds
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in bench.KPARAMS], [bench.SIZE] * 2, 1, bench.R, True, dev)
    upd = helpers.build_update_fn(K.shape, mp)
    from leniax_gb300 import _lib
    assert _lib.load().lgx_select_engine(upd.model.plan.handle, 1, n, 0) == _lib.ENGINES['resident']
    stats_fn = statistics.ComputeStatsFn([bench.SIZE] * 2, bench.R, bench.T_RATE)
    sd, fin = runner.run_scan_mem_optimized(None, torch.from_numpy(cells).to(dev), K[None],
                                            mp.get_gf_params(dev)[None], mp.get_kernels_weight_per_channel(dev)[None],
                                            torch.tensor([bench.T_RATE]), steps, bench.R, upd, stats_fn,
                                            with_box=True, with_centroid=True)
    res = {}
    for dt in (np.float32, np.float64):
        Ko, mpo = O.get_kernels_and_mapping([dict(p) for p in bench.KPARAMS], [bench.SIZE] * 2, 1, bench.R, True, dt)
        res[dt] = O.run_scan(cells[0].astype(dt), Ko, mpo['gf_params'], mpo['weights'], bench.T_RATE, steps, bench.R,
                             O.Model(mpo), keep_intermediary=False, workers=_workers(), with_box=True)
    (st32, f32), (st64, f64) = res[np.float32], res[np.float64]
    mass = sd['mass'][0].cpu().numpy()
    h = _check_chaotic_batch('search', mass, sd['N'][0].cpu().numpy(), sd['N_box'][0].cpu().numpy(),
                             fin[0].cpu().numpy(), st32, st64, f32, f64, min_decided=9)
    # centroid: absolute torus positions (circular differences), while the
    # world is alive and predictable, against the FP32 oracle's running error
    cen, c64, c32 = sd['mass_centroid'][0].cpu().numpy(), st64['mass_centroid'], st32['mass_centroid']

    def circ(a, b):
        d = np.abs(a - b)
        return np.minimum(d, bench.SIZE - d)

    env = np.maximum.accumulate(circ(c32, c64), axis=0)  # [T, n, 2]
    for w in range(n):
        t = slice(0, int(h[w]))
        alive = st64['mass'][t, w] > 1e-3
        tol = np.maximum(1e-4 * bench.SIZE, ENVELOPE * env[t, w])
        assert (circ(cen[t, w], c64[t, w]) <= tol)[alive].all(), w


def test_multichannel_256_c3k15(cuda):
    """The multi-channel workload: workloads.multichannel_params(3, 5, seed=0)
    on 256x256 (R=20, T=5 so dt=0.2), 4 of its worlds.  One step through
    lgx_update <= 1e-5 of the FP32 oracle; a 32-step rollout on the streamed
    engine (the bench's engine) with identical N and N_box."""
    dev = cuda
    C, size, Rw, Tm, n = 3, 256, 20.0, 5.0, 4
    kp = workloads.multichannel_params(C, 5, seed=0, world_R=Rw)
    cells = workloads.multichannel_cells(n, C, size, 64, seed=0)
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], [size, size], C, Rw, True, dev)
    upd = helpers.build_update_fn(K.shape, mp, 'v1', True)
    Ko, mpo = O.get_kernels_and_mapping([dict(p) for p in kp], [size, size], C, Rw, True, np.float32)
    model = O.Model(mpo, 'v1', True)
    dt = np.float32(1) / np.float32(Tm)
    so, fo, po = O.update(cells, Ko, mpo['gf_params'], mpo['weights'], dt, model)
    s, f, p = upd(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev),
                  mp.get_kernels_weight_per_channel(dev), torch.tensor(dt, device=dev))
    assert np.abs(p.cpu().numpy() - po).max() < 2e-6
    assert np.abs(s.cpu().numpy() - so).max() <= STEP_TOL
    assert np.abs(f.cpu().numpy() - fo).max() < 2e-4
    steps = 32
    stats_fn = statistics.ComputeStatsFn([size, size], Rw, Tm)
    sd, fin = runner.run_scan_mem_optimized(None, torch.from_numpy(cells[None]).to(dev), K[None],
                                            mp.get_gf_params(dev)[None], mp.get_kernels_weight_per_channel(dev)[None],
                                            torch.tensor([Tm]), steps, Rw, upd, stats_fn, engine='streamed',
                                            with_box=True, check_status=True)
    res = {}
    for dtp in (np.float32, np.float64):
        Kd, mpd = O.get_kernels_and_mapping([dict(p) for p in kp], [size, size], C, Rw, True, dtp)
        res[dtp] = O.run_scan(cells.astype(dtp), Kd, mpd['gf_params'], mpd['weights'], Tm, steps, Rw,
                              O.Model(mpd, 'v1', True), keep_intermediary=False, workers=_workers(), with_box=True)
    (st32, f32), (st64, f64) = res[np.float32], res[np.float64]
    _check_chaotic_batch('multichannel', sd['mass'][0].cpu().numpy(), sd['N'][0].cpu().numpy(),
                         sd['N_box'][0].cpu().numpy(), fin[0].cpu().numpy(), st32, st64, f32, f64, min_decided=n)
    cm, cm64 = sd['channel_mass'][0].cpu().numpy(), st64['channel_mass']
    assert cm.shape == cm64.shape == (steps, n, C)
    assert (np.abs(cm - cm64) <= 1e-4 * np.abs(cm64) + 1e-6).all()


@pytest.mark.parametrize('line_group', [2, 4])
def test_uneven_batch_sample_of_build_classes(cuda, line_group):
    """The uneven-batch workload as the bench builds it (workloads.build_classes:
    per-world R in [5, 26], m in [0.1, 0.35], s in [0.01, 0.05], dt in
    {0.05, 0.1, 0.2}, patches of side size/3), a per-class sample run through
    one UnevenBatch launch for 256 steps; every world against the oracle run
    alone (runner.py:119-164 per world)."""
    dev = cuda
    steps = 256
    full = workloads.build_classes(device=dev)
    take = {2: 3, 3: 2}
    sub = []
    for c in full:
        k = take[len(c.world)]
        sub.append(lbatch.WorldClass(cells0=c.cells0[:k].contiguous(), K=c.K[:k].contiguous(),
                                     gf_params=c.gf_params[:k].contiguous(), weights=c.weights[:k].contiguous(),
                                     T=c.T[:k].contiguous(), R=c.R[:k].contiguous()))
    b = lbatch.UnevenBatch(sub, steps, line_group=line_group)
    b.run()
    assert b.status() == 0
    res = b.results()
    for ci, c in enumerate(sub):
        world = list(c.world)
        cells = c.cells0.cpu().numpy()
        R, gfp, T = c.R.cpu().numpy(), c.gf_params.cpu().numpy(), c.T.cpu().numpy()
        out = {'st32': {'mass': [], 'N': [], 'N_box': []}, 'st64': {'mass': [], 'N': [], 'N_box': []}, 'f32': [],
               'f64': []}
        for w in range(c.n):
            kp = bump_kernel_params(m=float(gfp[w, 0]), s=float(gfp[w, 1]))
            for dtp, key in ((np.float32, '32'), (np.float64, '64')):
                Ko, mpo = O.get_kernels_and_mapping([dict(p) for p in kp], world, 1, float(R[w]), True, dtp)
                st, f = O.run_scan(cells[w][None, None].astype(dtp), Ko, mpo['gf_params'], mpo['weights'],
                                   float(T[w]), steps, float(R[w]), O.Model(mpo), keep_intermediary=False,
                                   workers=_workers(), with_box=True)
                for k in ('mass', 'N', 'N_box'):
                    out['st' + key][k].append(st[k][..., 0] if k == 'mass' else st[k][0])
                out['f' + key].append(f[0, 0])
        st32 = {k: np.stack(v, -1) if k == 'mass' else np.array(v) for k, v in out['st32'].items()}
        st64 = {k: np.stack(v, -1) if k == 'mass' else np.array(v) for k, v in out['st64'].items()}
        r = res[ci]
        _check_chaotic_batch(f'uneven {world}', r['stats']['mass'][:, :, 0].cpu().numpy().T,
                             r['stats']['N'][:, 0].cpu().numpy(), r['stats']['N_box'][:, 0].cpu().numpy(),
                             r['final'].cpu().numpy(), st32, st64, np.stack(out['f32']), np.stack(out['f64']),
                             min_decided=1)


def _replay_cells_grad(S, U, after, tgt, Kh, m, s, dt, clip):
    """float64 replay of the reverse pass on a given forward trajectory: S, U
    the states entering and the potentials of each step [T, H, W], `after`
    the states after each step; loss MSE(after[-1], tgt).  Returns
    dL/d(initial cells)."""
    P = tgt.size
    lam = 2 * (after[-1] - tgt) / P
    for t in reversed(range(S.shape[0])):
        mask = ((after[t] > 0) & (after[t] < 1)).astype(np.float64) if clip == 'mask' else 1.0
        d = (U[t] - m) / s
        a = mask * lam * dt * (-2 * np.exp(-d * d / 2) * d / s)
        lam = mask * lam + np.fft.irfft2(np.fft.rfft2(a) * np.conj(Kh), s=S.shape[1:])
    return lam


@pytest.mark.parametrize('clip', ['ste', 'mask'])
def test_differentiation_128_ckpt16_three_segments(cuda, clip):
    """The differentiation workload's setup (bench inputs of 128x128, the
    two-ring kernel b=[0.9, 1] of the loss, target from b=[1, 1] at m=0.16,
    s=0.017) over 48 steps with checkpoints every 16 (three segments, so the
    backward pass recomputes and chains three resident adjoint launches).
    Each world is its own solution, so every world has its own kernel and
    (m, s) gradients.  Two properties are checked separately:

    * exactness of the adjoint: its gradient equals a float64 replay of the
      reverse pass on the engine's own forward trajectory (<= 1e-4);
    * agreement with float64 autograd of leniax's graph: per world and
      gradient within max(1e-3, 4x the error of float32 autograd).  Chaotic
      worlds amplify any FP32 rounding, float32 autograd of the same graph
      included (up to 1e-2 relative on dL/ds at 48 steps), so the bound says
      "as accurate as FP32 arithmetic allows".  The mask clip makes the
      gradient discontinuous in the trajectory: it is held to this bound on
      worlds whose forward stays within the 1e-4 state band of FP64 (a
      nearly dead world whose FP32 forward drifts by 1e-3 moves its mask
      gradient by tens of percent; the straight-through gradient is held
      everywhere).  The 1e-3 bound must bind on at least two
      well-conditioned worlds with the straight-through clip and one with
      the mask clip (at 48 steps float32 autograd resolves the mask-clip
      gradients of only one of the bench's first 16 worlds to 2.5e-4, and
      its own forward leaves the 1e-4 band in 15 of them).  A gradient below 1e-6 of the batch's
      largest gradient of its kind is rounding residue: the engine's must
      then lie within that floor of it."""
    dev = cuda
    n, size, steps, ckpt = 8, bench.SIZE, 48, 16
    cells = bench.make_inputs(64, seed=4)[0, :n]  # [n, 1, H, W]
    kr64 = O.world_kernel(bench.R, [1.0, [0.9, 1.0]], 'gauss_bump', [1.0], [size, size])
    kt64 = O.world_kernel(bench.R, [1.0, [1.0, 1.0]], 'gauss_bump', [1.0], [size, size])
    m, s, w, T = 0.15, 0.015, 1.0, bench.T_RATE
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in bench.KPARAMS], [size, size], 1, bench.R, True, dev)
    upd = helpers.build_update_fn(K.shape, mp)
    targets, fin64 = [], []
    for i in range(n):
        with torch.no_grad():
            targets.append(GO.rollout(torch.from_numpy(cells[i].astype(np.float64)), torch.from_numpy(kt64), 0.16,
                                      0.017, 1.0, 1 / T, steps).numpy().astype(np.float32))
            fin64.append(GO.rollout(torch.from_numpy(cells[i].astype(np.float64)), torch.from_numpy(kr64), m, s, w,
                                    1 / T, steps).numpy())
    tgt = np.stack(targets)
    c0 = torch.from_numpy(cells[:, None]).to(dev).requires_grad_(True)  # [n sols, 1 init, 1, H, W]
    kr = torch.from_numpy(np.stack([kr64.astype(np.float32)] * n)).to(dev).requires_grad_(True)
    gf = torch.tensor([[[m, s]]] * n, device=dev, requires_grad=True)
    ww = torch.full((n, 1, 1), w, device=dev)
    fin = lgrad.rollout(c0, kr, gf, ww, torch.full((n, ), T), upd, steps, ckpt, clip)
    per_world = ((fin - torch.from_numpy(tgt[:, None]).to(dev))**2).mean(dim=(1, 2, 3, 4))
    per_world.sum().backward()
    g_e = [c0.grad[:, 0].cpu().numpy(), kr.grad.cpu().numpy(), gf.grad[:, 0, 0].cpu().numpy(),
           gf.grad[:, 0, 1].cpu().numpy()]
    fin_e = fin[:, 0].detach().cpu().numpy()

    def rel(a, b):
        return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))

    # exactness: float64 replay on the engine's own trajectory (states and
    # potentials from run_scan on the same spectrum)
    kh = lgrad.kernel_spectrum(kr.detach()[:1])
    Kh64 = np.fft.rfft2(kr64)
    for i in range(n):
        cs, _, ps, _ = runner.run_scan(None, torch.from_numpy(cells[i][None]).to(dev), kh[None, None],
                                       torch.tensor([[m, s]], device=dev), torch.ones((1, 1), device=dev),
                                       torch.tensor(T), steps, bench.R, upd,
                                       statistics.ComputeStatsFn([size] * 2, bench.R, T))
        S = cs[:, 0, 0].double().cpu().numpy()
        after = np.concatenate([S[1:], fin_e[i].astype(np.float64)])
        lam = _replay_cells_grad(S, ps[:, 0, 0].double().cpu().numpy(), after, tgt[i, 0].astype(np.float64), Kh64,
                                 m, s, 1 / T, clip)
        if np.linalg.norm(lam) > 0:
            assert rel(g_e[0][i], lam) <= 1e-4, (i, rel(g_e[0][i], lam))
    # agreement with float64 autograd; the batch's gradient scale sets the
    # absolute floor below which a gradient is rounding residue
    refs = []
    for i in range(n):
        ref = {}
        for dtp in (np.float32, np.float64):
            ref[dtp] = GO.loss_and_grads(cells[i].astype(dtp), kr64.astype(dtp), dtp(m), dtp(s), dtp(w), dtp(1 / T),
                                         steps, tgt[i].astype(dtp), clip=clip)
        refs.append(ref)
    scale = [max(np.linalg.norm(np.ravel(r[np.float64][1][j])) for r in refs) for j in range(4)]
    well_conditioned = 0
    for i in range(n):
        L64, g64 = refs[i][np.float64]
        g32 = refs[i][np.float32][1]
        assert abs(float(per_world[i]) - L64) <= 1e-4 * abs(L64) + 1e-9, (i, float(per_world[i]), L64)
        if clip == 'mask' and np.abs(fin_e[i] - fin64[i]).max() > 1e-4:
            continue  # forward outside the 1e-4 band: the mask gradient is checked by the replay above
        tight, nonzero = True, False
        for j, name in enumerate(('cells', 'kernel', 'm', 's')):
            ge, r64 = g_e[j][i], g64[j]
            floor = 1e-6 * scale[j]
            err = float(np.linalg.norm(np.ravel(ge) - np.ravel(r64)))
            if np.linalg.norm(np.ravel(r64)) <= floor:
                assert err <= floor, (i, name, err, floor)
                continue
            nonzero = True
            intrinsic = rel(g32[j], r64)
            tight &= intrinsic <= REL / 4
            assert err <= max(REL * np.linalg.norm(np.ravel(r64)), 4 * intrinsic * np.linalg.norm(np.ravel(r64)),
                              floor), (i, name, rel(ge, r64), intrinsic)
        well_conditioned += tight and nonzero
    assert well_conditioned >= (2 if clip == 'ste' else 1), well_conditioned
