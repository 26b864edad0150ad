"""Engine (CUDA, through the C ABI) vs the oracle and leniax's golden frames."""
import numpy as np
import pytest
import torch

from leniax_gb300 import helpers, kernels, runner, statistics
from oracle import lenia_oracle as O
from tests.cases import bump_kernel_params, golden_case, golden_world, patch_init, random_multichannel_params

pytestmark = pytest.mark.gpu

# single step vs leniax's FP32 op order: max abs error <= 1e-5
STEP_TOL = 1e-5


def engine_model(kparams, world, C, R, state_slug='v1', average=True, dev=None):
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kparams], list(world), C, R, True, dev)
    upd = helpers.build_update_fn(K.shape, mp, state_slug, average)
    return K, mp, upd


def oracle_model(kparams, world, C, R, state_slug='v1', average=True, dtype=np.float32):
    K, mp = O.get_kernels_and_mapping([dict(p) for p in kparams], list(world), C, R, True, dtype)
    return K, mp, O.Model(mp, state_slug, average)


def single_step_case(kparams, world, C, R, cells, T, state_slug='v1', average=True):
    dev = torch.device('cuda')
    K, mp, upd = engine_model(kparams, world, C, R, state_slug, average, dev)
    Ko, mpo, model = oracle_model(kparams, world, C, R, state_slug, average)
    dt = np.float32(1.) / np.float32(T)
    s_o, f_o, p_o = O.update(cells, Ko, mpo['gf_params'], mpo['weights'], dt, model)
    s, f, p = upd(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev), mp.get_kernels_weight_per_channel(dev),
                  torch.tensor(dt, device=dev))
    torch.cuda.synchronize()
    return (s.cpu().numpy(), f.cpu().numpy(), p.cpu().numpy()), (s_o, f_o, p_o)


@pytest.mark.parametrize('size', [32, 64, 128, 256, 512])
def test_update_single_step_bump_gaussian(cuda, size):
    R = 13 if size >= 64 else 6
    cells = patch_init(3, size, min(40, size // 2), seed=size)
    (s, f, p), (so, fo, po) = single_step_case(bump_kernel_params(), [size, size], 1, R, cells, 10)
    assert np.abs(p - po).max() < 2e-6
    assert np.abs(s - so).max() <= STEP_TOL
    assert np.abs(f - fo).max() < 1e-4


@pytest.mark.parametrize('name', ['orbium', 'orbium_scutium', 'aquarium'])
def test_update_single_step_golden_models(cuda, name):
    cfg, init, _ = golden_case(name)
    cells, _, _ = golden_world(cfg, init)
    rng = np.random.Generator(np.random.PCG64(7))
    cells = np.concatenate([cells, rng.random(cells.shape, dtype=np.float32) * 0.5])
    (s, f, p), (so, fo, po) = single_step_case(cfg['kernels_params'], cfg['world_size'], cfg['nb_channels'],
                                               cfg['R'], cells, cfg['T'], cfg['get_state_fn_slug'],
                                               cfg['weighted_average'])
    assert np.abs(p - po).max() < 2e-6
    assert np.abs(s - so).max() <= STEP_TOL
    assert np.abs(f - fo).max() < 2e-4


@pytest.mark.parametrize('slug', ['v1', 'v2', 'simple'])
@pytest.mark.parametrize('gf', ['poly_quad4', 'gaussian', 'gaussian_target', 'step', 'staircase', 'triangle',
                                'identity'])
def test_update_growth_and_state_functions(cuda, gf, slug):
    kp = bump_kernel_params()
    kp[0]['gf_slug'] = gf
    kp[0]['gf_params'] = [0.15, 0.03]
    cells = patch_init(2, 64, 30, seed=3)
    (s, f, p), (so, fo, po) = single_step_case(kp, [64, 64], 1, 10, cells, 10, slug, True)
    assert np.abs(p - po).max() < 2e-6
    # step-like growth functions flip where |potential - edge| < 1 ulp-scale error
    flips = np.abs(f - fo) > 1e-3
    assert flips.mean() < 1e-3
    ok = ~flips
    assert np.abs(s - so)[ok].max() <= STEP_TOL


@pytest.mark.parametrize('engine', ['resident', 'streamed'])
def test_run_scan_reproduces_orbium_golden(cuda, engine):
    cfg, init, last = golden_case('orbium')
    dev = torch.device('cuda')
    cells, _, _ = golden_world(cfg, init)
    K, mp, upd = engine_model(cfg['kernels_params'], cfg['world_size'], 1, cfg['R'], dev=dev)
    stats_fn = statistics.ComputeStatsFn(cfg['world_size'], cfg['R'], cfg['T'])
    cs, fs, ps, st = runner.run_scan(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev),
                                     mp.get_kernels_weight_per_channel(dev), torch.tensor(float(cfg['T'])),
                                     cfg['max_run_iter'], cfg['R'], upd, stats_fn, engine=engine)
    assert cs.shape == (128, 1, 1, 128, 128)
    np.testing.assert_array_almost_equal(last, cs[-1, 0].cpu().numpy(), decimal=4)


@pytest.mark.parametrize('name', ['orbium_scutium', 'aquarium'])
def test_run_scan_reproduces_multichannel_goldens(cuda, name):
    cfg, init, last = golden_case(name)
    dev = torch.device('cuda')
    cells, _, _ = golden_world(cfg, init)
    K, mp, upd = engine_model(cfg['kernels_params'], cfg['world_size'], cfg['nb_channels'], cfg['R'],
                              cfg['get_state_fn_slug'], cfg['weighted_average'], dev)
    stats_fn = statistics.ComputeStatsFn(cfg['world_size'], cfg['R'], cfg['T'])
    cs, _, _, st = runner.run_scan(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev),
                                   mp.get_kernels_weight_per_channel(dev), torch.tensor(float(cfg['T'])),
                                   cfg['max_run_iter'], cfg['R'], upd, stats_fn)
    np.testing.assert_array_almost_equal(last, cs[-1, 0].cpu().numpy(), decimal=cfg['decimal'])


def _oracle_rollout(kparams, world, C, R, T, cells, steps, dtype=np.float32, with_box=False):
    Ko, mpo, model = oracle_model(kparams, world, C, R, dtype=dtype)
    return O.run_scan(cells.astype(dtype), Ko, mpo['gf_params'], mpo['weights'], T, steps, R, model,
                      keep_intermediary=False, with_box=with_box)


@pytest.mark.parametrize('engine', ['resident', 'streamed', 'plain', 'plain_streamed'])
def test_rollout_matches_fp64_oracle(cuda, engine):
    # single world, 128^2, 128 steps: state max abs error and mass / centroid
    # relative error <= 1e-4 against the FP64 oracle
    dev = torch.device('cuda')
    cells = patch_init(1, 128, 40, seed=0)
    kp = bump_kernel_params()
    st64, fin64 = _oracle_rollout(kp, [128, 128], 1, 13, 10, cells, 128, np.float64)
    K, mp, upd = engine_model(kp, [128, 128], 1, 13, dev=dev)
    stats_fn = statistics.ComputeStatsFn([128, 128], 13, 10)
    sd, fin = runner.run_scan_mem_optimized(None, torch.from_numpy(cells[None]).to(dev), K[None],
                                            mp.get_gf_params(dev)[None], mp.get_kernels_weight_per_channel(dev)[None],
                                            torch.tensor([10.]), 128, 13, upd, stats_fn, engine=engine,
                                            with_centroid=True)
    fin = fin.cpu().numpy()[0]
    assert np.abs(fin - fin64).max() <= 1e-4
    mass = sd['mass'][0, :, 0].cpu().numpy()
    m64 = st64['mass'][:, 0]
    alive = m64 > 1e-3  # this world decays; relative errors are taken while it has mass
    assert alive.sum() > 10
    assert (np.abs(mass - m64)[alive] / m64[alive]).max() <= 1e-4
    assert np.abs(mass[~alive] - m64[~alive]).max() <= 1e-6
    cen = sd['mass_centroid'][0, :, 0].cpu().numpy()  # [T, 2] absolute torus positions
    c64 = st64['mass_centroid'][:, 0]
    d = np.abs(cen - c64)
    d = np.minimum(d, 128 - d)  # circular difference
    assert (d[alive] / np.maximum(c64[alive], 1.0)).max() <= 1e-4
    for key in ('mass_volume', 'growth', 'potential_volume', 'inertia'):
        a = sd[key][0, :, 0].cpu().numpy()
        b = st64[key][:, 0]
        assert (np.abs(a - b) / np.maximum(np.abs(b), 1e-3))[alive].max() <= 1e-3, key
    assert int(sd['N'][0, 0]) == int(st64['N'][0])


def test_mem_optimized_batch_matches_oracle_and_engines_agree(cuda):
    dev = torch.device('cuda')
    Ns, Ni, steps, size, R = 3, 5, 48, 64, 10
    ms = [0.15, 0.2, 0.12]
    cells = np.stack([patch_init(Ni, size, 24, seed=10 + s, scale_range=(0.5, 1.0)) for s in range(Ns)])
    Ks, gfs, ws = [], [], []
    upd = None
    for s in range(Ns):
        K, mp, u = engine_model(bump_kernel_params(m=ms[s], s=0.02), [size, size], 1, R, dev=dev)
        upd = upd or u
        Ks.append(K)
        gfs.append(mp.get_gf_params(dev))
        ws.append(mp.get_kernels_weight_per_channel(dev))
    Ts = torch.tensor([10., 5., 8.])
    stats_fn = statistics.ComputeStatsFn([size, size], R, 10)
    outs = {}
    for engine in ('resident', 'streamed'):
        outs[engine] = runner.run_scan_mem_optimized(None, torch.from_numpy(cells).to(dev), torch.stack(Ks),
                                                     torch.stack(gfs), torch.stack(ws), Ts, steps, R, upd, stats_fn,
                                                     engine=engine, with_box=True)
    for s in range(Ns):
        res = {}
        for dt in (np.float32, np.float64):
            Ko, mpo, model = oracle_model(bump_kernel_params(m=ms[s], s=0.02), [size, size], 1, R, dtype=dt)
            res[dt] = O.run_scan(cells[s].astype(dt), Ko, mpo['gf_params'], mpo['weights'], Ts[s].item(), steps, R,
                                 model, T_static=10, keep_intermediary=False, with_box=True)
        st, fin = res[np.float64]
        # noise worlds are chaotic: FP32 rounding differences grow over the
        # rollout.  The engine must stay within a few times the oracle's own
        # FP32-vs-FP64 spread.
        spread = np.abs(res[np.float32][1] - fin).max()
        for engine, (sd, fin_e) in outs.items():
            fe = fin_e[s].cpu().numpy()
            assert np.abs(fe - fin).max() <= max(2e-4, 8 * spread), (engine, spread)
            np.testing.assert_array_equal(sd['N'][s].cpu().numpy(), st['N'], err_msg=engine)
            np.testing.assert_array_equal(sd['N_box'][s].cpu().numpy(), st['N_box'], err_msg=engine)
            mass = sd['mass'][s].cpu().numpy()
            assert (np.abs(mass - st['mass']) / np.maximum(np.abs(st['mass']), 1e-3)).max() < 1e-4, engine
            cm = sd['channel_mass'][s].cpu().numpy()
            assert cm.shape == (steps, Ni, 1)


@pytest.mark.parametrize('size', [32, 64, 128])
def test_plain_engine_is_the_resident_step_one_launch_at_a_time(cuda, size):
    # the one-world-per-launch engine runs the resident kernel for one world
    # and one step per launch, chaining the carried shift through global
    # memory: states, statistics, centroids and trajectories must equal the
    # batched resident engine's bit for bit
    dev = torch.device('cuda')
    R, steps, Ns, Ni = {32: 6, 64: 10, 128: 13}[size], 12, 2, 3
    cells = np.stack([patch_init(Ni, size, size // 3, seed=60 + s, scale_range=(0.6, 1.0)) for s in range(Ns)])
    Ks, gfs, ws = [], [], []
    upd = None
    for s, (m, sg) in enumerate([(0.15, 0.015), (0.2, 0.03)]):
        K, mp, u = engine_model(bump_kernel_params(m=m, s=sg), [size, size], 1, R, dev=dev)
        upd = upd or u
        Ks.append(K)
        gfs.append(mp.get_gf_params(dev))
        ws.append(mp.get_kernels_weight_per_channel(dev))
    stats_fn = statistics.ComputeStatsFn([size, size], R, 10)
    outs = {}
    for engine in ('resident', 'plain'):
        outs[engine] = runner.run_scan_mem_optimized(None, torch.from_numpy(cells).to(dev), torch.stack(Ks),
                                                     torch.stack(gfs), torch.stack(ws), torch.tensor([10., 5.]), steps,
                                                     R, upd, stats_fn, engine=engine, with_box=True,
                                                     with_centroid=True)
    (sd_r, fin_r), (sd_p, fin_p) = outs['resident'], outs['plain']
    assert torch.equal(fin_r, fin_p)
    for k in sd_r:
        assert torch.equal(sd_r[k], sd_p[k]), k
    traj = {}
    for engine in ('resident', 'plain'):
        traj[engine] = runner.run_scan(None, torch.from_numpy(cells[0]).to(dev), Ks[0], gfs[0], ws[0],
                                       torch.tensor(10.), steps, R, upd, stats_fn, engine=engine)
    for a, b in zip(traj['resident'][:3], traj['plain'][:3]):
        assert torch.equal(a, b)


def test_partial_items_and_zero_steps(cuda):
    dev = torch.device('cuda')
    size = 32
    cells = patch_init(5, size, 12, seed=5)  # 5 worlds: the last CTA of 8 slices is partial
    K, mp, upd = engine_model(bump_kernel_params(), [size, size], 1, 6, dev=dev)
    stats_fn = statistics.ComputeStatsFn([size, size], 6, 10)
    sd, fin = runner.run_scan_mem_optimized(None, torch.from_numpy(cells[None]).to(dev), K[None],
                                            mp.get_gf_params(dev)[None], mp.get_kernels_weight_per_channel(dev)[None],
                                            torch.tensor([10.]), 16, 6, upd, stats_fn, engine='resident')
    st, fo = _oracle_rollout(bump_kernel_params(), [size, size], 1, 6, 10, cells, 16)
    assert np.abs(fin[0].cpu().numpy() - fo).max() < 1e-4
    sd0, fin0 = runner.run_scan_mem_optimized(None, torch.from_numpy(cells[None]).to(dev), K[None],
                                              mp.get_gf_params(dev)[None],
                                              mp.get_kernels_weight_per_channel(dev)[None], torch.tensor([10.]), 0, 6,
                                              upd, stats_fn)
    np.testing.assert_array_equal(fin0[0].cpu().numpy(), cells)
    assert float(sd0['N'].sum()) == 0.0


def test_trajectory_outputs_match_oracle(cuda):
    dev = torch.device('cuda')
    cfg, init, _ = golden_case('orbium')
    cells, Ko, mpo = golden_world(cfg, init)
    model = O.Model(mpo)
    cs_o, fs_o, ps_o, st_o = O.run_scan(cells, Ko, mpo['gf_params'], mpo['weights'], 10, 8, 13, model)
    K, mp, upd = engine_model(cfg['kernels_params'], cfg['world_size'], 1, 13, dev=dev)
    stats_fn = statistics.ComputeStatsFn(cfg['world_size'], 13, 10)
    for engine in ('resident', 'streamed'):
        cs, fs, ps, st = runner.run_scan(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev),
                                         mp.get_kernels_weight_per_channel(dev), torch.tensor(10.), 8, 13, upd,
                                         stats_fn, engine=engine)
        assert np.abs(cs.cpu().numpy() - cs_o).max() < 1e-5
        assert np.abs(ps.cpu().numpy() - ps_o).max() < 2e-6
        assert np.abs(fs.cpu().numpy() - fs_o).max() < 2e-4
        for k in statistics.STAT_KEYS:
            a, b = st[k].cpu().numpy(), st_o[k]
            assert a.shape == b.shape, k
            # the *_volume statistics count cells above EPSILON=1e-7; far from the
            # creature the FFT potential is round-off noise of that size, so a
            # few cells may flip between two FP32 implementations
            atol = 8 / 13.**2 if k.endswith('volume') or k.endswith('density') else 1e-4
            assert np.allclose(a, b, rtol=1e-4, atol=atol), (engine, k, np.abs(a - b).max())
        assert np.abs(st['N'].cpu().numpy() - st_o['N']).max() == 0


@pytest.mark.parametrize('size', [32, 64, 128, 256, 512])
def test_streamed_multichannel_status_word_and_engines_agree(cuda, size):
    # the staged (TMA / bulk) copies of the streamed engine all land: the
    # workspace status word stays 0, and the multi-channel rollout matches the
    # FP32 oracle step for step
    dev = torch.device('cuda')
    C, steps, R = 2, 6, size / 8
    kp = random_multichannel_params(C, 2, seed=size, R_range=(size / 16, size / 8), world_R=R)
    K, mp, upd = engine_model(kp, [size, size], C, R, dev=dev)
    cells = np.zeros((1, 3, C, size, size), np.float32)
    rng = np.random.Generator(np.random.PCG64(size))
    lo, p = size // 4, size // 2
    cells[..., lo:lo + p, lo:lo + p] = rng.random((1, 3, C, p, p), dtype=np.float32)
    stats_fn = statistics.ComputeStatsFn([size, size], R, 5)
    sd, fin = runner.run_scan_mem_optimized(None, torch.from_numpy(cells).to(dev), K[None], mp.get_gf_params(dev)[None],
                                            mp.get_kernels_weight_per_channel(dev)[None], torch.tensor([5.]), steps, R,
                                            upd, stats_fn, engine='streamed', check_status=True)
    Ko, mpo, model = oracle_model(kp, [size, size], C, R)
    st, fo = O.run_scan(cells[0], Ko, mpo['gf_params'], mpo['weights'], 5., steps, R, model, keep_intermediary=False)
    assert np.abs(fin[0].cpu().numpy() - fo).max() <= 1e-4
    np.testing.assert_array_equal(sd['N'][0].cpu().numpy(), st['N'])


def test_stop_count_equals_sequential_scan_of_engine_stats(cuda):
    # N from the warp-parallel heuristics kernel must equal leniax's sequential
    # check_heuristics scan (restated in the oracle) over the engine's own
    # statistics, for long rollouts where the monotone and mass-volume
    # counters can run past 128
    dev = torch.device('cuda')
    size, R, steps = 64, 10, 400
    cells = np.stack([patch_init(6, size, 24, seed=40 + s, scale_range=(0.3, 1.0)) for s in range(3)])
    Ks, gfs, ws = [], [], []
    upd = None
    for s, (m, sg) in enumerate([(0.15, 0.02), (0.12, 0.03), (0.2, 0.04)]):
        K, mp, u = engine_model(bump_kernel_params(m=m, s=sg), [size, size], 1, R, dev=dev)
        upd = upd or u
        Ks.append(K)
        gfs.append(mp.get_gf_params(dev))
        ws.append(mp.get_kernels_weight_per_channel(dev))
    stats_fn = statistics.ComputeStatsFn([size, size], R, 10)
    sd, _ = runner.run_scan_mem_optimized(None, torch.from_numpy(cells).to(dev), torch.stack(Ks), torch.stack(gfs),
                                          torch.stack(ws), torch.tensor([10., 10., 10.]), steps, R, upd, stats_fn)
    for s in range(3):
        st = {k: v[s].cpu().numpy() for k, v in sd.items() if k != 'N'}
        st['channel_mass'] = st['channel_mass']  # [T, Ni, C]
        cont = O.check_heuristics(st)
        np.testing.assert_array_equal(sd['N'][s].cpu().numpy(), cont.sum(axis=0))


@pytest.mark.parametrize('size', [32, 64])
def test_run_scan_mem_optimized_3d_matches_oracle(cuda, size):
    # 3D worlds through lgx_run's one-world-per-CTA engine (the plane-fused
    # items): final cells within a few times the oracle's FP32-vs-FP64 spread,
    # identical N and N_box, mass and centroid close
    from leniax_gb300 import _lib
    dev = torch.device('cuda')
    Ns, Ni, steps, R = 2, 3, 16, size / 6
    rng = np.random.Generator(np.random.PCG64(size))
    cells = np.zeros((Ns, Ni, 1, size, size, size), np.float32)
    p, lo = size // 3, (size - size // 3) // 2
    cells[..., lo:lo + p, lo:lo + p, lo:lo + p] = rng.random((Ns, Ni, 1, p, p, p), dtype=np.float32)
    ms = [0.15, 0.22]
    Ks, gfs, ws = [], [], []
    upd = None
    for s in range(Ns):
        K, mp, u = engine_model(bump_kernel_params(m=ms[s], s=0.03), [size] * 3, 1, R, dev=dev)
        upd = upd or u
        Ks.append(K)
        gfs.append(mp.get_gf_params(dev))
        ws.append(mp.get_kernels_weight_per_channel(dev))
    Ts = torch.tensor([10., 5.])
    stats_fn = statistics.ComputeStatsFn([size] * 3, R, 10)
    m = upd.model
    assert _lib.load().lgx_select_engine(m.plan.handle, Ns, Ni, 0) == _lib.ENGINES['cta']
    sd, fin = runner.run_scan_mem_optimized(None, torch.from_numpy(cells).to(dev), torch.stack(Ks), torch.stack(gfs),
                                            torch.stack(ws), Ts, steps, R, upd, stats_fn, with_box=True,
                                            with_centroid=True)
    for s in range(Ns):
        res = {}
        for dt in (np.float32, np.float64):
            Ko, mpo, model = oracle_model(bump_kernel_params(m=ms[s], s=0.03), [size] * 3, 1, R, dtype=dt)
            res[dt] = O.run_scan(cells[s].astype(dt), Ko, mpo['gf_params'], mpo['weights'], Ts[s].item(), steps, R,
                                 model, T_static=10, keep_intermediary=False, with_box=True)
        st, f64 = res[np.float64]
        spread = np.abs(res[np.float32][1] - f64).max()
        assert np.abs(fin[s].cpu().numpy() - f64).max() <= max(2e-4, 8 * spread)
        np.testing.assert_array_equal(sd['N'][s].cpu().numpy(), st['N'])
        np.testing.assert_array_equal(sd['N_box'][s].cpu().numpy(), st['N_box'])
        mass, m64, m32 = sd['mass'][s].cpu().numpy(), st['mass'], res[np.float32][0]['mass']
        assert (np.abs(mass - m64) <= np.maximum(1e-4 * np.abs(m64), 8 * np.abs(m32 - m64)) + 1e-7).all()
        cen, c64 = sd['mass_centroid'][s].cpu().numpy(), st['mass_centroid']
        d = np.abs(cen - c64)
        d = np.minimum(d, size - d)
        alive = m64 > 1e-3
        assert (d[alive] <= 1e-3 * size).all()


def _unfed_channel_params():
    # C = 2, K = 3: every kernel writes channel 0, so channel 1 gets no field
    # (its state only moves by dt * 0); weighted_sum mode keeps the field finite
    base = dict(k_slug='circle_2d', kf_slug='gauss_bump', kf_params=[1.0], gf_slug='gaussian', c_out=0)
    return [dict(base, k_params=[1.0, [1.0]], gf_params=[0.15, 0.015], h=0.5, c_in=0),
            dict(base, k_params=[0.6, [0.5, 1.0]], gf_params=[0.25, 0.03], h=0.3, c_in=1),
            dict(base, k_params=[0.8, [1.0]], gf_params=[0.2, 0.02], h=0.2, c_in=0)]


@pytest.mark.parametrize('size', [64, 128])
def test_streamed_channel_without_incoming_kernels(cuda, size):
    # the streamed row inverse fetches an unfed channel's state rows outside
    # the kernel items (no item of that channel starts its copy)
    R = 13
    rng = np.random.Generator(np.random.PCG64(size + 5))
    cells = np.zeros((2, 2, size, size), np.float32)
    lo = size // 4
    cells[:, :, lo:3 * lo, lo:3 * lo] = rng.random((2, 2, 2 * lo, 2 * lo), dtype=np.float32)
    (s, f, p), (so, fo, po) = single_step_case(_unfed_channel_params(), [size, size], 2, R, cells, 10, average=False)
    assert np.abs(p - po).max() < 2e-6
    assert np.abs(s - so).max() <= STEP_TOL
    assert np.abs(f - fo).max() < 2e-4
    assert np.abs(f[:, 1]).max() == 0.0  # channel 1: no field
    # a short rollout through lgx_run (fused next-step row FFTs of both channels)
    dev = torch.device('cuda')
    K, mp, upd = engine_model(_unfed_channel_params(), [size, size], 2, R, average=False, dev=dev)
    Ko, mpo, model = oracle_model(_unfed_channel_params(), [size, size], 2, R, average=False)
    steps = 4
    _, fin = runner.run_scan_mem_optimized(None, torch.from_numpy(cells[None]).to(dev), K[None],
                                           mp.get_gf_params(dev)[None], mp.get_kernels_weight_per_channel(dev)[None],
                                           torch.tensor([10.]), steps, R, upd,
                                           statistics.ComputeStatsFn([size, size], R, 10), engine='streamed',
                                           check_status=True)
    for i in range(2):
        _, fo_i = O.run_scan(cells[i:i + 1], Ko, mpo['gf_params'], mpo['weights'], 10, steps, R, model,
                             keep_intermediary=False)
        assert np.abs(fin[0, i].cpu().numpy() - fo_i[0]).max() <= 4 * STEP_TOL


@pytest.mark.parametrize('size', [32, 64])
def test_3d_update_single_step_matches_oracle(cuda, size):
    # core.update on 3D worlds runs one step of the one-world-per-CTA item,
    # field and potential as its step-0 trajectory; scalar and per-world dt
    R = size / 6
    rng = np.random.Generator(np.random.PCG64(size + 3))
    cells = np.zeros((3, 1, size, size, size), np.float32)
    p, lo = size // 3, (size - size // 3) // 2
    cells[..., lo:lo + p, lo:lo + p, lo:lo + p] = rng.random((3, 1, p, p, p), dtype=np.float32)
    (s, f, pt), (so, fo, po) = single_step_case(bump_kernel_params(s=0.03), [size] * 3, 1, R, cells, 10)
    assert np.abs(pt - po).max() < 5e-6
    assert np.abs(s - so).max() <= STEP_TOL
    assert np.abs(f - fo).max() < 2e-4
    dev = torch.device('cuda')
    K, mp, upd = engine_model(bump_kernel_params(s=0.03), [size] * 3, 1, R, dev=dev)
    Ko, mpo, model = oracle_model(bump_kernel_params(s=0.03), [size] * 3, 1, R)
    dts = np.array([0.1, 0.2, 0.05], np.float32)
    s2, _, _ = upd(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev),
                   mp.get_kernels_weight_per_channel(dev), torch.from_numpy(dts).to(dev))
    for i in range(3):
        so_i, _, _ = O.update(cells[i:i + 1], Ko, mpo['gf_params'], mpo['weights'], dts[i], model)
        assert np.abs(s2[i:i + 1].cpu().numpy() - so_i).max() <= STEP_TOL


def test_3d_run_scan_trajectories_match_oracle(cuda):
    dev = torch.device('cuda')
    size, R, steps = 32, 5.0, 6
    rng = np.random.Generator(np.random.PCG64(11))
    cells = np.zeros((1, 1, size, size, size), np.float32)
    cells[..., 11:21, 11:21, 11:21] = rng.random((1, 1, 10, 10, 10), dtype=np.float32)
    K, mp, upd = engine_model(bump_kernel_params(s=0.03), [size] * 3, 1, R, dev=dev)
    Ko, mpo, model = oracle_model(bump_kernel_params(s=0.03), [size] * 3, 1, R)
    cs_o, fs_o, ps_o, st_o = O.run_scan(cells, Ko, mpo['gf_params'], mpo['weights'], 10, steps, R, model)
    cs, fs, ps, st = runner.run_scan(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev),
                                     mp.get_kernels_weight_per_channel(dev), torch.tensor(10.), steps, R, upd,
                                     statistics.ComputeStatsFn([size] * 3, R, 10))
    assert tuple(cs.shape) == cs_o.shape and tuple(ps.shape) == ps_o.shape
    assert np.abs(cs.cpu().numpy() - cs_o).max() < 2e-5
    assert np.abs(ps.cpu().numpy() - ps_o).max() < 5e-6
    assert np.abs(fs.cpu().numpy() - fs_o).max() < 5e-4
    assert np.abs(st['N'].cpu().numpy() - st_o['N']).max() == 0