"""QD evaluation glue and device initial states on the GPU."""
import base64
import gzip

import numpy as np
import pytest
import torch

from leniax_gb300 import helpers, initializations, kernels, qd, runner, statistics
from leniax_gb300.constant import NB_CHARS
from oracle import lenia_oracle as O

pytestmark = pytest.mark.gpu


def qd_config(init_slug='perlin', steps=48, nb_init_search=4):
    return {
        'world_params': {'nb_channels': 1, 'R': 13, 'T': 10.0},
        'render_params': {'world_size': [128, 128]},
        'run_params': {'max_run_iter': steps, 'nb_init_search': nb_init_search, 'seed': 1},
        'algo': {'init_slug': init_slug},
        'kernels_params': [{
            'k_slug': 'circle_2d', 'k_params': [1.0, [1.0]], 'kf_slug': 'gauss_bump', 'kf_params': [4.0],
            'gf_slug': 'gaussian', 'gf_params': [0.15, 0.015], 'h': 1.0, 'c_in': 0, 'c_out': 0
        }],
        'genotype': [{'key': 'kernels_params.0.gf_params.0', 'domain': [0.1, 0.3], 'type': 'float'},
                     {'key': 'kernels_params.0.gf_params.1', 'domain': [0.01, 0.05], 'type': 'float'}],
        'phenotype': ['behaviours.mass', 'behaviours.mass_volume'],
    }


@pytest.mark.parametrize('kind', ['perlin', 'cropped_perlin'])
@pytest.mark.parametrize('world,R', [([128, 128], 13), ([96, 160], 7.5)])
def test_perlin_states_match_oracle_for_a_given_gradient_field(cuda, kind, world, R):
    # the device construction (noise, per-state normalisation, scaling,
    # compressible rounding, crop) against the oracle's restatement of
    # perlin.py:16-71 / initializations.py:35-116 from the same angles
    if kind == 'cropped_perlin' and world != [128, 128]:
        pytest.skip('cropped_perlin is defined on 128 x 128 worlds')
    nb_init, ms = 5, [0.15, 0.3]
    res = O.perlin_res(world, R)
    rng = np.random.Generator(np.random.PCG64(9))
    ang = (rng.random((2, nb_init) + tuple(res)) * 2 * np.pi).astype(np.float32)
    ref_fn = O.perlin_init if kind == 'perlin' else O.cropped_perlin_init
    for comp in (False, True):
        got = initializations.generate(kind, [1, 2], nb_init, world, R, ms, compressible=comp,
                                       angles=torch.from_numpy(ang)).cpu().numpy()
        for w in range(2):
            ref = ref_fn(ang[w].astype(np.float64), world, R, ms[w], compressible=comp)[:, 0]
            if not comp:
                assert np.abs(got[w] - ref).max() <= 2e-6, (kind, world, w)
            else:
                # a value within rounding distance of a half-quantum may round the other way
                quantum = 1 / (NB_CHARS**2 - 1)
                d = np.abs(got[w] - ref)
                assert d.max() <= quantum * 1.001 and (d > 1e-6).mean() < 1e-3, (kind, world, w)


@pytest.mark.parametrize('kind', ['random_uniform', 'perlin', 'cropped_perlin'])
def test_initial_states(cuda, kind):
    nb_init, R = 6, 13
    a = initializations.generate(kind, [11, 12], nb_init, [128, 128], R, [0.15, 0.2]).cpu().numpy()
    b = initializations.generate(kind, [11, 12], nb_init, [128, 128], R, [0.15, 0.2]).cpu().numpy()
    c = initializations.generate(kind, [13, 12], nb_init, [128, 128], R, [0.15, 0.2]).cpu().numpy()
    assert a.shape == (2, nb_init, 128, 128)
    np.testing.assert_array_equal(a, b)  # same seed, same states
    assert not np.array_equal(a[0], c[0]) and np.array_equal(a[1], c[1])
    q = a * (NB_CHARS**2 - 1)
    assert np.abs(q - np.round(q)).max() < 1e-2  # on the make_array_compressible grid
    if kind == 'random_uniform':
        maxv = np.linspace(0.4, 1., nb_init)
        for i in range(nb_init):
            assert a[0, i].min() >= 0 and a[0, i].max() <= maxv[i] + 1e-4 and a[0, i].max() > 0.9 * maxv[i]
            assert abs(a[0, i].mean() - maxv[i] / 2) < 0.01
    else:
        for w, m in enumerate([0.15, 0.2]):
            for i in range(nb_init):
                scale = m + i / nb_init * (min(1., 3 * m) - m)
                x = a[w, i]
                if kind == 'perlin':
                    assert abs(x.min()) < 1e-4 and abs(x.max() - scale) < 1e-3
                    assert x.std() > 0.05 * scale  # a noise field, not a constant
                else:
                    crop, pad = 2 * R, (128 - 2 * R) // 2
                    inner = x[pad:pad + crop, pad:pad + crop]
                    assert np.all(x[:pad] == 0) and np.all(x[pad + crop:] == 0) and inner.max() > 0


def test_dynamic_args_device_kernels_match_host_path(cuda):
    cfg = qd_config()
    inds = [qd.LeniaIndividual(cfg, 5 + i, [0.2 + 0.3 * i, 0.4]) for i in range(3)]
    _, (cells0, K, gf, w, T) = qd.get_dynamic_args(cfg, inds)
    assert tuple(cells0.shape) == (3, 4, 1, 128, 128)
    assert tuple(K.shape) == (3, 1, 1, 1, 128, 128) and K.dtype == torch.complex64
    assert tuple(gf.shape) == (3, 1, 2) and tuple(w.shape) == (3, 1, 1) and tuple(T.shape) == (3, )
    for i, ind in enumerate(inds):
        c = ind.get_config()
        Kh, mp = kernels.get_kernels_and_mapping([dict(p) for p in c['kernels_params']], [128, 128], 1, 13, True)
        assert (K[i, 0] - Kh[0]).abs().max().item() <= 2e-5 * Kh.abs().max().item()
        np.testing.assert_allclose(gf[i].cpu().numpy(), mp.get_gf_params().cpu().numpy())
    # genes reached the growth parameters
    assert abs(gf[1, 0, 0].item() - (0.1 + 0.2 * 0.5)) < 1e-6


def test_eval_fn_fitness_is_max_stop_count(cuda):
    cfg = qd_config(steps=48)
    inds = [qd.LeniaIndividual(cfg, 21 + i, [0.1 + 0.2 * i, 0.3 + 0.1 * i]) for i in range(4)]
    ev = qd.build_eval_lenia_config_mem_optimized_fn(cfg)
    out = ev(inds)
    # the same rollout through the runner
    _, args = qd.get_dynamic_args(cfg, inds, full_spectrum=False)
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in cfg['kernels_params']], [128, 128], 1, 13, True)
    upd = helpers.build_update_fn(K.shape, mp)
    stats, _ = runner.run_scan_mem_optimized(None, *args, 48, 13, upd,
                                             statistics.build_compute_stats_fn(cfg['world_params'],
                                                                               cfg['render_params']))
    N = stats['N'].cpu().numpy()
    for i, ind in enumerate(out):
        assert ind.fitness == N[i].max()
        assert ind.qd_config['algo']['best_init_idxs'] == [int(j) for j in np.nonzero(N[i] == N[i].max())[0]]
        assert len(ind.features) == 2
        b = int(np.argmax(N[i]))
        ns = max(int(ind.fitness), 128)
        m = stats['mass'][i, ns - 128:ns, b].double().mean().item() if ns - 128 < 48 else float('nan')
        assert (np.isnan(m) and np.isnan(ind.features[0])) or abs(ind.features[0] - m) < 1e-9


def test_codec_batch_on_device_states(cuda):
    from leniax_gb300 import loader
    x = initializations.generate('perlin', [3, 4, 5], 2, [64, 64], 5, [0.2] * 3, compressible=False)
    on_dev = loader.compress_batch(x.reshape(6, 1, 64, 64))
    on_host = loader.compress_batch(x.reshape(6, 1, 64, 64).cpu())
    # gzip headers carry the compression time (as leniax's strings do): compare the payloads
    payload = lambda z: gzip.decompress(base64.decodebytes(z.encode('utf-8')))  # noqa: E731
    assert [payload(z) for z in on_dev] == [payload(z) for z in on_host]
    back = loader.decompress_array(on_dev[4], device=x.device)
    assert torch.equal(back, loader.make_array_compressible(x.reshape(6, 1, 64, 64)[4]))
