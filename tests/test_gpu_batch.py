"""Uneven batch engine (lgx_batch_run) against the oracle, world by world.

Every world of a mixed batch (2D 32^2 / 64^2 / 128^2 / 256^2, 3D 32^3 / 64^3,
per-world R, m, s, T) must reproduce the oracle's rollout of that world alone
(run_scan, runner.py:119-164): final cells within a few times the oracle's own
FP32-vs-FP64 spread, identical N and N_box, mass and centroid close."""
import numpy as np
import pytest
import torch

from leniax_gb300 import batch as lbatch
from oracle import lenia_oracle as O
from tests.cases import bump_kernel_params

pytestmark = pytest.mark.gpu

# (nb_dims, size, n_worlds, R range): partial items for the 8- and 4-world
# resident items, several big worlds per class
SPEC = [(2, 32, 9, (5, 8)), (2, 64, 5, (8, 12)), (2, 128, 2, (10, 15)), (2, 256, 2, (13, 26)), (3, 32, 2, (5, 8)),
        (3, 64, 1, (8, 12))]


def _init(n, nd, size, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    p = size // 3
    lo = (size - p) // 2
    cells = np.zeros((n, ) + (size, ) * nd, dtype=np.float32)
    noise = rng.random((n, ) + (p, ) * nd, dtype=np.float32) * rng.uniform(0.5, 1.0, size=(n, ) + (1, ) * nd).astype(
        np.float32)
    cells[(slice(None), ) + (slice(lo, lo + p), ) * nd] = noise
    return cells


def _world_params(spec, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for nd, size, n, (rlo, rhi) in spec:
        R = rng.integers(rlo, rhi + 1, size=n).astype(np.float32)
        m = rng.uniform(0.12, 0.3, size=n).astype(np.float32)
        s = rng.uniform(0.015, 0.045, size=n).astype(np.float32)
        T = rng.choice(np.array([5., 10., 20.], dtype=np.float32), size=n)
        out.append((R, m, s, T))
    return out


def _classes(dev, spec, params, seed=0, slug='gaussian'):
    classes, cells = [], []
    for ci, ((nd, size, n, _), (R, m, s, T)) in enumerate(zip(spec, params)):
        c0 = _init(n, nd, size, seed + ci)
        kp = bump_kernel_params()[0]
        K = lbatch.world_spectra([size] * nd, R, kp, dev)
        classes.append(
            lbatch.WorldClass(cells0=torch.from_numpy(c0).to(dev), K=K,
                              gf_params=torch.from_numpy(np.stack([m, s], 1)).to(dev), weights=torch.ones(n, device=dev),
                              T=torch.from_numpy(T).to(dev), R=torch.from_numpy(R).to(dev), gf_slug=slug))
        cells.append(c0)
    return classes, cells


def _oracle_world(nd, size, c0, R, m, s, T, steps, dtype, slug='gaussian'):
    kp = bump_kernel_params(m=float(m), s=float(s))
    kp[0]['gf_slug'] = slug
    Ko, mp = O.get_kernels_and_mapping([dict(p) for p in kp], [size] * nd, 1, float(R), True, dtype)
    model = O.Model(mp, 'v1', True)
    cells = c0[None, None].astype(dtype)
    return O.run_scan(cells, Ko, mp['gf_params'], mp['weights'], float(T), steps, float(R), model,
                      keep_intermediary=False, with_box=True)


def test_uneven_batch_matches_oracle_per_world(cuda):
    dev = torch.device('cuda')
    steps = 32
    params = _world_params(SPEC, 7)
    classes, cells = _classes(dev, SPEC, params)
    b = lbatch.UnevenBatch(classes, steps)
    b.run()
    res = b.results()
    assert b.status() == 0  # every staged copy landed
    for ci, ((nd, size, n, _), (R, m, s, T)) in enumerate(zip(SPEC, params)):
        out = res[ci]
        fin = out['final'].cpu().numpy()
        st = {k: v.cpu().numpy() for k, v in out['stats'].items()}
        for w in range(n):
            o64, f64 = _oracle_world(nd, size, cells[ci][w], R[w], m[w], s[w], T[w], steps, np.float64)
            o32, f32 = _oracle_world(nd, size, cells[ci][w], R[w], m[w], s[w], T[w], steps, np.float32)
            tag = f'{nd}D {size} world {w}'
            spread = np.abs(f32 - f64).max()
            assert np.abs(fin[w] - f64[0, 0]).max() <= max(2e-4, 8 * spread), (tag, spread)
            assert int(st['N'][w, 0]) == int(o64['N'][0]), tag
            assert int(st['N_box'][w, 0]) == int(o64['N_box'][0]), tag
            mass, m64, m32 = st['mass'][w, :, 0], o64['mass'][:, 0], o32['mass'][:, 0]
            tol = np.maximum(1e-4 * np.abs(m64), 8 * np.abs(m32 - m64)) + 1e-7
            assert (np.abs(mass - m64) <= tol).all(), tag
            alive = m64 > 1e-3
            cen, c64 = st['mass_centroid'][w, :, 0], o64['mass_centroid'][:, 0]
            d = np.abs(cen - c64)
            d = np.minimum(d, size - d)
            assert (d[alive] <= 1e-3 * size).all(), tag


def test_queue_order_and_grid_do_not_change_results(cuda):
    # every world is computed by exactly one CTA from its own inputs: the
    # schedule must not change a single bit
    dev = torch.device('cuda')
    spec = [(2, 64, 6, (8, 12)), (2, 256, 3, (13, 20)), (3, 32, 3, (5, 8))]
    params = _world_params(spec, 3)
    classes, _ = _classes(dev, spec, params)
    outs = []
    for kw in (dict(order='largest_first'), dict(order='as_given', grid=5),
               dict(order='explicit', class_order=[2, 0, 1], grid=3)):
        b = lbatch.UnevenBatch(classes, 12, **kw)
        b.run()
        outs.append([r['final'].clone() for r in b.results()] + [b.outputs[i]['stats'].clone() for i in range(3)])
    for other in outs[1:]:
        for a, c in zip(outs[0], other):
            assert torch.equal(a, c)


def test_line_group_variants_agree(cuda):
    dev = torch.device('cuda')
    spec = [(3, 32, 2, (5, 8)), (3, 64, 1, (8, 12))]
    params = _world_params(spec, 11)
    classes, _ = _classes(dev, spec, params)
    fins = []
    for lg in (2, 4):
        b = lbatch.UnevenBatch(classes, 8, line_group=lg)
        b.run()
        fins.append([r['final'].clone() for r in b.results()])
    for a, c in zip(*fins):
        assert (a - c).abs().max().item() <= 1e-5


def test_graph_replay_matches_launch_and_sees_new_inputs(cuda):
    dev = torch.device('cuda')
    spec = [(2, 32, 8, (5, 8)), (2, 128, 2, (10, 15)), (3, 32, 1, (5, 8))]
    params = _world_params(spec, 5)
    classes, _ = _classes(dev, spec, params)
    ref = lbatch.UnevenBatch(classes, 10)
    ref.run()
    want = [r['final'].clone() for r in ref.results()]
    g = lbatch.UnevenBatch(classes, 10).capture()
    g.run()
    torch.cuda.synchronize()
    for a, r in zip(want, g.results()):
        assert torch.equal(a, r['final'])
    # next generation: new initial cells written in place, graph replayed
    for inp in g.inputs:
        inp['cells0'].mul_(0.5)
    g.run()
    ref2 = lbatch.UnevenBatch([lbatch.WorldClass(**{**c.__dict__, 'cells0': inp['cells0']})
                               for c, inp in zip(classes, g.inputs)], 10)
    ref2.run()
    torch.cuda.synchronize()
    for a, b in zip(ref2.results(), g.results()):
        assert torch.equal(a['final'], b['final'])


def test_generic_growth_and_state_paths(cuda):
    # poly_quad4 uses its specialised epilogue; step growth the generic one
    dev = torch.device('cuda')
    spec = [(2, 64, 4, (8, 10)), (2, 256, 1, (14, 16)), (3, 32, 1, (5, 6))]
    for slug in ('poly_quad4', 'step'):
        params = _world_params(spec, 13)
        classes, cells = _classes(dev, spec, params, slug=slug)
        b = lbatch.UnevenBatch(classes, 6)
        b.run()
        res = b.results()
        for ci, ((nd, size, n, _), (R, m, s, T)) in enumerate(zip(spec, params)):
            fin = res[ci]['final'].cpu().numpy()
            for w in range(n):
                o32, f32 = _oracle_world(nd, size, cells[ci][w], R[w], m[w], s[w], T[w], 6, np.float32, slug)
                o64, f64 = _oracle_world(nd, size, cells[ci][w], R[w], m[w], s[w], T[w], 6, np.float64, slug)
                spread = np.abs(f32 - f64).max()
                assert np.abs(fin[w] - f64[0, 0]).max() <= max(2e-4, 8 * spread), (slug, nd, size, w)


def test_autotuner_picks_a_candidate_and_caches_it(cuda, tmp_path, monkeypatch):
    from leniax_gb300 import autotune
    monkeypatch.setenv('LGX_AUTOTUNE_CACHE', str(tmp_path / 'tune.json'))
    dev = torch.device('cuda')
    spec = [(2, 64, 8, (8, 12)), (2, 256, 2, (13, 20)), (3, 32, 2, (5, 8))]
    classes, _ = _classes(dev, spec, _world_params(spec, 17))
    res = autotune.tune(classes, 16, probe_steps=2, reps=1)
    assert res['settings'] in [{k: v for k, v in c.items() if k != 'ms'} for c in res['candidates']]
    s1 = autotune.tuned_settings(classes, 16)
    s2 = autotune.tuned_settings(classes, 16)
    assert s1 == s2 and (tmp_path / 'tune.json').exists()


def test_tuned_settings_with_other_shapes_keep_the_results(cuda, tmp_path, monkeypatch):
    # classes outside the persistent shapes are not timed; the tuned class
    # order indexes the full class list; tuned and untuned batches agree
    # (the untuned one uses the tuned 3D line width: widths differ in
    # rounding, within the line-width test's 1e-5)
    from leniax_gb300 import autotune
    monkeypatch.setenv('LGX_AUTOTUNE_CACHE', str(tmp_path / 'tune.json'))
    dev = torch.device('cuda')
    spec = [(2, 45, 2, (6, 9)), (2, 64, 8, (8, 12)), (3, 24, 2, (4, 6)), (3, 32, 2, (5, 8))]
    classes, _ = _classes(dev, spec, _world_params(spec, 23))
    res = autotune.tune(classes, 8, probe_steps=2, reps=1)
    assert res['item_ms'][0] is None and res['item_ms'][2] is None
    assert res['item_ms'][1] > 0 and res['item_ms'][3] > 0
    if 'class_order' in res['settings']:
        assert sorted(res['settings']['class_order']) == [1, 3]
    tuned = lbatch.UnevenBatch(classes, 8, **res['settings']).run().results()
    plain = lbatch.UnevenBatch(classes, 8, line_group=res['settings']['line_group']).run().results()
    for a, b in zip(tuned, plain):
        assert (a['final'] - b['final']).abs().max().item() <= 1e-5
        assert torch.equal(a['stats']['N'], b['stats']['N'])


def test_classes_of_any_shape_run_beside_the_persistent_launch(cuda):
    # shapes the persistent launch does not take (100^2, odd 45^2, prime-
    # factored 66^2, 3D 24^3) run through lgx_run with every world its own
    # solution and its own statistics R and T; every world matches the
    # oracle run alone, and a graph replay reproduces a launch
    dev = torch.device('cuda')
    spec = [(2, 64, 3, (8, 12)), (2, 100, 2, (10, 16)), (2, 45, 2, (6, 9)), (2, 66, 2, (8, 12)),
            (3, 24, 2, (4, 6))]
    params = _world_params(spec, 11)
    classes, cells = _classes(dev, spec, params)
    steps = 16
    b = lbatch.UnevenBatch(classes, steps)
    b.run()
    res = b.results()
    assert b.status() == 0
    for ci, ((nd, size, n, _), (R, m, s, T)) in enumerate(zip(spec, params)):
        fin = res[ci]['final'].cpu().numpy()
        st = {k: v.cpu().numpy() for k, v in res[ci]['stats'].items()}
        for w in range(n):
            o64, f64 = _oracle_world(nd, size, cells[ci][w], R[w], m[w], s[w], T[w], steps, np.float64)
            o32, f32 = _oracle_world(nd, size, cells[ci][w], R[w], m[w], s[w], T[w], steps, np.float32)
            tag = f'{nd}D {size} world {w}'
            spread = np.abs(f32 - f64).max()
            assert np.abs(fin[w] - f64[0, 0]).max() <= max(2e-4, 8 * spread), (tag, spread)
            assert int(st['N'][w, 0]) == int(o64['N'][0]), tag
            assert int(st['N_box'][w, 0]) == int(o64['N_box'][0]), tag
            mass, m64, m32 = st['mass'][w, :, 0], o64['mass'][:, 0], o32['mass'][:, 0]
            tol = np.maximum(1e-4 * np.abs(m64), 8 * np.abs(m32 - m64)) + 1e-7
            assert (np.abs(mass - m64) <= tol).all(), tag
            # per-world R and T reach the statistics (mass_volume counts / R^2)
            mv, mv64 = st['mass_volume'][w, :, 0], o64['mass_volume'][:, 0]
            assert np.allclose(mv, mv64, rtol=1e-4, atol=8 / float(R[w])**2), tag
    want = [r['final'].clone() for r in res]
    g = lbatch.UnevenBatch(classes, steps).capture()
    g.run()
    torch.cuda.synchronize()
    for a, r in zip(want, g.results()):
        assert torch.equal(a, r['final'])
