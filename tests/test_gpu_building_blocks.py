"""The step's building blocks on the device against the oracle: potentials
(``core.get_potential_fft`` core.py:52-102, ``core.get_potential``
core.py:105-146 with the reference's conv KAT), growth functions
(growth_functions.py), fields (``core.get_field`` core.py:163-199 with
``weighted_sum`` / ``weighted_mean`` core.py:202-242), state updates
(core.py:245-319), the builders of helpers.py:430-516, and their
composition against the fused step."""
import numpy as np
import pytest
import torch

from leniax_gb300 import core, growth_functions, helpers, kernels
from oracle import lenia_oracle as O
from tests.cases import golden_case, golden_world

pytestmark = pytest.mark.gpu


def _dev(x, dev):
    return torch.from_numpy(np.ascontiguousarray(x)).to(dev)


@pytest.mark.parametrize('name', ['orbium', 'aquarium'])
def test_get_potential_fft_matches_the_oracle(cuda, name):
    cfg, init, _ = golden_case(name)
    cells, K, mp = golden_world(cfg, init)
    tc = O.tc_indices_of(mp['true_channels'])
    po = O.get_potential_fft(cells, K, tc)
    p = core.get_potential_fft(_dev(cells, cuda), _dev(K.astype(np.complex64), cuda), tc)
    assert p.shape == po.shape
    assert np.abs(p.cpu().numpy() - po).max() < 1e-5


def test_get_potential_conv_kat(cuda):
    # tests/test_core.py:55-103 through the builder of helpers.py:430-487
    cells = np.ones([1, 2, 2, 2], np.float32)
    cells[0, 0] = 0.1
    cells[0, 1] = 0.2
    K = np.ones([4, 1, 3, 3], np.float32)
    K[0], K[1], K[2], K[3] = 0.1, 0.2, 0.3, 0
    fn = helpers.build_get_potential_fn(K.shape, [True, True, True, False], fft=False)
    pot = fn(_dev(cells, cuda), _dev(K, cuda))
    true = np.ones([1, 3, 2, 2], np.float32)
    true[0, 0], true[0, 1], true[0, 2] = 0.09, 0.18, 0.54
    np.testing.assert_allclose(pot.cpu().numpy(), true, rtol=1e-6)


def test_get_potential_direct_matches_the_oracle(cuda):
    cfg, init, _ = golden_case('aquarium')
    cells, _, mp = golden_world(cfg, init)
    Kc, mpo = O.get_kernels_and_mapping(cfg['kernels_params'], cfg['world_size'], cfg['nb_channels'], cfg['R'], False,
                                        np.float32)
    tc = O.tc_indices_of(mpo['true_channels'])
    po = O.get_potential_conv(cells, Kc, O.conv_padding(Kc.shape), tc)
    fn = helpers.build_get_potential_fn(Kc.shape, mpo['true_channels'], fft=False)
    p = fn(_dev(cells, cuda), _dev(Kc, cuda))
    assert np.abs(p.cpu().numpy() - po).max() < 1e-5


@pytest.mark.parametrize('slug', sorted(growth_functions.register))
def test_growth_functions_match_the_oracle(cuda, slug):
    rng = np.random.Generator(np.random.PCG64(11))
    X = rng.random((3, 40, 40), dtype=np.float32) * 0.5
    params = np.array([0.2, 0.05], np.float32)
    got = growth_functions.register[slug](_dev(params, cuda), _dev(X, cuda)).cpu().numpy()
    want = O.GF_REGISTER[slug](params, X)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize('average', [True, False])
def test_get_field_and_weighting_match_the_oracle(cuda, average):
    rng = np.random.Generator(np.random.PCG64(12))
    slugs = ['gaussian', 'poly_quad4', 'triangle']
    pot = rng.random((2, 3, 24, 20), dtype=np.float32) * 0.4
    gf = np.array([[0.15, 0.03], [0.2, 0.04], [0.1, 0.05]], np.float32)
    w = np.array([[1.0, 0.5, 0.0], [0.0, 0.25, 2.0]], np.float32)
    want = O.get_field(pot, gf, w, slugs, average)
    weighted = core.weighted_mean if average else core.weighted_sum
    got = core.get_field(_dev(pot, cuda), _dev(gf, cuda), _dev(w, cuda),
                         tuple(growth_functions.register[s] for s in slugs), weighted)
    np.testing.assert_allclose(got.cpu().numpy(), want, rtol=1e-5, atol=1e-6)
    # the merge alone, and a caller's own merge over the device growth fields
    fields = np.stack([O.GF_REGISTER[s](gf[i], pot[:, i]) for i, s in enumerate(slugs)], axis=1)
    merged = weighted(_dev(fields, cuda), _dev(w, cuda)).cpu().numpy()
    ref = O.weighted_mean(fields, w) if average else O.weighted_sum(fields, w)
    np.testing.assert_allclose(merged, ref, rtol=1e-5, atol=1e-6)
    own = core.get_field(_dev(pot, cuda), _dev(gf, cuda), _dev(w, cuda), tuple(slugs),
                         lambda f, ww: torch.einsum('ck,nk...->nc...', ww, f))
    np.testing.assert_allclose(own.cpu().numpy(), O.weighted_sum(fields, w), rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize('slug', ['v1', 'v2', 'simple'])
def test_state_functions_match_the_oracle(cuda, slug):
    rng = np.random.Generator(np.random.PCG64(13))
    state = rng.random((3, 2, 16, 16), dtype=np.float32)
    field = rng.random((3, 2, 16, 16), dtype=np.float32) * 2 - 1
    fn = {'v1': core.get_state, 'v2': core.get_state_v2, 'simple': core.get_state_simple}[slug]
    for dt in (np.float32(0.1), np.array([0.1, 0.2, 0.5], np.float32)):
        got = fn(None, _dev(state, cuda), _dev(field, cuda), _dev(np.asarray(dt), cuda)).cpu().numpy()
        want = O.STATE_REGISTER[slug](state, field, dt)
        np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-7)


def test_building_blocks_compose_to_the_step(cuda):
    # potential -> field -> state through the builders equals the fused update
    cfg, init, _ = golden_case('aquarium')
    cells, _, _ = golden_world(cfg, init)
    dev = cuda
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in cfg['kernels_params']], cfg['world_size'],
                                            cfg['nb_channels'], cfg['R'], True, dev)
    upd = helpers.build_update_fn(K.shape, mp, 'v1', cfg['weighted_average'])
    pot_fn = helpers.build_get_potential_fn(K.shape, mp.true_channels)
    field_fn = helpers.build_get_field_fn(mp.cin_gfs, cfg['weighted_average'])
    c = _dev(cells, dev)
    gf, w = mp.get_gf_params(dev), mp.get_kernels_weight_per_channel(dev)
    dt = torch.tensor(1. / cfg['T'], device=dev)
    s, f, p = upd(None, c, K, gf, w, dt)
    p2 = pot_fn(c, K)
    f2 = field_fn(p2, gf, w)
    s2 = core.get_state(None, c, f2, dt)
    assert torch.abs(p2 - p).max().item() < 1e-6
    assert torch.abs(f2 - f).max().item() < 1e-4
    assert torch.abs(s2 - s).max().item() < 1e-5
