"""The oracle is pinned to leniax's own golden frames and known-answer tests
(CPU only)."""
import numpy as np
import pytest

from oracle import lenia_oracle as O
from tests.cases import golden_case, golden_world


@pytest.mark.parametrize('name', ['orbium', 'orbium_scutium', 'aquarium'])
def test_oracle_reproduces_leniax_golden_frames(name):
    # leniax tests/test_pipeline.py:35,92,111: assert_array_almost_equal(decimal=4|3)
    cfg, init, last = golden_case(name)
    cells, K, mp = golden_world(cfg, init, np.float32)
    model = O.Model(mp, cfg['get_state_fn_slug'], cfg['weighted_average'])
    cs, _, _, st = O.run_scan(cells, K, mp['gf_params'], mp['weights'], cfg['T'], cfg['max_run_iter'], cfg['R'], model)
    assert cs.shape[0] == cfg['max_run_iter']
    np.testing.assert_array_almost_equal(last, cs[-1, 0], decimal=cfg['decimal'])


def test_oracle_eager_run_matches_scan():
    cfg, init, last = golden_case('orbium')
    cells, K, mp = golden_world(cfg, init)
    model = O.Model(mp)
    cs, _, _, st = O.run_eager(cells, K, mp['gf_params'], mp['weights'], cfg['T'], cfg['max_run_iter'], cfg['R'],
                               model)
    assert len(cs) == 128  # tests/test_pipeline.py:34
    np.testing.assert_array_almost_equal(last, cs[-1, 0], decimal=4)


def test_get_state_kat():
    # tests/test_core.py:159-185
    s1 = np.ones((25, 25), np.float32) * .5
    f1 = np.ones((25, 25), np.float32) * 3
    np.testing.assert_array_almost_equal(O.get_state_v1(s1, f1, np.float32(1. / 3.)), np.ones((25, 25)))
    s2 = np.ones((25, 25), np.float32) * .2
    np.testing.assert_array_almost_equal(O.get_state_v1(s2, f1, np.float32(1. / 6.)), np.ones((25, 25)) * .7)


def test_conv_potential_kat():
    # tests/test_core.py:55-103: 2x2 torus, 2 channels, 3 true kernels of 4 slots
    cells = np.ones([1, 2, 2, 2], np.float32)
    cells[0, 0] = 0.1
    cells[0, 1] = 0.2
    K = np.ones([4, 1, 3, 3], np.float32)
    K[0], K[1], K[2], K[3] = 0.1, 0.2, 0.3, 0
    tc = O.tc_indices_of([True, True, True, False])
    pot = O.get_potential_conv(cells, K, O.conv_padding(K.shape), tc)
    true = np.ones([1, 3, 2, 2], np.float32)
    true[0, 0], true[0, 1], true[0, 2] = 0.09, 0.18, 0.54
    np.testing.assert_allclose(pot, true, rtol=1e-6)


def test_conv_and_fft_potential_agree():
    cfg, init, _ = golden_case('aquarium')
    cells, K, mp = golden_world(cfg, init, np.float64)
    Kc, _ = O.get_kernels_and_mapping(cfg['kernels_params'], cfg['world_size'], cfg['nb_channels'], cfg['R'], False,
                                      np.float64)
    small = cells[:, :, 40:88, 40:88].copy()
    # same kernels on a 128-torus: compare the FFT and direct potentials at full size
    pf = O.get_potential_fft(cells, K, O.tc_indices_of(mp['true_channels']))
    pc = O.get_potential_conv(cells, Kc, O.conv_padding(Kc.shape), O.tc_indices_of(mp['true_channels']))
    assert small.shape[-1] == 48
    np.testing.assert_allclose(pf, pc, atol=1e-9)


def test_mass_volume_heuristic_kat():
    # tests/test_statistics.py:14-31
    R = 13.
    mv = np.array([800, 1600, 2400, 3200]) / R**2
    cnt = np.array([10, 70, O.MASS_VOLUME_STOP_STEP - 1, O.MASS_VOLUME_STOP_STEP])
    cond, nxt = O.mass_volume_heuristic(mv, cnt)
    np.testing.assert_array_equal(cond, [True, True, True, False])
    np.testing.assert_array_equal(nxt, [1, 1, O.MASS_VOLUME_STOP_STEP, O.MASS_VOLUME_STOP_STEP + 1])


def test_monotonic_heuristic_kat():
    # tests/test_statistics.py:33-50
    mass = np.array([1.1, 0.9, 0.9, 0.9])
    sign = np.sign(mass - np.array([1, 1, 1, 1]))
    prev = np.array([1, 1, -1, -1])
    cnt = np.array([40, O.MONOTONIC_STOP_STEP, 30, O.MONOTONIC_STOP_STEP])
    cond, nxt = O.monotonic_heuristic(sign, prev, cnt)
    np.testing.assert_array_equal(cond, [True, True, True, False])
    np.testing.assert_array_equal(nxt, [41, 1, 31, O.MONOTONIC_STOP_STEP + 1])


def test_kernel_shapes():
    # tests/test_kernels.py:12-20 (circle_2d R=5 -> [1, 10, 10]); tests/test_qd.py:88 (FFT K shape)
    k = O.circle_kernel(5, [1., [1.]], 'poly_quad', [4])
    assert k.shape == (1, 10, 10)
    assert abs(k.sum() - 1) < 1e-6
    K, mp = O.get_kernels_and_mapping([{
        'k_slug': 'circle_2d', 'k_params': [1, [1.]], 'kf_slug': 'poly_quad', 'kf_params': [4], 'gf_slug':
        'poly_quad4', 'gf_params': [0.15, 0.015], 'h': 1, 'c_in': 0, 'c_out': 0
    }], [64, 64], 1, 13)
    assert K.shape == (1, 1, 1, 64, 64)


def test_fp32_mode_tracks_fp64_over_rollout():
    cfg, init, _ = golden_case('orbium')
    c32, K32, mp32 = golden_world(cfg, init, np.float32)
    c64, K64, mp64 = golden_world(cfg, init, np.float64)
    a = O.run_scan(c32, K32, mp32['gf_params'], mp32['weights'], 10, 64, 13, O.Model(mp32))[0]
    b = O.run_scan(c64, K64, mp64['gf_params'], mp64['weights'], 10, 64, 13, O.Model(mp64))[0]
    assert np.abs(a[-1] - b[-1]).max() < 1e-4


def test_rle_decoder_shape():
    cfg, init, _ = golden_case('orbium')
    assert init.shape == (1, 20, 20)
    assert 0.0 <= init.min() and init.max() <= 1.0
