"""Cell-state codec (leniax loader.py) round trips, checked with the oracle's
restatement of the reference decoder."""
import base64
import gzip

import numpy as np
import pytest
import torch

from leniax_gb300 import loader
from oracle import lenia_oracle as O


def _cells(seed, shape):
    return torch.from_numpy(np.random.Generator(np.random.PCG64(seed)).random(shape, dtype=np.float32))


@pytest.mark.parametrize('shape', [(1, 64, 64), (3, 32, 48), (2, 8, 8, 8)])
def test_gzip_codec_round_trip_and_reference_decoder(shape):
    x = _cells(len(shape), shape)
    s = loader.compress_array(x)
    want = loader.make_array_compressible(x)
    got = loader.decompress_array(s)
    assert tuple(got.shape) == shape
    assert torch.equal(got, want)
    np.testing.assert_array_equal(O.gzip_decode(s), want.numpy())  # the reference's decoder restated


def test_batch_compress_matches_single():
    x = _cells(7, (5, 1, 32, 32))
    batch = loader.compress_batch(x, workers=3)
    # gzip headers carry the compression time (as leniax's strings do): compare the payloads
    payload = lambda z: gzip.decompress(base64.decodebytes(z.encode('utf-8')))  # noqa: E731
    assert [payload(z) for z in batch] == [payload(loader.compress_array(x[i])) for i in range(5)]


def test_two_character_codec():
    for v in (0, 1, 111, 112, 5000, loader.MAX_VAL):
        assert loader.ch2val(loader.val2ch(v)) == v
    vals = [0, 17, 12543, 4000, 9, 112]
    code = ''.join(loader.val2ch(v) for v in vals) + '::2;3'
    got = loader.decompress_array(code)
    assert torch.allclose(got, torch.tensor(vals, dtype=torch.float32).reshape(2, 3) / loader.MAX_VAL)
    with pytest.raises(ValueError):
        loader.decompress_array('not a cell code')


@pytest.mark.parametrize('case', ['orbium', 'orbium_scutium'])
def test_run_length_codec_decodes_the_reference_fixtures(case):
    # the fixture's own run-length string against the cells it encodes (the
    # decoded state the golden last frames are reproduced from)
    import json
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
    code = json.load(open(os.path.join(here, f'{case}.json')))['cells_code']
    init = np.load(os.path.join(here, f'{case}_init.npy'))
    got = loader.deprecated_decompress_array(code, 3)
    np.testing.assert_array_equal(got, init)
    np.testing.assert_array_equal(O.rle_decode(code, 3), init)
    assert torch.equal(loader.decompress_array(code, 3), torch.from_numpy(init))  # the fallback chain ends there
    # the encoder's string decodes to the same cells
    np.testing.assert_array_equal(loader.deprecated_decompress_array(loader.deprecated_compress_array(init), 3), init)


def test_run_length_codec_symbols_counts_and_blocks():
    assert [loader.rle_value(s) for s in ('.', 'b', 'o', 'A', 'X', 'pA', 'pX', 'qA', 'yO')] == \
        [0, 0, 255, 1, 24, 25, 48, 49, 255]
    assert all(loader.rle_value(loader.rle_symbol(v)) == v for v in range(256))
    x = np.array([[1.0, 1.0], [1.0, 0.0]], np.float32)
    assert loader.deprecated_compress_array(x) == '2yO$yO.!'  # 255 is written 'yO' ('o' is read only)
    # a count before a delimiter adds empty rows; short rows are padded with zeros
    got = loader.deprecated_decompress_array('2o$3.A2$o!', 2)
    want = np.zeros((4, 4), np.float32)
    want[0, :2] = 1
    want[1, 3] = 1 / 255
    want[3, 0] = 1
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(O.rle_decode('2o$3.A2$o!', 2), want)
    # 3D: '%' closes a plane
    cube = np.zeros((2, 2, 3), np.float32)
    cube[0, 0, 0], cube[1, 1, 2] = 1, 100 / 255
    code = loader.deprecated_compress_array(cube)
    np.testing.assert_array_equal(loader.deprecated_decompress_array(code, 3), cube)


def test_npz_fallback_and_load_raw_cells(tmp_path):
    import io
    import pickle
    q = (np.arange(12, dtype=np.uint8) * 20).reshape(3, 4)
    buf = io.BytesIO()
    np.savez(buf, x=q)
    s = buf.getvalue().decode('latin1')
    np.testing.assert_allclose(loader.decompress_array(s).numpy(), q / 255., rtol=1e-6)
    cfg = {'world_params': {'nb_dims': 2, 'nb_channels': 1}, 'run_params': {'init_cells': '2o$o.!'}}
    np.testing.assert_array_equal(loader.load_raw_cells(cfg).numpy(), [[[1, 1], [1, 0]]])  # channel axis put back
    cfg['run_params'] = {'cells': [[0.5, 0.25]], 'init_cells': 'MISSING'}
    assert loader.load_raw_cells(cfg).numel() == 0
    np.testing.assert_array_equal(loader.load_raw_cells(cfg, use_init_cells=False).numpy(), [[[0.5, 0.25]]])
    # last_frame.p beside the configuration: numpy arrays only
    frame = np.linspace(0, 1, 8, dtype=np.float32).reshape(1, 2, 4)
    (tmp_path / 'last_frame.p').write_bytes(pickle.dumps(frame))
    cfg = {'world_params': {'nb_dims': 2, 'nb_channels': 1}, 'run_params': {'init_cells': 'last_frame.p'},
           'main_path': str(tmp_path)}
    np.testing.assert_array_equal(loader.load_raw_cells(cfg).numpy(), frame)
    (tmp_path / 'last_frame.p').write_bytes(pickle.dumps(print))  # a callable is refused
    with pytest.raises(pickle.UnpicklingError):
        loader.load_raw_cells(cfg)


def test_init_places_string_encoded_cells():
    from leniax_gb300 import helpers
    cfg = {'world_params': {'nb_dims': 2, 'nb_channels': 1, 'R': 5, 'T': 10},
           'render_params': {'world_size': [16, 16]},
           'run_params': {'init_cells': '2o$o.!'},
           'kernels_params': [{'k_slug': 'circle_2d', 'k_params': [1.0, [1.0]], 'kf_slug': 'gauss_bump',
                               'kf_params': [4.0], 'gf_slug': 'gaussian', 'gf_params': [0.15, 0.015], 'h': 1.0,
                               'c_in': 0, 'c_out': 0}]}
    cells, K, _ = helpers.init(cfg, device=torch.device('cpu'))
    want = helpers.create_init_cells([16, 16], 1, [np.array([[[1, 1], [1, 0]]], np.float32)])
    np.testing.assert_array_equal(cells.numpy(), want)


def test_reference_loader_tests():
    # tests/test_loader.py:15-70, with numpy inputs as there
    from leniax_gb300.constant import NB_CHARS
    vals = list(range(256))
    assert [loader.ch2val(loader.val2ch(v)) for v in vals] == vals
    assert [loader.char2val_deprecated(loader.val2char_deprecated(v)) for v in vals] == vals
    cells = np.arange(0, 1e5, 100) / 1e5
    out = loader.decompress_array(loader.compress_array(cells), 1)
    np.testing.assert_array_almost_equal(cells, out.numpy(), decimal=4)
    out = loader.decompress_array(loader.compress_array(out), 1)
    np.testing.assert_array_almost_equal(cells, out.numpy(), decimal=4)
    comp = loader.make_array_compressible(cells)
    np.testing.assert_array_almost_equal(comp.numpy(), loader.decompress_array(loader.compress_array(comp), 1).numpy(),
                                         decimal=9)
    grid = (np.arange(0, NB_CHARS**2, 8, dtype=np.int32) / (NB_CHARS**2 - 1)).reshape(32, 49)
    np.testing.assert_array_almost_equal(grid, loader.decompress_array(loader.compress_array(grid)).numpy(),
                                         decimal=4)
