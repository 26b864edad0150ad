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
