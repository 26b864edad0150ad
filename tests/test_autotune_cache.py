"""Autotuner cache (host logic, no GPU): results are stored per signature in
the JSON file named by LGX_AUTOTUNE_CACHE and a cached entry is returned
without re-tuning."""
import json

from leniax_gb300 import autotune


def test_store_and_load_round_trip(tmp_path, monkeypatch):
    path = tmp_path / 'sub' / 'tune.json'
    monkeypatch.setenv('LGX_AUTOTUNE_CACHE', str(path))
    assert autotune.cache_path() == str(path)
    assert autotune._load() == {}  # no file yet
    autotune._store('dev|2d64x8:gaussian:v1', {'settings': {'order': 'largest_first', 'line_group': 4}})
    autotune._store('dev|3d64x2:gaussian:v1', {'settings': {'order': 'explicit', 'class_order': [0],
                                                            'line_group': 2}})
    data = json.loads(path.read_text())
    assert set(data) == {'dev|2d64x8:gaussian:v1', 'dev|3d64x2:gaussian:v1'}
    assert autotune._load()['dev|3d64x2:gaussian:v1']['settings']['line_group'] == 2


def test_cached_settings_skip_tuning(tmp_path, monkeypatch):
    monkeypatch.setenv('LGX_AUTOTUNE_CACHE', str(tmp_path / 'tune.json'))
    monkeypatch.setattr(autotune, 'signature', lambda classes: 'dev|sig')
    autotune._store('dev|sig', {'settings': {'order': 'largest_first', 'line_group': 4, 'grid': 0}})

    def no_tuning(*a, **k):
        raise AssertionError('a cached signature must not be re-tuned')

    monkeypatch.setattr(autotune, 'tune', no_tuning)
    assert autotune.tuned_settings([], 16) == {'order': 'largest_first', 'line_group': 4, 'grid': 0}


def test_corrupt_cache_reads_as_empty(tmp_path, monkeypatch):
    path = tmp_path / 'tune.json'
    path.write_text('{not json')
    monkeypatch.setenv('LGX_AUTOTUNE_CACHE', str(path))
    assert autotune._load() == {}
