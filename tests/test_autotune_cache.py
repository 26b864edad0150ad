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


def _cls(world, n=2):
    import torch
    from leniax_gb300.batch import WorldClass
    z = torch.zeros(n)
    return WorldClass(torch.zeros((n, ) + tuple(world)), None, torch.zeros(n, 2), z, z, z)


def test_signature_names_every_side(monkeypatch):
    # worlds of 26 x 100 and 26 x 50 are different classes, and so are their tunings
    monkeypatch.setattr(autotune.torch.cuda, 'get_device_name', lambda dev=None: 'dev')
    a = autotune.signature([_cls((64, 64)), _cls((26, 100))])
    b = autotune.signature([_cls((64, 64)), _cls((26, 50))])
    assert a != b and a == 'dev|2d64x64:n2:gaussian:v1,2d26x100:n2:gaussian:v1'


def test_persistent_shapes_and_untuned_classes():
    from leniax_gb300.batch import persistent_shape
    assert all(persistent_shape(w) for w in ((32, 32), (64, 64), (128, 128), (256, 256), (32, 32, 32), (64, 64, 64)))
    assert not any(persistent_shape(w) for w in ((100, 100), (64, 128), (48, 48, 48), (64, 64, 32), (512, 512)))
    # classes the persistent launch does not take need no timing: the defaults come back
    res = autotune.tune([_cls((100, 100)), _cls((24, 24, 24))], 16)
    assert res['settings'] == {'order': 'largest_first', 'line_group': 4, 'grid': 0}
    assert res['item_ms'] == [None, None] and res['candidates'] == []
