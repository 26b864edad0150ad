"""Autotuner of the uneven-batch launch.

For a set of world classes it chooses, by timing short rollouts on the
device it will run on:

* the queue order: every class alone is timed to measure the cost of one of
  its work items, and the classes are queued by measured item cost, largest
  first (longest-processing-time-first scheduling of the persistent CTAs);
  the built-in estimate (``'largest_first'``) stays a candidate;
* the 3D line-transform width (2 or 4 lanes per y/z line, i.e. a radix-32 or
  radix-16 in-register pass for 64^3) when a 3D class is present;
* the persistent grid: one CTA per SM, or fewer when the queue is shorter.

Only the classes of the persistent launch are tuned; classes of other shapes
run through one ``lgx_run`` each whatever the settings.

Results are cached per device and class signature in a JSON file
(``$LGX_AUTOTUNE_CACHE`` or ``~/.cache/leniax_gb300/autotune.json``).
"""
import json
import math
import os
import threading
from typing import Dict, List

import torch

from .batch import UnevenBatch, WorldClass, persistent_shape

_lock = threading.Lock()


def cache_path() -> str:
    p = os.environ.get('LGX_AUTOTUNE_CACHE')
    if p:
        return p
    return os.path.join(os.path.expanduser('~'), '.cache', 'leniax_gb300', 'autotune.json')


def signature(classes: List[WorldClass]) -> str:
    dev = classes[0].cells0.device
    name = torch.cuda.get_device_name(dev)
    parts = [f'{len(c.world)}d{"x".join(map(str, c.world))}:n{c.n}:{c.gf_slug}:{c.state_slug}' for c in classes]
    return name + '|' + ','.join(parts)


def _load() -> Dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key: str, value: Dict):
    path = cache_path()
    with _lock:
        data = _load()
        data[key] = value
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            tmp = path + f'.{os.getpid()}.tmp'
            with open(tmp, 'w') as f:
                json.dump(data, f, indent=1, sort_keys=True)
            os.replace(tmp, path)
        except OSError:
            pass  # a read-only home only costs a re-tune


def _time(batch: UnevenBatch, reps: int) -> float:
    """Median device time (ms) of ``reps`` launches after one warm-up."""
    batch.launch()
    ts = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        batch.launch()
        b.record()
        b.synchronize()
        ts.append(a.elapsed_time(b))
    ts.sort()
    return ts[len(ts) // 2]


def _items(c: WorldClass) -> int:
    nd, size = len(c.world), c.world[0]
    per = {(2, 32): 8, (2, 64): 4, (2, 128): 1}.get((nd, size), 1)
    return (c.n + per - 1) // per


def tune(classes: List[WorldClass], steps: int, probe_steps: int = 8, reps: int = 3) -> Dict:
    """Time the candidates on ``probe_steps``-step rollouts of the persistent
    classes; return the best settings (keyword arguments of
    :class:`UnevenBatch`, class indices into ``classes``) and the timings."""
    probe_steps = max(1, min(int(steps), int(probe_steps)))
    pers = [i for i, c in enumerate(classes) if persistent_shape(c.world)]
    if not pers:
        return {'settings': dict(order='largest_first', line_group=4, grid=0), 'item_ms': [None] * len(classes),
                'probe_steps': probe_steps, 'candidates': []}
    sub = [classes[i] for i in pers]
    sms = torch.cuda.get_device_properties(sub[0].cells0.device).multi_processor_count
    has3d = any(len(c.world) == 3 for c in sub)
    lgs = [4, 2] if has3d else [4]
    # measured cost of one item of each class, with the best line width per class
    item_ms = [None] * len(classes)
    for i in pers:
        c, best = classes[i], math.inf
        for lg in (lgs if len(c.world) == 3 else [4]):
            b = UnevenBatch([c], probe_steps, line_group=lg, with_stats=False)
            t = _time(b, reps)
            waves = math.ceil(_items(c) / min(sms, _items(c)))
            best = min(best, t / waves)
        item_ms[i] = best
    measured = sorted(range(len(sub)), key=lambda j: -item_ms[pers[j]])
    cands = []
    for lg in lgs:
        cands.append(dict(order='explicit', class_order=measured, line_group=lg, grid=0))
        cands.append(dict(order='largest_first', line_group=lg, grid=0))
    timings = []
    for kw in cands:
        b = UnevenBatch(sub, probe_steps, with_stats=False, **kw)
        timings.append((_time(b, reps), kw))
    timings.sort(key=lambda x: x[0])
    best = dict(timings[0][1])
    if 'class_order' in best:  # indices into the persistent classes -> into ``classes``
        best['class_order'] = [pers[j] for j in best['class_order']]
    return {'settings': best, 'item_ms': item_ms, 'probe_steps': probe_steps,
            'candidates': [{'ms': t, **kw} for t, kw in timings]}


def tuned_settings(classes: List[WorldClass], steps: int, refresh: bool = False) -> Dict:
    """Cached :func:`tune` result for these classes on this device."""
    key = signature(classes)
    if not refresh:
        hit = _load().get(key)
        if hit and 'settings' in hit:
            return dict(hit['settings'])
    res = tune(classes, steps)
    _store(key, res)
    return dict(res['settings'])
