"""Generate the golden fixtures under tests/golden/ from leniax's own test fixtures.

Run where the leniax sources are available, passing the root of the leniax
project (or setting ``LENIAX_SRC``)::

    python tests/golden/make_golden.py --ref <leniax project root>

It reads ``tests/fixtures/{orbium-test,orbium-scutium-test,aquarium-test}.yaml``
(a small YAML subset parser: PyYAML is not installed) and the matching golden
last frames ``*_last_frame*.p`` (numpy pickles, loaded with an unpickler that
admits numpy's array-reconstruction classes only).  For each case it writes:

* ``<case>.json``      -- world/run params, v2 kernel params
                          (v1 -> v2 migration as in leniax ``utils.py:91-124``)
                          the fixture's own v1 kernel entries (``kernels_params_v1``)
                          and its encoded initial cells (``cells_code``, when the
                          fixture gives them as a string)
* ``<case>_init.npy``  -- decoded initial cells ``[C, h, w]`` (float32)
* ``<case>_last.npy``  -- leniax's golden state after ``max_run_iter - 1`` steps

The test suite only reads these outputs; it never touches the reference tree.
"""
import argparse
import json
import os
import pickle
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import lenia_oracle as O  # noqa: E402

CASES = {
    'orbium': ('orbium-test.yaml', 'orbium-test_last_frame.p', 4),
    'orbium_scutium': ('orbium-scutium-test.yaml', 'orbium-scutium-test_last_frame2.p', 4),
    'aquarium': ('aquarium-test.yaml', 'aquarium-test_last_frame.p', 3),
}


def _scalar(v: str):
    v = v.strip()
    if v == '':
        return None
    if v[0] in '[{':
        return json.loads(v)
    if (v[0] == v[-1]) and v[0] in '"\'':
        return v[1:-1]
    for cast in (int, float):
        try:
            return cast(v)
        except ValueError:
            pass
    if v in ('true', 'false'):
        return v == 'true'
    return v


def parse_yaml_subset(text: str):
    """Indentation-based parser for the mappings / block lists / flow lists /
    scalars used by leniax's test fixtures."""
    lines = []
    for raw in text.splitlines():
        if not raw.strip() or raw.strip().startswith('#'):
            continue
        lines.append((len(raw) - len(raw.lstrip(' ')), raw.strip()))

    def parse_block(i, indent):
        if i < len(lines) and lines[i][1].startswith('- '):
            out = []
            while i < len(lines) and lines[i][0] == indent and lines[i][1].startswith('- '):
                item_indent = indent + 2
                first = lines[i][1][2:]
                sub = [(item_indent, first)]
                j = i + 1
                while j < len(lines) and lines[j][0] >= item_indent:
                    sub.append(lines[j])
                    j += 1
                if ':' in first and not first.startswith(('[', '"', "'")):
                    saved = lines[:]
                    lines[i:j] = sub
                    val, _ = parse_block(i, item_indent)
                    lines[:] = saved
                    out.append(val)
                else:
                    out.append(_scalar(first))
                i = j
            return out, i
        out = {}
        while i < len(lines) and lines[i][0] == indent:
            key, _, rest = lines[i][1].partition(':')
            rest = rest.strip()
            if rest == '':
                if i + 1 < len(lines) and lines[i + 1][0] > indent:
                    val, i = parse_block(i + 1, lines[i + 1][0])
                elif i + 1 < len(lines) and lines[i + 1][0] == indent and lines[i + 1][1].startswith('- '):
                    val, i = parse_block(i + 1, indent)
                else:
                    val, i = None, i + 1
            else:
                val, i = _scalar(rest), i + 1
            out[key.strip()] = val
        return out, i

    val, _ = parse_block(0, lines[0][0])
    return val


class _NumpyOnlyUnpickler(pickle.Unpickler):
    ALLOWED = {
        ('numpy.core.multiarray', '_reconstruct'),
        ('numpy._core.multiarray', '_reconstruct'),
        ('numpy', 'ndarray'),
        ('numpy', 'dtype'),
    }

    def find_class(self, module, name):
        if (module, name) in self.ALLOWED:
            if module.startswith('numpy.core'):
                module = module.replace('numpy.core', 'numpy._core')
            return super().find_class(module, name)
        raise pickle.UnpicklingError(f'blocked {module}.{name}')


def load_frame(path):
    with open(path, 'rb') as f:
        return np.asarray(_NumpyOnlyUnpickler(f).load(), dtype=np.float32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', default=os.environ.get('LENIAX_SRC'),
                    help='root of the leniax project (default: $LENIAX_SRC)')
    args = ap.parse_args()
    if not args.ref:
        ap.error('pass --ref <leniax project root> or set LENIAX_SRC')
    fx = os.path.join(args.ref, 'tests', 'fixtures')
    for case, (yml, frame, decimal) in CASES.items():
        cfg = parse_yaml_subset(open(os.path.join(fx, yml)).read())
        wp = cfg['world_params']
        rp = cfg['render_params']
        nb_dims = int(wp['nb_dims'])
        world_size = [2**int(rp['size_power2'])] * nb_dims
        kernels = O.kernels_v1_to_v2(cfg['kernels_params']['k'])
        cells = cfg['run_params'].get('init_cells', cfg['run_params']['cells'])
        raw = O.decode_cells(cells, nb_dims + 1)
        if raw.ndim == nb_dims and int(wp['nb_channels']) == 1:
            raw = raw[np.newaxis]
        out = {
            'name': case,
            'world_size': world_size,
            'nb_channels': int(wp['nb_channels']),
            'R': wp['R'],
            'T': wp['T'],
            'get_state_fn_slug': wp.get('get_state_fn_slug', 'v1'),
            'weighted_average': wp.get('weighted_average', True),
            'max_run_iter': int(cfg['run_params']['max_run_iter']),
            'decimal': decimal,
            'kernels_params': kernels,
            'kernels_params_v1': cfg['kernels_params']['k'],
        }
        if isinstance(cells, str):
            out['cells_code'] = cells
        with open(os.path.join(HERE, f'{case}.json'), 'w') as f:
            json.dump(out, f, indent=1)
        np.save(os.path.join(HERE, f'{case}_init.npy'), raw.astype(np.float32))
        last = load_frame(os.path.join(fx, frame))
        if last.ndim == 4:
            last = last[0]
        np.save(os.path.join(HERE, f'{case}_last.npy'), last)
        print(case, raw.shape, last.shape, out['max_run_iter'])


if __name__ == '__main__':
    main()
