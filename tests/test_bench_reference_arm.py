"""The reference arm of bench.py (host only): ``--warmup`` untimed and
``--steps`` timed bounded samples of the workload through the oracle, one
JSON object with the bench line's keys."""
import argparse

import bench


def test_reference_arm_line_keys_and_units():
    args = argparse.Namespace(gpus=1, steps=2, warmup=1)
    line = bench.run_reference(args, budget_s=1.0)  # the smallest sample: 16 Euler steps
    assert line['impl'] == 'reference' and line['metric'] == line['unit'] == bench.METRIC
    assert line['steps'] == 2 and line['warmup'] == 1 and line['higher_is_better'] is True
    assert line['value'] > 0 and line['ms_per_step'] > 0
    assert line['config']['workload'] == bench.WORKLOAD
    assert line['config']['step'] == f'{bench.CPU_SAMPLE_WORLDS} worlds x 16 Euler steps of the workload'
    # value = cell-updates of the timed samples / their time
    cells = bench.CPU_SAMPLE_WORLDS * bench.P_CELLS * 16
    assert abs(line['value'] * line['ms_per_step'] / 1e3 - cells) <= 1e-6 * cells
    cb = line['cpu_baseline']
    assert cb['kind'] == 'port' and cb['value'] == line['value'] and cb['cores'] >= 1
    assert line['e2e'] == {'value': line['value'], 'unit': bench.METRIC, 'h2d_bytes_per_step': 0,
                           'd2h_bytes_per_step': 0}
