"""leniax's pipeline goldens through the eager and scanned drivers
(``tests/test_pipeline.py:18-130`` of leniax): ``helpers.init_and_run`` with
``with_jit=False`` (the eager ``runner.run``, runner.py:16-116) and
``with_jit=True`` (``runner.run_scan``, runner.py:119-164) on the orbium,
orbium-scutium and aquarium fixtures; ``len(all_cells) == max_run_iter`` and
the last frame equal to leniax's golden frame at the reference's decimals."""
import numpy as np
import pytest
import torch

from leniax_gb300 import helpers
from tests.cases import golden_case

pytestmark = pytest.mark.gpu


def _config(cfg, init):
    """A leniax v2 config dict of a golden case (what get_container returns
    for the fixture YAML: world, render and run parameters, kernels)."""
    return {
        'world_params': {
            'nb_dims': len(cfg['world_size']), 'nb_channels': cfg['nb_channels'], 'R': cfg['R'], 'T': cfg['T'],
            'get_state_fn_slug': cfg['get_state_fn_slug'], 'weighted_average': cfg['weighted_average']
        },
        'render_params': {'world_size': list(cfg['world_size'])},
        'run_params': {'init_cells': init, 'max_run_iter': cfg['max_run_iter']},
        'kernels_params': [dict(k) for k in cfg['kernels_params']],
    }


@pytest.mark.parametrize('with_jit', [False, True])
@pytest.mark.parametrize('name', ['orbium', 'orbium_scutium', 'aquarium'])
def test_init_and_run_reproduces_golden(cuda, name, with_jit):
    cfg, init, last = golden_case(name)
    all_cells, all_fields, all_pots, stats = helpers.init_and_run(None, _config(cfg, init), with_jit=with_jit,
                                                                  device=cuda)
    all_cells = all_cells[:, 0]
    assert len(all_cells) == cfg['max_run_iter']
    assert all_fields.shape[0] == all_pots.shape[0] == cfg['max_run_iter']
    np.testing.assert_array_almost_equal(last, all_cells[-1].cpu().numpy(), decimal=cfg['decimal'])


def test_eager_run_truncates_at_its_stop_step(cuda):
    # runner.py:84-104: the eager loop breaks once should_continue drops after
    # START_CHECK_STOP; the returned trajectory and N stop there
    from leniax_gb300 import kernels, runner, statistics
    from oracle import lenia_oracle as O
    from tests.cases import bump_kernel_params, patch_init
    dev = cuda
    cells = patch_init(1, 64, 24, seed=2)
    kp = bump_kernel_params(m=0.3, s=0.02)  # a world that dies within a few dozen steps
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], [64, 64], 1, 10, True, dev)
    upd = helpers.build_update_fn(K.shape, mp)
    cs, fs, ps, st = runner.run(None, torch.from_numpy(cells).to(dev), K, mp.get_gf_params(dev),
                                mp.get_kernels_weight_per_channel(dev), torch.tensor(10.), 200, 10, upd,
                                statistics.ComputeStatsFn([64, 64], 10, 10), stat_trunc=True)
    Ko, mpo = O.get_kernels_and_mapping([dict(p) for p in kp], [64, 64], 1, 10, True, np.float32)
    cs_o, fs_o, ps_o, st_o = O.run_eager(cells, Ko, mpo['gf_params'], mpo['weights'], 10, 200, 10, O.Model(mpo),
                                         stat_trunc=True)
    assert int(st['N']) == int(st_o['N']) < 199
    assert cs.shape[0] == cs_o.shape[0]
    assert np.abs(cs.cpu().numpy() - cs_o).max() < 1e-4
