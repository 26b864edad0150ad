"""Failure detection without a GPU fault: the engines' bounded mbarrier wait
is driven to its limit by a self-test kernel (an arrival that nothing makes),
the timeout status comes back to the host, and the context keeps working."""
import numpy as np
import pytest
import torch

from leniax_gb300 import _lib, helpers, kernels, runner, statistics
from tests.cases import bump_kernel_params, patch_init

pytestmark = pytest.mark.gpu


def _short_rollout(cuda):
    kp = bump_kernel_params()
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], [64, 64], 1, 10, True, cuda)
    upd = helpers.build_update_fn(K.shape, mp)
    stats_fn = statistics.ComputeStatsFn([64, 64], 10, 10.)
    cells = torch.from_numpy(patch_init(2, 64, 24, seed=3)[None]).to(cuda)
    _, fin = runner.run_scan_mem_optimized(None, cells, K[None], mp.get_gf_params(cuda)[None],
                                           mp.get_kernels_weight_per_channel(cuda)[None], torch.tensor([10.]), 16,
                                           10, upd, stats_fn, check_status=True)
    return fin.cpu().numpy()


def test_bounded_wait_times_out_into_the_status_word(cuda):
    before = _short_rollout(cuda)
    lib = _lib.load()
    st = torch.zeros(1, dtype=torch.int32, device=cuda)
    _lib.check(lib.lgx_selftest_wait_timeout(2000, st.data_ptr(), torch.cuda.current_stream(cuda).cuda_stream))
    torch.cuda.synchronize()
    assert st.item() == 1  # the wait gave up and said so
    # the context is intact: the same rollout gives the same bits
    np.testing.assert_array_equal(_short_rollout(cuda), before)


def test_selftest_rejects_bad_arguments(cuda):
    lib = _lib.load()
    st = torch.zeros(1, dtype=torch.int32, device=cuda)
    assert lib.lgx_selftest_wait_timeout(0, st.data_ptr(), None) == 1  # LGX_ERR_INVALID
    assert lib.lgx_selftest_wait_timeout(10, None, None) == 1
