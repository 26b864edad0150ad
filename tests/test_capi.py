"""C ABI: the library loads, exports every symbol include/*.h declares, and
validates plans on the host (no device work; runs without a GPU)."""
import ctypes
import glob
import os
import re

import pytest

from leniax_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, 'include', '*.h')):
        txt = open(h).read()
        syms |= set(re.findall(r'LGX_API\s+[\w\s\*]+?\b(lgx_\w+)\s*\(', txt))
    return syms


def test_header_declares_expected_api():
    syms = declared_symbols()
    assert set(_lib.EXPORTED) <= syms, set(_lib.EXPORTED) - syms


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for s in declared_symbols():
        assert hasattr(lib, s), s
    assert lib.lgx_version() == 2


def _plan(**kw):
    args = dict(nb_dims=2, world=(128, 128), nb_channels=1, kernel_cin=[0], kernel_slot=[0], growth_ids=[1],
                max_k=1, state_fn=0, weighted_average=True)
    args.update(kw)
    return _lib.Plan(**args)


def test_plan_accepts_valid_models():
    p = _plan()
    lib = _lib.load()
    assert lib.lgx_select_engine(p.handle, 1, 4, 0) == 1  # resident for C=1 K=1 128^2
    assert lib.lgx_select_engine(p.handle, 1, 4, 2) == 2
    p2 = _plan(nb_channels=3, kernel_cin=[0, 1, 2], kernel_slot=[0, 0, 0], growth_ids=[1, 1, 0], world=(256, 256))
    assert lib.lgx_select_engine(p2.handle, 1, 4, 0) == 2  # streamed
    assert lib.lgx_run_workspace_bytes(p2.handle, 2, 3, 16, 0) > 0


@pytest.mark.parametrize('side', [48, 72, 100, 112, 480])
def test_sides_that_are_not_powers_of_two_take_the_nd_engine(side):
    # even sides of factors 2, 3, 5, 7: the N-D engine by default, the
    # mixed-radix streamed step on request
    lib = _lib.load()
    p = _plan(world=(side, side))
    assert lib.lgx_select_engine(p.handle, 1, 2, 0) == _lib.ENGINES['nd']
    assert lib.lgx_select_engine(p.handle, 1, 2, _lib.ENGINES['streamed']) == _lib.ENGINES['streamed']
    assert lib.lgx_update_workspace_bytes(p.handle, 3) > 0
    assert lib.lgx_run_workspace_bytes(p.handle, 1, 2, 4, 0) > 0
    assert lib.lgx_run_workspace_bytes(p.handle, 1, 2, 4, _lib.ENGINES['streamed']) > 0


def test_3d_plans_select_the_cta_engine_and_size_workspaces():
    lib = _lib.load()
    p = _plan(nb_dims=3, world=(32, 32, 32))
    assert lib.lgx_select_engine(p.handle, 1, 2, 0) == _lib.ENGINES['cta']
    assert lib.lgx_update_workspace_bytes(p.handle, 3) > 0  # core.update on 3D worlds
    assert lib.lgx_run_workspace_bytes(p.handle, 1, 2, 4, 0) > 0
    # several channels in 3D: the general N-D engine
    p2 = _plan(nb_dims=3, world=(32, 32, 32), nb_channels=2, kernel_cin=[0, 1], kernel_slot=[0, 0], growth_ids=[1, 1])
    assert lib.lgx_select_engine(p2.handle, 1, 2, 0) == _lib.ENGINES['nd']
    assert lib.lgx_update_workspace_bytes(p2.handle, 3) > 0


@pytest.mark.parametrize('nb_dims,world', [(3, (48, 48, 48)), (3, (24, 40, 36)), (2, (100, 128)), (2, (45, 45)),
                                           (2, (35, 64)), (3, (128, 128, 128))])
def test_other_worlds_select_the_nd_engine_and_its_adjoint(nb_dims, world):
    # leniax's get_potential_fft transforms any world shape (core.py:74-87):
    # odd, non-square and 3D sides of factors 2, 3, 5, 7 run on the N-D engine
    lib = _lib.load()
    for attr in ('lgx_adjoint_workspace_bytes', 'lgx_adjoint_kernel_grad_acc_bytes'):
        getattr(lib, attr).restype = ctypes.c_size_t
        getattr(lib, attr).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    p = _plan(nb_dims=nb_dims, world=world, nb_channels=2, kernel_cin=[0, 1, 1], kernel_slot=[0, 0, 1],
              growth_ids=[1, 0, 2], max_k=2)
    assert lib.lgx_select_engine(p.handle, 1, 2, 0) == _lib.ENGINES['nd']
    assert lib.lgx_run_workspace_bytes(p.handle, 1, 2, 4, 0) > 0
    assert lib.lgx_update_workspace_bytes(p.handle, 3) > 0
    assert lib.lgx_adjoint_workspace_bytes(p.handle, 2, 3) > 0
    cells = 1
    for w in world:
        cells *= w
    assert lib.lgx_adjoint_kernel_grad_acc_bytes(p.handle, 2, 3) == 2 * 3 * 3 * cells * 8


@pytest.mark.parametrize('world', [(66, 66), (127, 127), (26, 100), (1031, 64), (2048, 2048), (4096, 16)])
def test_any_side_up_to_2048_and_smooth_sides_up_to_4096_take_the_nd_engine(world):
    # sides with a prime factor above 7 run Bluestein lines (up to 2048);
    # sides of factors 2, 3, 5, 7 up to 4096
    lib = _lib.load()
    p = _plan(world=world)
    assert lib.lgx_select_engine(p.handle, 1, 2, 0) == _lib.ENGINES['nd']
    assert lib.lgx_run_workspace_bytes(p.handle, 1, 2, 4, 0) > 0
    assert lib.lgx_update_workspace_bytes(p.handle, 3) > 0


def _smooth(n):
    for p in (2, 3, 5, 7):
        while n % p == 0:
            n //= p
    return n == 1


def test_side_rule_over_every_side():
    # a plan takes side n iff 2 <= n <= 4096 with prime factors 2, 3, 5, 7
    # (mixed-radix lines) or 2 <= n <= 2048 (Bluestein lines); every
    # accepted side runs on some engine with a sized workspace
    lib = _lib.load()
    for n in range(1, 4101):
        want = 2 <= n and ((n <= 4096 and _smooth(n)) or n <= 2048)
        try:
            p = _plan(world=(n, 16))
        except _lib.LgxError as e:
            assert not want and e.code == _lib.LGX_ERR_UNSUPPORTED, n
            continue
        assert want, n
        assert lib.lgx_select_engine(p.handle, 1, 1, 0) >= 0, n
        assert lib.lgx_run_workspace_bytes(p.handle, 1, 1, 2, 0) > 0, n


@pytest.mark.parametrize('kw,code', [
    (dict(world=(2053, 64)), _lib.LGX_ERR_UNSUPPORTED),  # a prime above 2048 (Bluestein lines up to 2048)
    (dict(world=(64, 4094)), _lib.LGX_ERR_UNSUPPORTED),  # 4094 = 2 * 23 * 89, above 2048
    (dict(world=(8192, 8192)), _lib.LGX_ERR_UNSUPPORTED),  # sides up to 4096
    (dict(nb_dims=3, world=(32, 4099, 32)), _lib.LGX_ERR_UNSUPPORTED),
    (dict(world=(1, 32)), _lib.LGX_ERR_UNSUPPORTED),  # sides from 2
    (dict(nb_dims=4), _lib.LGX_ERR_INVALID),
    (dict(kernel_cin=[1]), _lib.LGX_ERR_INVALID),
    (dict(growth_ids=[42]), _lib.LGX_ERR_UNSUPPORTED),
    (dict(state_fn=7), _lib.LGX_ERR_INVALID),
    (dict(kernel_slot=[3]), _lib.LGX_ERR_INVALID),
    (dict(nb_channels=0), _lib.LGX_ERR_INVALID),
])
def test_plan_rejects_bad_models(kw, code):
    with pytest.raises(_lib.LgxError) as e:
        _plan(**kw)
    assert e.value.code == code
    assert _lib.load().lgx_last_error()


def test_run_rejects_bad_jobs_without_device_work():
    p = _plan()
    lib = _lib.load()
    job = _lib.Rollout()
    job.n_sols, job.n_init, job.steps = 1, 1, 4
    assert lib.lgx_run(p.handle, ctypes.byref(job), None, 0, None) == _lib.LGX_ERR_INVALID  # null tensors
    buf = (ctypes.c_float * 16)()
    addr = ctypes.addressof(buf)
    job.cells0 = job.k_half = job.gf_params = job.weights = job.T = addr
    job.stats_R, job.stats_T = 13., 10.
    assert lib.lgx_run(p.handle, ctypes.byref(job), None, 0, None) == _lib.LGX_ERR_WORKSPACE
    job.n_init = 0
    assert lib.lgx_run(p.handle, ctypes.byref(job), None, 0, None) == _lib.LGX_ERR_INVALID
    job.n_init, job.stats_R = 1, 0.
    assert lib.lgx_run(p.handle, ctypes.byref(job), None, 0, None) == _lib.LGX_ERR_INVALID


def test_update_fn_refuses_cpu_tensors():
    import torch
    from leniax_gb300 import helpers, kernels
    from tests.cases import bump_kernel_params
    K, m = kernels.get_kernels_and_mapping(bump_kernel_params(), [64, 64], 1, 13, device='cpu')
    u = helpers.build_update_fn(K.shape, m)
    with pytest.raises(ValueError, match='CUDA'):
        u(None, torch.zeros(1, 1, 64, 64), K, m.get_gf_params(), m.get_kernels_weight_per_channel(), 0.1)


def test_batch_rejects_bad_jobs_without_device_work():
    from leniax_gb300 import batch as lbatch
    lib = lbatch._bind(_lib.load())
    buf = (ctypes.c_float * 16)()
    addr = ctypes.addressof(buf)
    arr = (lbatch.BatchClassC * 2)()
    for c in arr:
        c.nb_dims, c.size, c.n_worlds, c.gf_id, c.state_fn, c.mean = 2, 64, 3, 1, 0, 1
        c.cells0 = c.k_half = c.gf_params = c.weights = c.T = c.final_cells = addr
    job = lbatch.BatchJobC()
    job.n_classes, job.steps, job.classes = 2, 4, arr
    nbytes = ctypes.c_size_t(0)

    def code():
        return lib.lgx_batch_workspace_bytes(ctypes.byref(job), ctypes.byref(nbytes))

    arr[1].size = 48  # not a supported side
    assert code() == _lib.LGX_ERR_UNSUPPORTED and nbytes.value == 0
    arr[1].nb_dims, arr[1].size = 3, 128  # 3D 128^3 is not supported
    assert code() == _lib.LGX_ERR_UNSUPPORTED
    arr[1].nb_dims, arr[1].size = 3, 32
    arr[1].stats = addr  # statistics without stats_R / stats_T
    assert code() == _lib.LGX_ERR_INVALID
    arr[1].stats = None
    arr[0].cells0 = None
    assert code() == _lib.LGX_ERR_INVALID
    arr[0].cells0 = addr
    job.order = 2  # explicit order without class_order
    assert code() == _lib.LGX_ERR_INVALID
    order = (ctypes.c_int * 2)(1, 1)
    job.class_order = order
    assert code() == _lib.LGX_ERR_INVALID  # not a permutation
    job.order, job.line_group = 0, 3
    assert code() == _lib.LGX_ERR_INVALID
    job.line_group, job.n_classes = 0, 9
    assert code() == _lib.LGX_ERR_INVALID
    job.n_classes = 2
    assert lib.lgx_batch_run(ctypes.byref(job), None, 0, None) == _lib.LGX_ERR_WORKSPACE
