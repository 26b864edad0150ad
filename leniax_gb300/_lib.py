"""ctypes binding of the engine's C ABI (``include/lenia_gb300.h``).

The shared library is built in-tree (``leniax_gb300/_lgx.so``) by
``leniax_gb300.build``.  There is no fallback: if the library is missing or a
call fails, an exception is raised.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, '_lgx.so')

# status codes, growth / state ids, engines (mirror the header)
LGX_OK = 0
LGX_ERR_INVALID = 1
LGX_ERR_UNSUPPORTED = 2
LGX_ERR_CUDA = 3
LGX_ERR_WORKSPACE = 4
LGX_ERR_TIMEOUT = 5

GF_IDS = {
    'poly_quad4': 0,
    'gaussian': 1,
    'gaussian_target': 2,
    'step': 3,
    'staircase': 4,
    'triangle': 5,
    'identity': 6,
}
STATE_IDS = {'v1': 0, 'v2': 1, 'simple': 2}
ENGINES = {'auto': 0, 'resident': 1, 'streamed': 2, 'plain': 3, 'cta': 4, 'plain_streamed': 5, 'nd': 6}
NSTAT_SCALAR = 11

EXPORTED = (
    'lgx_version', 'lgx_last_error', 'lgx_plan_create', 'lgx_plan_destroy', 'lgx_select_engine',
    'lgx_run_workspace_bytes', 'lgx_run', 'lgx_update_workspace_bytes', 'lgx_update', 'lgx_fp32_probe',
    'lgx_batch_workspace_bytes', 'lgx_batch_run', 'lgx_workspace_status', 'lgx_ring_kernels_workspace_bytes',
    'lgx_ring_kernels', 'lgx_selftest_wait_timeout', 'lgx_adjoint_kernel_grad_acc_bytes', 'lgx_kernel_spectrum_nd',
    'lgx_kernel_spectrum_nd_workspace_bytes', 'lgx_plan_set_adjoint_engine', 'lgx_growth', 'lgx_weighted',
    'lgx_field', 'lgx_state'
)


class LgxError(RuntimeError):
    """Error returned by the engine's C ABI."""

    def __init__(self, code, msg):
        super().__init__(f'lgx error {code}: {msg}')
        self.code = code


class ModelDesc(ctypes.Structure):
    _fields_ = [
        ('nb_dims', ctypes.c_int),
        ('world', ctypes.c_int * 3),
        ('nb_channels', ctypes.c_int),
        ('nb_kernels', ctypes.c_int),
        ('max_k', ctypes.c_int),
        ('kernel_cin', ctypes.POINTER(ctypes.c_int)),
        ('kernel_slot', ctypes.POINTER(ctypes.c_int)),
        ('growth_fn', ctypes.POINTER(ctypes.c_int)),
        ('state_fn', ctypes.c_int),
        ('weighted_average', ctypes.c_int),
    ]


_fp = ctypes.c_void_p


class Rollout(ctypes.Structure):
    _fields_ = [
        ('n_sols', ctypes.c_int),
        ('n_init', ctypes.c_int),
        ('steps', ctypes.c_int),
        ('cells0', _fp),
        ('k_half', _fp),
        ('gf_params', _fp),
        ('weights', _fp),
        ('T', _fp),
        ('stats_R', ctypes.c_float),
        ('stats_T', ctypes.c_float),
        ('final_cells', _fp),
        ('stats', _fp),
        ('n_continue', _fp),
        ('n_box', _fp),
        ('traj_cells', _fp),
        ('traj_field', _fp),
        ('traj_potential', _fp),
        ('engine', ctypes.c_int),
        ('centroid', _fp),
        ('main_events', _fp * 2),
        ('stats_R_sol', _fp),
        ('stats_T_sol', _fp),
    ]


_lock = threading.Lock()
_lib = None


def load():
    """Load the engine library (once).  Raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f'leniax_gb300 engine library not built: {LIB_PATH} missing '
                               '(run `python -m leniax_gb300.build`)')
        lib = ctypes.CDLL(LIB_PATH)
        lib.lgx_version.restype = ctypes.c_int
        lib.lgx_last_error.restype = ctypes.c_char_p
        lib.lgx_plan_create.argtypes = [ctypes.POINTER(ModelDesc), ctypes.POINTER(ctypes.c_void_p)]
        lib.lgx_plan_create.restype = ctypes.c_int
        lib.lgx_plan_destroy.argtypes = [ctypes.c_void_p]
        lib.lgx_plan_destroy.restype = None
        lib.lgx_select_engine.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.lgx_select_engine.restype = ctypes.c_int
        lib.lgx_run_workspace_bytes.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.lgx_run_workspace_bytes.restype = ctypes.c_size_t
        lib.lgx_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(Rollout), ctypes.c_void_p, ctypes.c_size_t,
                                ctypes.c_void_p]
        lib.lgx_run.restype = ctypes.c_int
        lib.lgx_update_workspace_bytes.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.lgx_update_workspace_bytes.restype = ctypes.c_size_t
        lib.lgx_update.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 5 + [ctypes.c_int] + \
            [ctypes.c_void_p] * 3 + [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
        lib.lgx_update.restype = ctypes.c_int
        lib.lgx_workspace_status.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        lib.lgx_workspace_status.restype = ctypes.c_int
        lib.lgx_fp32_probe.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        lib.lgx_fp32_probe.restype = ctypes.c_longlong
        lib.lgx_selftest_wait_timeout.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        lib.lgx_selftest_wait_timeout.restype = ctypes.c_int
        vp, ci, cl = ctypes.c_void_p, ctypes.c_int, ctypes.c_long
        lib.lgx_growth.argtypes = [ci, ci, cl, ctypes.POINTER(ci), vp, vp, vp, vp]
        lib.lgx_weighted.argtypes = [ci, ci, ci, cl, vp, vp, ci, vp, vp]
        lib.lgx_field.argtypes = [ci, ci, ci, cl, ctypes.POINTER(ci), vp, vp, vp, ci, vp, vp]
        lib.lgx_state.argtypes = [ci, ci, cl, ci, vp, vp, vp, ci, vp, vp]
        for f in (lib.lgx_growth, lib.lgx_weighted, lib.lgx_field, lib.lgx_state):
            f.restype = ci
        if lib.lgx_version() != 2:
            raise RuntimeError('leniax_gb300 engine ABI version mismatch')
        _lib = lib
        return lib


def workspace_status(ws_ptr: int, stream_handle: int) -> int:
    """Device status word of the last call that used this workspace (0 = ok);
    synchronises the stream."""
    out = ctypes.c_int(0)
    check(load().lgx_workspace_status(ws_ptr, stream_handle, ctypes.byref(out)))
    return out.value


def check(code):
    if code != LGX_OK:
        msg = load().lgx_last_error().decode('utf-8', 'replace')
        raise LgxError(code, msg)


class Plan:
    """Owns an ``lgx_plan`` built from a model description."""

    def __init__(self, nb_dims, world, nb_channels, kernel_cin, kernel_slot, growth_ids, max_k, state_fn,
                 weighted_average):
        lib = load()
        K = len(kernel_cin)
        self._cin = (ctypes.c_int * K)(*kernel_cin)
        self._slot = (ctypes.c_int * K)(*kernel_slot)
        self._gf = (ctypes.c_int * K)(*growth_ids)
        d = ModelDesc()
        d.nb_dims = nb_dims
        for i, w in enumerate(world):
            d.world[i] = int(w)
        d.nb_channels = nb_channels
        d.nb_kernels = K
        d.max_k = max_k
        d.kernel_cin = self._cin
        d.kernel_slot = self._slot
        d.growth_fn = self._gf
        d.state_fn = state_fn
        d.weighted_average = 1 if weighted_average else 0
        self.desc = d
        h = ctypes.c_void_p()
        check(lib.lgx_plan_create(ctypes.byref(d), ctypes.byref(h)))
        self.handle = h
        self.nb_dims, self.world, self.C, self.K, self.max_k = nb_dims, tuple(world), nb_channels, K, max_k

    def __del__(self):
        h = getattr(self, 'handle', None)
        if h is not None and h.value and _lib is not None:
            _lib.lgx_plan_destroy(h)
            self.handle = None
