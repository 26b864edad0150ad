"""GB300-native Lenia engine: a drop-in for leniax's hot path
(``core.update``, ``runner.run_scan``, ``runner.run_scan_mem_optimized``)
running hand-written sm_103a CUDA kernels behind a C ABI
(``include/lenia_gb300.h``)."""
from . import constant, growth_functions, kernels, core, statistics, runner, helpers  # noqa: F401
from ._lib import LgxError, load  # noqa: F401

__all__ = ['constant', 'growth_functions', 'kernels', 'core', 'statistics', 'runner', 'helpers', 'LgxError', 'load']
