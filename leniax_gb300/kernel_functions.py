"""Kernel functions and their plugin registry (leniax
``kernel_functions.py``): ``fn(params, X)`` on distances ``X`` in [0, 1)
(numpy, float32), used by the host kernel builders of
:mod:`leniax_gb300.kernels` (kernels.py:206, 252, 302).  ``register`` is the
dict those builders look slugs up in (kernel_functions.py:253-261), so an
entry a user adds here is used by ``kernels.get_kernels_and_mapping``.  The
device builder ``kernels.ring_kernels`` runs the seven built-in functions
only (``kernels.KF_IDS``)."""
from .kernels import gauss, gauss_bump, kf_register, poly_quad, staircase, step, threshold, triangle

register = kf_register

__all__ = ['register', 'poly_quad', 'gauss_bump', 'gauss', 'step', 'threshold', 'staircase', 'triangle']
