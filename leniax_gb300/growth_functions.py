"""Growth-function plugin registry (leniax ``growth_functions.py:256-264``).

The engine evaluates growth functions on the device; this registry maps the
reference's slugs to the engine's function ids (``LGX_GF_*`` in
``include/lenia_gb300.h``).  The formulas, in the reference's op order, are in
``csrc/common.cuh`` (``growth_fn``).
"""
from ._lib import GF_IDS

register = dict(GF_IDS)
