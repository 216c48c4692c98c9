"""suzerain_gb300: GB300-native batched BSMBSM implicit solve.

The compute lives in libsuzerain_gb300.so (hand-written CUDA for sm_103a
behind the C ABI of include/suzerain_gb300.h); this package is its host-side
face: ctypes bindings, the seeded synthetic inputs, the resident-batch plan
and the solver-specification grammar.  Nothing here computes on the CPU.
"""
from . import _native, build  # noqa: F401
from ._native import load, last_error  # noqa: F401

__all__ = ["load", "last_error", "build"]
