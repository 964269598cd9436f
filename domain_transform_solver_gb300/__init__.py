"""GB300-native Domain Transform Solver (DTS) and Hardware-Friendly
Bilateral Solver (HFBS).

The compute path is libdtsgb.so (hand-written sm_103a CUDA behind the C ABI
of include/dtsgb.h); this package is its Python mirror of the reference's
class API.  Importing the package loads the library and fails loudly when it
is missing.
"""
from ._lib import DtsgbError, load as _load
from .solvers import *  # noqa: F401,F403
from .solvers import __all__ as _solvers_all

_load()

__all__ = list(_solvers_all)
