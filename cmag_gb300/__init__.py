"""cmag_gb300 -- GB300-native (sm_103a) weakly-compressible SPH time step of cmag.

The compute path is libcmag_sph.so (hand-written CUDA for sm_103a behind the C
ABI of include/cmag_sph.h); this package holds its ctypes binding and a Python
mirror of the reference solver classes."""
from . import _abi  # noqa: F401
from ._abi import *  # noqa: F401,F403
from ._lib import CmagError, LIB_PATH, lib  # noqa: F401
from .batch import Batch  # noqa: F401
from .systems import (DamBreakSystem, PeristalsisSystem, PoiseuilleFlowSystem,  # noqa: F401
                      sort_particles)
