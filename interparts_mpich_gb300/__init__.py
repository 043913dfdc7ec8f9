"""GB300-native immersed-boundary RK3 substep of the InterPartS particle-resolved DNS.

The compute path is the CUDA library libibm_rk3.so (csrc/, C ABI in
include/ibm_rk3.h); this package builds it in-tree and mirrors the
reference driver's subroutine API on top of it.
"""
from ._abi import (IBM_BC_FREESLIP, IBM_BC_NOSLIP, IBM_MODE_MIXED, IBM_MODE_MIXED_LEARNED, IBM_MODE_PLAIN_FP64,
                   ParticleState)
from .cases import Case, channel_case, settling_case
from .solver import IBMError, IBMSolver, library_path, load_library

__all__ = ["IBMSolver", "IBMError", "Case", "channel_case", "settling_case", "ParticleState", "load_library",
           "library_path", "IBM_MODE_PLAIN_FP64", "IBM_MODE_MIXED", "IBM_MODE_MIXED_LEARNED", "IBM_BC_NOSLIP",
           "IBM_BC_FREESLIP"]
