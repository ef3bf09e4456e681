"""GB300-native (sm_103a) hybrid PIC ion step of SWAP behind its Fortran
subroutine interface.  See include/swap_gpu.h for the C-ABI."""
from .hybrid import Hybrid, RunConfig, config  # noqa: F401

__all__ = ["Hybrid", "RunConfig", "config"]
