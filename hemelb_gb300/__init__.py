"""GB300-native HemeLB lattice-Boltzmann update (D3Q19, sm_103a).

The compute lives in libhemelb_gb300.so (hand-written CUDA kernels behind the C
ABI declared in include/hemelb_gb300.h); this package holds its in-tree build,
a ctypes binding and a thin Python mirror of the reference's LBM interface.
"""
from . import capi  # noqa: F401
from .capi import (FP16, FP32DEV, FP64, IOLET_LADD, IOLET_NASH, KERNEL_LBGK,  # noqa: F401
                   KERNEL_TRT, WALL_BFL, WALL_SBB, HlbgError)
from .lbm import (LBM, Case, InOutLetCosine, InOutLetParabolicVelocity,  # noqa: F401
                  LbmParameters, SyntheticGeometry)

__all__ = ["LBM", "LbmParameters", "SyntheticGeometry", "InOutLetCosine",
           "InOutLetParabolicVelocity", "Case", "HlbgError"]
