"""phinum_gb300 -- GB300-native (sm_103a) lattice hot path of PhiNum.

The product is the C-ABI library libphinum_gpu.so (include/phinum_gpu.h),
built from phinum_gb300/csrc by phinum_gb300.build.  This package holds its
sources, the build step, the C++ adapter for the reference host
(adapter/phinum_dynamics.cpp) and a thin Python binding.
"""
from . import _lib  # noqa: F401
from ._lib import FP32, FP32_KAHAN, FP32_PAIR, FP64, ISLAND_DELTA, ISLAND_ENERGY, ISLAND_REFERENCE, PhnError  # noqa: F401
from .lattice import Adjoint, Ensemble, Lattice, Params, device_count  # noqa: F401
