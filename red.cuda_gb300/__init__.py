"""red.cuda_gb300 -- GB300-native (sm_103a) implementation of red.cuda's
integration hot path.

The compute path is libredgb.so (CUDA kernels + a C++ host layer behind a C
ABI, declared in include/redgb.h).  This Python package is a thin ctypes
mirror of that ABI plus host utilities (red file formats, synthetic disks).
"""
from . import types, redio, ic  # noqa: F401
