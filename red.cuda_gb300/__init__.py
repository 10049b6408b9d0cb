"""red.cuda_gb300 -- GB300-native (sm_103a) implementation of red.cuda's
integration hot path.

The compute path is libredgb.so: CUDA kernels (csrc/kernels.cu) and a C++
host layer (csrc/sim.cu) behind the C ABI of include/redgb.h.  This Python
package is a thin ctypes mirror of that ABI (lib.py) plus host utilities:
red's record types (types.py), file formats (redio.py) and synthetic disks
(ic.py).
"""
from . import types, redio, ic, shard, proposer  # noqa: F401
from .build import build  # noqa: F401
from .lib import Sim, RedError, load, EXPORTS  # noqa: F401
