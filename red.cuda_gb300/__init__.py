"""red.cuda_gb300 -- GB300-native (sm_103a) implementation of red.cuda's
integration hot path.

The compute path is libredgb.so behind the C ABI of include/redgb.h: the
fused stage kernel (csrc/stage.cuh, one translation unit per arithmetic mode:
csrc/stage_{mixed,fp32,fp64,exact}.cu), the step controller, y_{n+1},
collision, ejection and state-transfer kernels (csrc/kernels.cu), the C++ host
layer (planner, graph capture, events, autotuner: csrc/sim.cu), the
allocation-free gravity entry point (csrc/noalloc.cu), the GPU disk generator
(csrc/populate.cu) and the learned step proposer (csrc/proposer.cu).  This
Python package is a thin ctypes mirror of that ABI (lib.py) plus host
utilities: red's record types (types.py), file formats (redio.py), synthetic
disks (ic.py), the per-rank split (shard.py) and the proposer's training loop
(proposer.py).  The red-compatible command-line driver is driver/redgb_run.cpp.
"""
from . import types, redio, ic, shard, proposer  # noqa: F401
from .build import build  # noqa: F401
from .lib import Sim, RedError, load, EXPORTS  # noqa: F401
