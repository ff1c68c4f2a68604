"""minifem: GB300 (sm_103a) implementation of Mini-FEM's assembly step.

Python mirror of the reference operators (src/headers/assembly.h,
src/headers/preconditioner.h, src/headers/matrix.h, src/headers/coloring.h) over
the C ABI of include/mfem_gpu.h.  Everything computes on the GPU; there is no
CPU fallback.
"""
from ._native import (AUTO, ATOMIC, FP32, FP64, GATHER, OP_ELA, OP_LAP, ORDER_REFERENCE,  # noqa: F401
                      ORDER_SORTED, SCATTER, MfemError, lib)
from .api import (Assembler, Batch, assembly, prec_init, prec_inversion, op_dim,  # noqa: F401
                  op_id)
from . import meshgen  # noqa: F401
