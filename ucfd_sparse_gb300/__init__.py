"""ucfd_sparse_gb300 -- GB300 (sm_103a) implementation of UCFD_SPARSE's
implicit hot path: colored LU-SGS, block LU-SGS with 5x5 face Jacobians, and
the BSR matvec / BLU-SGS preconditioner / GMRES(m) Krylov path, behind the
reference library's own C entry points (``include/*.h``,
``lib/libucfd_gb300.so``).

Submodules:
  lib           ctypes binding of every C entry point
  coloredlusgs  array (colored) LU-SGS API of the reference examples
  flowsys       FlowSys LU-SGS / BLU-SGS object API
  krylov        SpMat / Precon / Solver (GMRES)
  adjoint       torch.autograd.Function of one colored LU-SGS step
  meshgen       seeded synthetic meshes (jittered/permuted hex, Kuhn tets)
"""
from .lib import PREC_FP32, PREC_FP64, PREC_FP64_FMA, UCFDError, load  # noqa: F401

__version__ = "1.0"
