"""Python mirror of the Krylov API (``ucfdmat.h``, ``ucfdprecon.h``,
``ucfdsolver.h``): BSR matrices, BLU-SGS preconditioners and GMRES(m)."""
from __future__ import annotations

from ctypes import byref, c_double, c_int, c_void_p

import numpy as np

from .lib import PREC_FP32, PREC_FP64, PREC_FP64_FMA, call, load, ptr

__all__ = ["SpMat", "Precon", "Solver"]


class SpMat:
    def __init__(self, bn, blk, rowptr, colidx, values, cuda=False):
        load()
        self._h = c_void_p()
        self._keep = [rowptr, colidx, values]
        self.bn, self.blk = bn, blk
        call("UCFDMatCreateCUDABSR" if cuda else "UCFDMatCreateBSR", byref(self._h), bn, blk, ptr(rowptr),
             ptr(colidx), ptr(values))

    def mult(self, alpha, x, beta, y, fp32=False, precision=None):
        """y = alpha A x + beta y; precision (PREC_*) picks the arithmetic
        (default FP64 in the reference's order, or FP32 values with fp32)."""
        if precision is not None:
            call("UCFDMatMultPrecision", alpha, self._h, ptr(x), beta, ptr(y), precision)
        else:
            call("UCFDMatMultFP32" if fp32 else "UCFDMatMult", alpha, self._h, ptr(x), beta, ptr(y))

    def update_values(self):
        call("UCFDMatUpdateValues", self._h)

    def destroy(self):
        if self._h:
            call("UCFDMatDestroy", byref(self._h))

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Precon:
    def __init__(self, rowptr=None, colidx=None, diagslots=None, values=None, none=False):
        load()
        self._h = c_void_p()
        self._keep = [rowptr, colidx, diagslots, values]
        if none:
            call("UCFDPreconCreateNone", byref(self._h))
        else:
            call("UCFDPreconCreatefromArrays", byref(self._h), ptr(rowptr), ptr(colidx), ptr(diagslots),
                 ptr(values))

    def set_blusgs(self, bn, block):
        call("UCFDPreconSetBLUSGS", byref(self._h), bn, block)

    def set_pblusgs(self, bn, block, ncolors, icolors, cuda=False):
        icolors = np.ascontiguousarray(icolors, dtype=np.int32)
        self._keep.append(icolors)
        call("UCFDPreconSetCUDABLUSGS" if cuda else "UCFDPreconSetPBLUSGS", byref(self._h), bn, block, ncolors,
             ptr(icolors))

    def set_bilu(self, bn, block):
        call("UCFDPreconSetBILU", byref(self._h), bn, block)

    def set_pbilu(self, bn, block, ncolors, icolors, cuda=False):
        icolors = np.ascontiguousarray(icolors, dtype=np.int32)
        self._keep.append(icolors)
        call("UCFDPreconSetCUDABILU" if cuda else "UCFDPreconSetPBILU", byref(self._h), bn, block, ncolors,
             ptr(icolors))

    def set_ilu(self, n):
        call("UCFDPreconSetILU", byref(self._h), n)

    def set_precision(self, prec):
        call("UCFDPreconSetPrecision", self._h, prec)

    def prepare(self):
        call("UCFDPreconPrepare", self._h)

    def apply(self, b):
        call("UCFDPreconApply", self._h, ptr(b))

    def levels(self) -> int:
        n = c_int()
        call("UCFDPreconGetLevels", self._h, byref(n))
        return n.value

    def destroy(self):
        if self._h:
            call("UCFDPreconDestroy", byref(self._h))

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Solver:
    """GMRES(m) (the default) or, with kind="bicgstab", BiCGSTAB (m unused)."""

    def __init__(self, n, m, maxiter, tol, cuda=False, kind="gmres"):
        load()
        self._h = c_void_p()
        if kind == "bicgstab":
            call("UCFDSolverCreateBICGSTAB", byref(self._h), n, maxiter, tol)
        else:
            call("UCFDSolverCreateCUDAGMRES" if cuda else "UCFDSolverCreateGMRES", byref(self._h), n, m, maxiter,
                 tol)
        self.maxiter = maxiter

    def set_precision(self, prec):
        call("UCFDSolverSetPrecision", self._h, prec)

    def set_cycle_exit(self, on=True):
        """GMRES: end a restart cycle once its residual estimate is low enough
        (UCFDSolverSetCycleExit; default off, the reference's iteration)."""
        call("UCFDSolverSetCycleExit", self._h, 1 if on else 0)

    def trace(self):
        call("UCFDSolverTraceResidualHistory", self._h)

    def solve(self, pc: Precon, A: SpMat, x, b):
        call("UCFDSolve", self._h, pc._h, A._h, ptr(x), ptr(b))

    def result(self):
        st, it, res = c_int(), c_int(), c_double()
        call("UCFDSolverGetResult", self._h, byref(st), byref(it), byref(res))
        return st.value, it.value, res.value

    def history(self):
        h = np.zeros(self.maxiter)
        call("UCFDSolverGetResidualHistory", self._h, ptr(h))
        return h

    def arnoldi_steps(self) -> int:
        n = c_int()
        call("UCFDSolverGetArnoldiSteps", self._h, byref(n))
        return n.value

    def destroy(self):
        if self._h:
            call("UCFDSolverDestroy", byref(self._h))

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
