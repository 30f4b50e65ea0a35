"""ctypes binding of libucfd_gb300.so.

Every entry point of ``include/*.h`` is declared here with its C argument
types, the way the reference examples bind their library
(``examples/omp3d.py:22-35``).  Array arguments accept numpy arrays (host
memory) or torch tensors (host or CUDA memory); they are passed as raw
pointers.  There is no fallback: if the library is missing, ``load()``
raises.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, byref, c_char_p, c_double, c_int, c_size_t, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libucfd_gb300.so")

_I, _D, _P = c_int, c_double, c_void_p


class TransferStats(ctypes.Structure):
    """``UCFDTransferStats`` of ucfd_gb300.h."""

    _fields_ = [("h2d_ms", c_double), ("h2d_bytes", c_double), ("d2h_ms", c_double), ("d2h_bytes", c_double),
                ("h2d_copies", ctypes.c_longlong), ("d2h_copies", ctypes.c_longlong)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def transfer_timing(on: bool) -> None:
    """Start (clearing the counters) or stop timing the library's host<->device copies."""
    call("UCFDSetTransferTiming", 1 if on else 0)


def transfer_stats() -> dict:
    st = TransferStats()
    call("UCFDGetTransferStats", ctypes.addressof(st))
    return st.as_dict()


HOST_STAGE, HOST_MAP = 0, 1


def set_host_array_access(mode: int) -> None:
    """UCFD_HOST_STAGE (0): host arrays are copied to the GPU; UCFD_HOST_MAP
    (1, the default): page-locked host face Jacobians are read in place by
    the kernels."""
    call("UCFDSetHostArrayAccess", int(mode))


def host_array_access() -> int:
    return int(load().UCFDGetHostArrayAccess())


class LaunchConfig(ctypes.Structure):
    """``UCFDLaunchConfig`` of ucfdlusgs.h."""

    _fields_ = [("threads_per_block", c_int), ("sweep_variant", c_int), ("run_mode", c_int), ("ms", c_double)]

    def as_dict(self) -> dict:
        return {"threads_per_block": self.threads_per_block, "sweep_variant": self.sweep_variant,
                "run_mode": self.run_mode, "ms": self.ms}


# name -> (restype, argtypes)
SIGNATURES = {
    # ucfd_gb300.h
    "UCFDGetLastError": (c_char_p, []),
    "UCFDSetConstants": (_I, [_D, _D, _D]),
    "UCFDVersion": (c_char_p, []),
    "UCFDDeviceInfo": (_I, [c_char_p, c_size_t, POINTER(c_int)]),
    "UCFDSelfTestTimeouts": (_I, [POINTER(c_int), POINTER(c_int)]),
    "UCFDSetTransferTiming": (_I, [_I]),
    "UCFDGetTransferStats": (_I, [_P]),
    "UCFDSetHostArrayAccess": (_I, [_I]),
    "UCFDGetHostArrayAccess": (_I, []),
    # ucfdmesh.h
    "UCFDMakeNeiEle": (_I, [_I, _I, _I, _P]),
    "UCFDMakeColoring": (_I, [_I, _I, _I, _P]),
    "UCFDGreedyColoring": (_I, [_I, _I, _P, _P, _P, _P, POINTER(c_int)]),
    "UCFDGreedyColoringCSR": (_I, [_I, _P, _P, _P, _P, _P, POINTER(c_int)]),
    "UCFDBFSColoringCSR": (_I, [_I, _P, _P, _P, _P, _P, POINTER(c_int)]),
    # ucfdlusgs.h
    "UCFDFlowSysCreate": (_I, [POINTER(c_void_p), _I, _I, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "UCFDFlowSysSetElement": (_I, [POINTER(c_void_p), _I, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "UCFDFlowSysDestroy": (_I, [POINTER(c_void_p)]),
    "UCFDFlowSysSetLUSGS": (_I, [POINTER(c_void_p), _P, _P]),
    "UCFDLUSGS_Pack": (_I, [_P, _I, _D, _D]),
    "UCFDLUSGS_Update": (_I, [_P, _I]),
    "UCFDLUSGS_NSPrepare": (_I, [_P, _D]),
    "UCFDLUSGS_RANSPrepare": (_I, [_P, _D]),
    "UCFDLUSGS_NSLowerSweep": (_I, [_P, _D]),
    "UCFDLUSGS_NSUpperSweep": (_I, [_P, _D]),
    "UCFDLUSGS_RANSLowerSweep": (_I, [_P, _D]),
    "UCFDLUSGS_RANSUpperSweep": (_I, [_P, _D]),
    "UCFDLUSGS_NSRANSPrepare": (_I, [_P, _D]),
    "UCFDLUSGS_NSRANSLowerSweep": (_I, [_P, _D]),
    "UCFDLUSGS_NSRANSUpperSweep": (_I, [_P, _D]),
    "UCFDFlowSysSetBLUSGS": (_I, [POINTER(c_void_p), _P, _P]),
    "UCFDBLUSGS_Pack": (_I, [_P, _I, _D]),
    "UCFDBLUSGS_KWSST_Pack": (_I, [_P, _I, _D, _D]),
    "UCFDBLUSGS_SA_Pack": (_I, [_P, _I, _D, _D]),
    "UCFDBLUSGS_Update": (_I, [_P, _I]),
    "UCFDBLUSGS_SubResidual": (_I, [_P, _I]),
    "UCFDBLUSGS_NSPrepare": (_I, [_P]),
    "UCFDBLUSGS_RANSPrepare": (_I, [_P]),
    "UCFDBLUSGS_NSLowerSweep": (_I, [_P]),
    "UCFDBLUSGS_RANSLowerSweep": (_I, [_P]),
    "UCFDBLUSGS_NSUpperSweep": (_I, [_P]),
    "UCFDBLUSGS_RANSUpperSweep": (_I, [_P]),
    "UCFDBLUSGS_Reset": (_I, [_P]),
    "UCFDFlowSysSetColoring": (_I, [_P, _P]),
    "UCFDFlowSysColorGreedy": (_I, [_P, POINTER(c_int)]),
    "UCFDFlowSysGetLevels": (_I, [_P, POINTER(c_int)]),
    "UCFDFlowSysSetPrecision": (_I, [_P, _I]),
    "UCFDFlowSysSetLaunch": (_I, [_P, _I]),
    "UCFDFlowSysAutotune": (_I, [_P, _I, POINTER(LaunchConfig)]),
    "UCFDFlowSysGetLaunchConfig": (_I, [_P, POINTER(LaunchConfig)]),
    "UCFDFlowSysSetLaunchConfig": (_I, [_P, POINTER(LaunchConfig)]),
    "UCFDFlowSysSetStream": (_I, [_P, _P, _I]),
    "UCFDLUSGS_Run": (_I, [_P, _I, _D, _I, _I, _P]),
    "UCFDBLUSGS_Solve": (_I, [_P, _D, _I, _I, POINTER(c_int), POINTER(c_double)]),
    "UCFDBLUSGS_Residual": (_I, [_P, POINTER(c_double)]),
    "UCFDBLUSGS_ResidualNoAlloc": (_I, [_P, _P]),
    # coloredlusgs.h
    "UCFDLegacySetDims": (_I, [_I, _I, _I]),
    "UCFDLegacySetPrecision": (_I, [_I]),
    "UCFDLegacyLastStatus": (_I, []),
    "serial_pre_lusgs": (None, [_I, _I, _D, _P, _P, _P, _P]),
    "parallel_pre_lusgs": (None, [_I, _I, _D, _P, _P, _P, _P]),
    "ns_serial_lower_sweep": (None, [_I, _I] + [_P] * 8),
    "ns_serial_upper_sweep": (None, [_I, _I] + [_P] * 8),
    "rans_serial_lower_sweep": (None, [_I, _I] + [_P] * 8),
    "rans_serial_upper_sweep": (None, [_I, _I] + [_P] * 8),
    "ns_parallel_lower_sweep": (None, [_I, _I, _I, _I] + [_P] * 10),
    "ns_parallel_upper_sweep": (None, [_I, _I, _I, _I] + [_P] * 10),
    "rans_parallel_lower_sweep": (None, [_I, _I, _I, _I] + [_P] * 10),
    "rans_parallel_upper_sweep": (None, [_I, _I, _I, _I] + [_P] * 10),
    "lusgs_serial_ns_update": (None, [_I, _P, _P]),
    "lusgs_parallel_ns_update": (None, [_I, _P, _P]),
    "lusgs_serial_rans_update": (None, [_I, _P, _P]),
    "lusgs_parallel_rans_update": (None, [_I, _P, _P]),
    "serial_ns_lower_sweep": (None, [_I, _I] + [_P] * 7),
    "serial_ns_upper_sweep": (None, [_I, _I] + [_P] * 7),
    "serial_ns_lusgs_update": (None, [_I, _P, _P]),
    "parallel_ns_lower_sweep": (None, [_I, _I, _I, _I] + [_P] * 9),
    "parallel_ns_upper_sweep": (None, [_I, _I, _I, _I] + [_P] * 9),
    # ucfdadjoint.h
    "UCFDReverseFaces": (_I, [_I, _I, _P, _P]),
    "UCFDColoredStep": (_I, [_I, _I, _I, _I, _I, _I, _P, _P, _I, _P, _P, _D] + [_P] * 10),
    "UCFDColoredStepAdjoint": (_I, [_I, _I, _I, _I, _I, _I, _P, _P, _P, _I, _P, _P, _D] + [_P] * 14),
    # ucfdmat.h
    "UCFDMatInit": (_I, [POINTER(c_void_p)]),
    "UCFDMatDestroy": (_I, [POINTER(c_void_p)]),
    "UCFDMatMult": (_I, [_D, _P, _P, _D, _P]),
    "UCFDMatMultFP32": (_I, [_D, _P, _P, _D, _P]),
    "UCFDMatMultPrecision": (_I, [_D, _P, _P, _D, _P, _I]),
    "UCFDMatCreateCSR": (_I, [POINTER(c_void_p), _I, _P, _P, _P]),
    "UCFDMatCreateBSR": (_I, [POINTER(c_void_p), _I, _I, _P, _P, _P]),
    "UCFDMatCreateCUDACSR": (_I, [POINTER(c_void_p), _I, _P, _P, _P]),
    "UCFDMatCreateCUDABSR": (_I, [POINTER(c_void_p), _I, _I, _P, _P, _P]),
    "UCFDMatUpdateValues": (_I, [_P]),
    "UCFDMatGetType": (_I, [_P, POINTER(c_char_p)]),
    # ucfdprecon.h
    "UCFDPreconCreatefromArrays": (_I, [POINTER(c_void_p), _P, _P, _P, _P]),
    "UCFDPreconCreateNone": (_I, [POINTER(c_void_p)]),
    "UCFDPreconPrepare": (_I, [_P]),
    "UCFDPreconDestroy": (_I, [POINTER(c_void_p)]),
    "UCFDPreconSetBLUSGS": (_I, [POINTER(c_void_p), _I, _I]),
    "UCFDPreconSetPBLUSGS": (_I, [POINTER(c_void_p), _I, _I, _I, _P]),
    "UCFDPreconSetCUDABLUSGS": (_I, [POINTER(c_void_p), _I, _I, _I, _P]),
    "UCFDPreconApply": (_I, [_P, _P]),
    "UCFDPreconSetPrecision": (_I, [_P, _I]),
    "UCFDPreconGetLevels": (_I, [_P, POINTER(c_int)]),
    # ucfdsolver.h
    "UCFDSolverInit": (_I, [POINTER(c_void_p)]),
    "UCFDSolverDestroy": (_I, [POINTER(c_void_p)]),
    "UCFDSolve": (_I, [_P, _P, _P, _P, _P]),
    "UCFDSolverGetResult": (_I, [_P, POINTER(c_int), POINTER(c_int), POINTER(c_double)]),
    "UCFDSolverTraceResidualHistory": (_I, [_P]),
    "UCFDSolverGetResidualHistory": (_I, [_P, _P]),
    "UCFDSolverCreateGMRES": (_I, [POINTER(c_void_p), _I, _I, _I, _D]),
    "UCFDSolverCreateBICGSTAB": (_I, [POINTER(c_void_p), _I, _I, _D]),
    "UCFDPreconSetILU": (_I, [POINTER(c_void_p), _I]),
    "UCFDPreconSetBILU": (_I, [POINTER(c_void_p), _I, _I]),
    "UCFDPreconSetPBILU": (_I, [POINTER(c_void_p), _I, _I, _I, _P]),
    "UCFDPreconSetCUDABILU": (_I, [POINTER(c_void_p), _I, _I, _I, _P]),
    "UCFDSolverCreateCUDAGMRES": (_I, [POINTER(c_void_p), _I, _I, _I, _D]),
    "UCFDSolverSetPrecision": (_I, [_P, _I]),
    "UCFDSolverSetHappyTol": (_I, [_P, _D]),
    "UCFDSolverSetCycleExit": (_I, [_P, _I]),
    "UCFDSolverGetArnoldiSteps": (_I, [_P, POINTER(c_int)]),
}

PREC_FP64, PREC_FP64_FMA, PREC_FP32 = 0, 1, 2

_lib = None


class UCFDError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where} failed with status {status}: {msg}")
        self.status = status


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the library (built by ``ucfd_sparse_gb300._build.build()``)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                           "(the CUDA library is required; there is no CPU fallback)")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def last_error() -> str:
    return load().UCFDGetLastError().decode()


def check(status: int, where: str) -> None:
    if status != 0:
        raise UCFDError(status, where, last_error())


def call(name: str, *args):
    """Call a status-returning entry point and raise on failure."""
    st = getattr(load(), name)(*args)
    check(st, name)
    return st


def call_void(name: str, *args):
    """Call a void array-API entry point and raise if it recorded a failure."""
    lib = load()
    getattr(lib, name)(*args)
    st = lib.UCFDLegacyLastStatus()
    check(st, name)


def ptr(a) -> int | None:
    """Raw data pointer of a numpy array or torch tensor (None for None)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags.c_contiguous:
            raise ValueError("arrays must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensors must be contiguous")
        return a.data_ptr()
    raise TypeError(f"unsupported array type {type(a)}")


def exported_symbols() -> list[str]:
    return sorted(SIGNATURES)
