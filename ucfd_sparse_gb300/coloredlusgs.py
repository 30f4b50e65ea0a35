"""Python mirror of the colored (array-based) LU-SGS entry points.

Same function names and argument lists as the ctypes bindings of the
reference examples (``examples/omp3d.py:22-35``, ``examples/mpi3d.py:21-34``);
arrays are numpy arrays or torch tensors (host or CUDA).  ``colored_step``
runs one whole pre / lower / upper / update step over a colouring.
"""
from __future__ import annotations

import numpy as np

from .lib import PREC_FP64, PREC_FP64_FMA, call, call_void, load, ptr

__all__ = ["set_dims", "set_precision", "serial_pre_lusgs", "parallel_pre_lusgs", "ns_serial_lower_sweep",
           "ns_serial_upper_sweep", "ns_parallel_lower_sweep", "ns_parallel_upper_sweep",
           "rans_parallel_lower_sweep", "rans_parallel_upper_sweep", "rans_serial_lower_sweep",
           "rans_serial_upper_sweep", "lusgs_serial_ns_update", "lusgs_parallel_ns_update",
           "lusgs_parallel_rans_update", "lusgs_serial_rans_update", "colored_step", "make_nei_ele",
           "make_coloring", "greedy_coloring"]


def set_dims(nvars: int, nfvars: int, ndims: int):
    call("UCFDLegacySetDims", nvars, nfvars, ndims)


def set_precision(prec: int = PREC_FP64):
    call("UCFDLegacySetPrecision", prec)


def serial_pre_lusgs(neles, nface, factor, fnorm_vol, dt, diag, fspr):
    call_void("serial_pre_lusgs", neles, nface, factor, ptr(fnorm_vol), ptr(dt), ptr(diag), ptr(fspr))


def parallel_pre_lusgs(neles, nface, factor, fnorm_vol, dt, diag, fspr):
    call_void("parallel_pre_lusgs", neles, nface, factor, ptr(fnorm_vol), ptr(dt), ptr(diag), ptr(fspr))


def _serial(name):
    def f(neles, nface, nei_ele, fnorm_vol, vec_fnorm, upts, rhs, dub, diag, fspr):
        call_void(name, neles, nface, ptr(nei_ele), ptr(fnorm_vol), ptr(vec_fnorm), ptr(upts), ptr(rhs),
                  ptr(dub), ptr(diag), ptr(fspr))
    f.__name__ = name
    return f


def _parallel(name):
    def f(n0, ne, neles, nface, nei_ele, icolor, lcolor, fnorm_vol, vec_fnorm, upts, rhs, dub, diag, fspr):
        call_void(name, n0, ne, neles, nface, ptr(nei_ele), ptr(icolor), ptr(lcolor), ptr(fnorm_vol),
                  ptr(vec_fnorm), ptr(upts), ptr(rhs), ptr(dub), ptr(diag), ptr(fspr))
    f.__name__ = name
    return f


def _update(name):
    def f(neles, upts, rhs):
        call_void(name, neles, ptr(upts), ptr(rhs))
    f.__name__ = name
    return f


ns_serial_lower_sweep = _serial("ns_serial_lower_sweep")
ns_serial_upper_sweep = _serial("ns_serial_upper_sweep")
rans_serial_lower_sweep = _serial("rans_serial_lower_sweep")
rans_serial_upper_sweep = _serial("rans_serial_upper_sweep")
ns_parallel_lower_sweep = _parallel("ns_parallel_lower_sweep")
ns_parallel_upper_sweep = _parallel("ns_parallel_upper_sweep")
rans_parallel_lower_sweep = _parallel("rans_parallel_lower_sweep")
rans_parallel_upper_sweep = _parallel("rans_parallel_upper_sweep")
lusgs_serial_ns_update = _update("lusgs_serial_ns_update")
lusgs_parallel_ns_update = _update("lusgs_parallel_ns_update")
lusgs_serial_rans_update = _update("lusgs_serial_rans_update")
lusgs_parallel_rans_update = _update("lusgs_parallel_rans_update")


def colored_step(c: dict, icolor, ranges, diag, dub, rans: bool = False):
    """One colored LU-SGS step on the arrays of ``c`` (keys of
    ``meshgen.lusgs_case``): pre, lower sweep colour by colour, upper sweep
    in reverse colour order, update (omp3d.py:76-94 generalised to any
    number of colours).  ``ranges`` are the exclusive colour ends in icolor."""
    N, nf = c["neles"], c["nface"]
    lcolor = c["lcolor"]
    bounds = [0] + list(ranges)
    parallel_pre_lusgs(N, nf, 1.0, c["fnorm_vol"], c["dt"], diag, c["fspr"])
    lower = rans_parallel_lower_sweep if rans else ns_parallel_lower_sweep
    upper = rans_parallel_upper_sweep if rans else ns_parallel_upper_sweep
    args = (c["nei_ele"], icolor, lcolor, c["fnorm_vol"], c["vec_fnorm"], c["upts"], c["rhs"], dub, diag,
            c["fspr"])
    for k in range(len(ranges)):
        lower(bounds[k], bounds[k + 1], N, nf, *args)
    for k in reversed(range(len(ranges))):
        upper(bounds[k], bounds[k + 1], N, nf, *args)
    (lusgs_parallel_rans_update if rans else lusgs_parallel_ns_update)(N, c["upts"], c["rhs"])


# ---- connectivity and colouring (ucfdmesh.h) ---------------------------------
def make_nei_ele(m: int, n: int, l: int) -> np.ndarray:
    """pbutils.make_nei_ele (examples/utils/pbutils.py:4-36), native."""
    out = np.empty((6, m * n * l), dtype=np.int32)
    call("UCFDMakeNeiEle", m, n, l, ptr(out))
    return out


def make_coloring(m: int, n: int, l: int) -> np.ndarray:
    """pbutils.make_coloring (examples/utils/pbutils.py:39-56), native."""
    out = np.empty(m * n * l, dtype=np.int32)
    call("UCFDMakeColoring", m, n, l, ptr(out))
    return out


def greedy_coloring(nei_ele: np.ndarray):
    """Greedy first-fit colouring of a [nface, neles] table in index order.
    Returns (icolor, ranges, lcolor) with 1-based lcolor."""
    from ctypes import byref, c_int
    nface, neles = nei_ele.shape
    nei = np.ascontiguousarray(nei_ele, dtype=np.int32)
    lcolor = np.empty(neles, dtype=np.int32)
    icolor = np.empty(neles, dtype=np.int32)
    ranges = np.empty(64, dtype=np.int32)
    nc = c_int()
    call("UCFDGreedyColoring", neles, nface, ptr(nei), ptr(lcolor), ptr(icolor), ptr(ranges), byref(nc))
    return icolor, [int(x) for x in ranges[:nc.value]], lcolor


def greedy_coloring_csr(rowptr: np.ndarray, colidx: np.ndarray, order: str = "index"):
    """First-fit greedy colouring of a CSR graph -> (icolor, ranges, lcolor).

    order "index" visits cells by index (UCFDGreedyColoringCSR); "bfs" in
    breadth-first order (UCFDBFSColoringCSR), which needs fewer colours."""
    from ctypes import byref, c_int
    n = rowptr.shape[0] - 1
    rp = np.ascontiguousarray(rowptr, dtype=np.int32)
    ci = np.ascontiguousarray(colidx, dtype=np.int32)
    lcolor = np.empty(n, dtype=np.int32)
    icolor = np.empty(n, dtype=np.int32)
    ranges = np.empty(64, dtype=np.int32)
    nc = c_int()
    fn = {"index": "UCFDGreedyColoringCSR", "bfs": "UCFDBFSColoringCSR"}[order]
    call(fn, n, ptr(rp), ptr(ci), ptr(lcolor), ptr(icolor), ptr(ranges), byref(nc))
    return icolor, [int(x) for x in ranges[:nc.value]], lcolor
