"""Test infrastructure: ctypes drivers of the CPU oracle.

Two CPU implementations of the hot path are wrapped here, both used only as
checkers by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
bench.py:

* ``Port``  -- oracle/ucfd_oracle.c, the C restatement of the reference
  algorithm (built by ``make -C oracle port`` into oracle/_build/);
* ``Ref``   -- the reference library itself, compiled from the reference
  sources by ``make -C oracle ref`` into oracle/_ref/ (only where the
  reference source tree is present).

The functions below drive whole steps (pre/lower/upper/update, BLU-SGS
sweeps, BSR/GMRES solves) on numpy arrays and return numpy results.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, byref, c_double, c_int, c_int8, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")
# root of a UCFD_SPARSE source tree; the reference libraries are built only
# where this names one
REF_SRC = os.environ.get("UCFD_REFERENCE_SRC")

_I, _D, _P = c_int, c_double, c_void_p


def build_port() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


def build_ref() -> bool:
    """Compile the reference sources into oracle/_ref (False if
    UCFD_REFERENCE_SRC does not name a source tree)."""
    if not ref_src_present():
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"], check=True)
    return True


def ref_src_present() -> bool:
    return bool(REF_SRC) and os.path.isdir(os.path.join(REF_SRC, "src", "lusgs"))


def ref_available() -> bool:
    return os.path.exists(os.path.join(REF, "liblusgs_ref.so")) and os.path.exists(
        os.path.join(REF, "libkrylov_ref.so"))


def P(a):
    return None if a is None else a.ctypes.data


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


# ---------------------------------------------------------------------------
# the C restatement
# ---------------------------------------------------------------------------
class Port:
    def __init__(self, fast: bool = False):
        name = "liboracle_fast.so" if fast else "liboracle_pin.so"
        path = os.path.join(BUILD, name)
        if not os.path.exists(path):
            build_port()
        L = ctypes.CDLL(path)
        sig = {
            "oracle_set_constants": (None, [_D, _D]),
            "oracle_lusgs_pack": (None, [_I, _I, _I, _I, _D, _D] + [_P] * 8),
            "oracle_lusgs_update": (None, [_I, _I, _I, _P, _P, _P]),
            "oracle_lusgs_prepare": (None, [_I, _I, _I, _D, _P, _P, _P, _P, _P, _P]),
            "oracle_lusgs_lower": (None, [_I, _I, _I, _D, _P, _I, _I, _I, _I, _I] + [_P] * 10),
            "oracle_lusgs_upper": (None, [_I, _I, _I, _D, _P, _I, _I, _I, _I, _I] + [_P] * 10),
            "oracle_legacy_pre": (None, [_I, _I, _D, _P, _P, _P, _P]),
            "oracle_legacy_sweep": (None, [_I, _I, _I, _I, _I, _I, _I, _I, _I] + [_P] * 10),
            "oracle_legacy_serial_sweep": (None, [_I, _I, _I, _I, _I, _I, _I] + [_P] * 8),
            "oracle_legacy_update": (None, [_I, _I, _I, _I, _P, _P]),
            "oracle_ludcmp": (None, [_I, _P]),
            "oracle_lusub": (None, [_I, _P, _P]),
            "oracle_blusgs_pack": (None, [_I, _I, _I, _I, _D, _P, _P, _P, _P, _P]),
            "oracle_tblusgs_pack": (None, [_I, _I, _I, _I, _I, _D, _D, _P, _P, _P, _P, _P]),
            "oracle_blusgs_update": (None, [_I, _I, _I, _P, _P, _P]),
            "oracle_blusgs_sub_residual": (None, [_I, _I, _I, _P, _P, _P, _P, _P]),
            "oracle_blusgs_prepare": (None, [_I, _I, _I] + [_P] * 7),
            "oracle_blusgs_lower": (None, [_I, _I, _I, _I, _I] + [_P] * 10),
            "oracle_blusgs_upper": (None, [_I, _I, _I, _I, _I] + [_P] * 10),
            "oracle_bsr_spmv": (None, [_I, _I, _P, _P, _P, _D, _P, _D, _P]),
            "oracle_blusgs_precon_prepare": (None, [_I, _I, _P, _P, _P]),
            "oracle_blusgs_precon_apply": (None, [_I, _I, _P, _P, _P, _P, _P, _P]),
            "oracle_pblusgs_precon_apply": (None, [_I, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
            "oracle_gmres": (_I, [_I, _I, _P, _P, _P, _I, _I, _P, _P, _P, _I, _I, _D, _D, _P, _P,
                                  POINTER(c_int), POINTER(c_double), _P]),
            "oracle_lusubmattrans": (None, [_I, _P, _P]),
            "oracle_bilu_prepare": (None, [_I, _I, _P, _P, _P, _P]),
            "oracle_bilu_apply": (None, [_I, _I, _P, _P, _P, _P, _P]),
            "oracle_ilu_prepare": (None, [_I, _P, _P, _P, _P]),
            "oracle_ilu_apply": (None, [_I, _P, _P, _P, _P, _P]),
            "oracle_bicgstab": (_I, [_I, _I, _P, _P, _P, _I, _I, _P, _P, _P, _P, _I, _D, _P, _P,
                                     POINTER(c_int), POINTER(c_double), _P]),
            "oracle_greedy_coloring_csr": (_I, [_I, _P, _P, _P]),
        }
        for n, (r, a) in sig.items():
            f = getattr(L, n)
            f.restype = r
            f.argtypes = a
        self.L = L

    # ---- colouring --------------------------------------------------------
    def greedy_coloring_csr(self, rowptr, colidx):
        """Greedy first-fit colouring in index order -> (icolor, ranges,
        lcolor): cells grouped by colour in ascending index, the end of each
        colour's range, 1-based colour of each cell."""
        rp, ci = _i32(rowptr), _i32(colidx)
        n = rp.shape[0] - 1
        col = np.empty(n, dtype=np.int32)
        nc = self.L.oracle_greedy_coloring_csr(n, P(rp), P(ci), P(col))
        if nc < 0:
            raise MemoryError("oracle_greedy_coloring_csr: allocation failed")
        icolor = np.argsort(col, kind="stable").astype(np.int32)
        ranges = [int(x) for x in np.cumsum(np.bincount(col, minlength=nc))]
        return icolor, ranges, col + 1

    # ---- colored array API ------------------------------------------------
    def legacy_step(self, c: dict, icolor, ranges, lcolor, nsteps: int = 1, rans: bool = False,
                    nfvars: int = 5, ndims: int = 3):
        """nsteps colored LU-SGS steps; returns (upts, rhs, dub, diag)."""
        N, nf, nv = c["neles"], c["nface"], c["nvars"]
        upts, rhs = c["upts"].copy(), c["rhs"].copy()
        dub = np.zeros_like(rhs)
        diag = np.zeros(N)
        icolor, lcolor = _i32(icolor), _i32(lcolor)
        nei, fnv, vec, fspr, dt = _i32(c["nei_ele"]), _f64(c["fnorm_vol"]), _f64(c["vec_fnorm"]), _f64(
            c["fspr"]), _f64(c["dt"])
        bounds = [0] + list(ranges)
        for _ in range(nsteps):
            rhs[:] = c["rhs"]
            self.L.oracle_legacy_pre(N, nf, 1.0, P(fnv), P(dt), P(diag), P(fspr))
            for k in range(len(ranges)):
                self.L.oracle_legacy_sweep(0, int(rans), bounds[k], bounds[k + 1], N, nf, nv, nfvars, ndims, P(nei),
                                           P(icolor), P(lcolor), P(fnv), P(vec), P(upts), P(rhs), P(dub), P(diag),
                                           P(fspr))
            for k in reversed(range(len(ranges))):
                self.L.oracle_legacy_sweep(1, int(rans), bounds[k], bounds[k + 1], N, nf, nv, nfvars, ndims, P(nei),
                                           P(icolor), P(lcolor), P(fnv), P(vec), P(upts), P(rhs), P(dub), P(diag),
                                           P(fspr))
            self.L.oracle_legacy_update(int(rans), N, nv, nfvars, P(upts), P(rhs))
        return upts, rhs, dub, diag

    def legacy_serial_step(self, c: dict, nfvars=5, ndims=3, rans=False):
        N, nf, nv = c["neles"], c["nface"], c["nvars"]
        upts, rhs = c["upts"].copy(), c["rhs"].copy()
        dub = np.zeros_like(rhs)
        diag = np.zeros(N)
        nei, fnv, vec, fspr, dt = _i32(c["nei_ele"]), _f64(c["fnorm_vol"]), _f64(c["vec_fnorm"]), _f64(
            c["fspr"]), _f64(c["dt"])
        self.L.oracle_legacy_pre(N, nf, 1.0, P(fnv), P(dt), P(diag), P(fspr))
        for up in (0, 1):
            self.L.oracle_legacy_serial_sweep(up, int(rans), N, nf, nv, nfvars, ndims, P(nei), P(fnv), P(vec),
                                              P(upts), P(rhs), P(dub), P(diag), P(fspr))
        self.L.oracle_legacy_update(int(rans), N, nv, nfvars, P(upts), P(rhs))
        return upts, rhs, dub, diag

    # ---- FlowSys scalar LU-SGS --------------------------------------------
    def flowsys_lusgs_step(self, fs: dict, upts, rhs, dt, dsrc, fspr, tfspr=None, kappa=1.0, a0=0.0,
                           turb_factor=1.0, rans=False, nsteps=1):
        """Pack / NSPrepare / NS lower / NS upper [/ RANS ...] / Update."""
        N, nv, nfv = fs["nlocal"], fs["nvars"], fs["nfvars"]
        ndims, nF = fs.get("ndims", 3), fs["nfaces"]
        neles = dt.shape[0]
        ids = _i32(fs["cell_ids"])
        upts = _f64(upts).copy()
        u = np.zeros(nv * N)
        du = np.zeros(nv * N)
        diag = np.zeros(nv * N)
        rp, ci, sl, sd = _i32(fs["rowptr"]), _i32(fs["colidx"]), _i32(fs["slots"]), np.ascontiguousarray(
            fs["sides"], dtype=np.int8)
        fa, fn, rv = _f64(fs["face_area"]), _f64(fs["face_normal"]), _f64(fs["rcp_vol"])
        rhs, dt, dsrc, fspr = _f64(rhs), _f64(dt), _f64(dsrc), _f64(fspr)
        tf = _f64(tfspr) if tfspr is not None else None
        for _ in range(nsteps):
            self.L.oracle_lusgs_pack(N, neles, nv, nfv, turb_factor, a0, P(ids), P(upts), P(rhs), P(dt), P(dsrc),
                                     P(u), P(du), P(diag))
            self.L.oracle_lusgs_prepare(N, 0, nfv, kappa, P(rp), P(sl), P(fa), P(rv), P(fspr), P(diag))
            g = (P(rp), P(ci), P(sd), P(sl), P(fa), P(fn), P(rv), P(diag), P(u), P(du))
            self.L.oracle_lusgs_lower(0, 0, nfv, kappa, P(fspr), N, nv, nfv, ndims, nF, *g)
            self.L.oracle_lusgs_upper(0, 0, nfv, kappa, P(fspr), N, nv, nfv, ndims, nF, *g)
            if rans:
                self.L.oracle_lusgs_prepare(N, nfv, nv, kappa, P(rp), P(sl), P(fa), P(rv), P(tf), P(diag))
                self.L.oracle_lusgs_lower(1, nfv, nv, kappa, P(tf), N, nv, nfv, ndims, nF, *g)
                self.L.oracle_lusgs_upper(1, nfv, nv, kappa, P(tf), N, nv, nfv, ndims, nF, *g)
            self.L.oracle_lusgs_update(N, neles, nv, P(ids), P(du), P(upts))
        return upts, du.reshape(nv, N), diag.reshape(nv, N)

    # ---- FlowSys BLU-SGS ---------------------------------------------------
    def flowsys_blusgs(self, fs: dict, rhs, dt, jmat, vol, upts, nsweeps=1, a0=0.0):
        """Pack / NSPrepare / Reset / (lower, upper, SubResidual) x nsweeps /
        Update.  Returns (upts, du [N][nv] AoS, resid [nv][neles], LU diag)."""
        N, nv, nfv, nF = fs["nlocal"], fs["nvars"], fs["nfvars"], fs["nfaces"]
        neles = dt.shape[0]
        ids = _i32(fs["cell_ids"])
        rp, ci, sl, sd = _i32(fs["rowptr"]), _i32(fs["colidx"]), _i32(fs["slots"]), np.ascontiguousarray(
            fs["sides"], dtype=np.int8)
        fa, rv = _f64(fs["face_area"]), _f64(fs["rcp_vol"])
        rhs, dt, jmat, vol = _f64(rhs), _f64(dt), _f64(jmat), _f64(vol)
        upts = _f64(upts).copy()
        rrhs = np.zeros(N * nv)
        diag = np.zeros(N * nfv * nfv)
        du = np.zeros(N * nv)
        dup = np.zeros(N * nv)
        res = np.zeros(nv * neles)
        self.L.oracle_blusgs_pack(N, neles, nv, nfv, a0, P(ids), P(rhs), P(dt), P(rrhs), P(diag))
        self.L.oracle_blusgs_prepare(N, nfv, nF, P(rp), P(sl), P(sd), P(fa), P(rv), P(diag), P(jmat))
        for _ in range(nsweeps):
            g = (P(rp), P(ci), P(sd), P(sl), P(fa), P(rv), P(rrhs), P(diag), P(jmat), P(du))
            self.L.oracle_blusgs_lower(0, nfv, N, nv, nF, *g)
            self.L.oracle_blusgs_upper(0, nfv, N, nv, nF, *g)
            self.L.oracle_blusgs_sub_residual(N, neles, nv, P(ids), P(vol), P(du), P(dup), P(res))
        self.L.oracle_blusgs_update(N, neles, nv, P(ids), P(du), P(upts))
        return upts, du.reshape(N, nv), res.reshape(nv, neles), diag.reshape(N, nfv, nfv)

    def blusgs_phases(self, fs: dict, rhs, dt, jmat, vol, upts, a0=0.0):
        """The steps of flowsys_blusgs as separate calls (for timing them one
        by one): see BlusgsPhases."""
        return _PortBlusgsPhases(self, fs, rhs, dt, jmat, vol, upts, a0)

    # ---- Krylov -------------------------------------------------------------
    def bsr_spmv(self, s: dict, x, alpha=1.0, beta=0.0, y=None):
        bn, blk = s["bn"], s["blk"]
        y = np.zeros(bn * blk) if y is None else _f64(y).copy()
        x = _f64(x)
        self.L.oracle_bsr_spmv(bn, blk, P(_i32(s["rowptr"])), P(_i32(s["colidx"])), P(_f64(s["values"])), alpha,
                               P(x), beta, P(y))
        return y

    def precon_diag(self, s: dict):
        bn, blk = s["bn"], s["blk"]
        d = np.zeros(bn * blk * blk)
        self.L.oracle_blusgs_precon_prepare(bn, blk, P(_i32(s["diagslots"])), P(_f64(s["values"])), P(d))
        return d

    def precon_apply(self, s: dict, b, icolors=None):
        bn, blk = s["bn"], s["blk"]
        d = self.precon_diag(s)
        b = _f64(b).copy()
        args = (P(_i32(s["rowptr"])), P(_i32(s["colidx"])), P(_i32(s["diagslots"])), P(_f64(s["values"])), P(d),
                P(b))
        if icolors is None:
            self.L.oracle_blusgs_precon_apply(bn, blk, *args)
        else:
            ic = _i32(icolors)
            self.L.oracle_pblusgs_precon_apply(bn, blk, len(ic) - 1, P(ic), *args)
        return b

    def gmres(self, s: dict, b, m=30, maxiter=50, tol=1e-10, pc="blusgs", icolors=None, haptol=1e-12, x0=None):
        bn, blk = s["bn"], s["blk"]
        kind = {"none": 0, "blusgs": 1, "pblusgs": 2}[pc]
        d = self.precon_diag(s) if kind else np.zeros(1)
        ic = _i32(icolors) if icolors is not None else np.zeros(1, dtype=np.int32)
        x = np.zeros(bn * blk) if x0 is None else _f64(x0).copy()
        it, res = c_int(), c_double()
        hist = np.zeros(maxiter + 1)
        st = self.L.oracle_gmres(bn, blk, P(_i32(s["rowptr"])), P(_i32(s["colidx"])), P(_f64(s["values"])), kind,
                                 len(ic) - 1, P(ic), P(_i32(s["diagslots"])), P(d), m, maxiter, tol, haptol, P(x),
                                 P(_f64(b)), byref(it), byref(res), P(hist))
        return x, st, it.value, res.value, hist[:it.value + 1]

    def bilu_factor(self, s: dict):
        """Block ILU(0) factors (bilu.c:5-62) of s["values"], natural order."""
        v = _f64(s["values"]).copy()
        self.L.oracle_bilu_prepare(s["bn"], s["blk"], P(_i32(s["rowptr"])), P(_i32(s["colidx"])),
                                   P(_i32(s["diagslots"])), P(v))
        return v

    def bilu_apply(self, s: dict, fvalues, b):
        b = _f64(b).copy()
        self.L.oracle_bilu_apply(s["bn"], s["blk"], P(_i32(s["rowptr"])), P(_i32(s["colidx"])),
                                 P(_i32(s["diagslots"])), P(_f64(fvalues)), P(b))
        return b

    def ilu_factor(self, s: dict):
        """Scalar ILU(0) factors (ilu.c:4-47) of a CSR matrix (blk 1)."""
        v = _f64(s["values"]).copy()
        self.L.oracle_ilu_prepare(s["bn"], P(_i32(s["rowptr"])), P(_i32(s["colidx"])), P(_i32(s["diagslots"])),
                                  P(v))
        return v

    def ilu_apply(self, s: dict, fvalues, b):
        b = _f64(b).copy()
        self.L.oracle_ilu_apply(s["bn"], P(_i32(s["rowptr"])), P(_i32(s["colidx"])), P(_i32(s["diagslots"])),
                                P(_f64(fvalues)), P(b))
        return b

    def bicgstab(self, s: dict, b, maxiter=50, tol=1e-10, pc="blusgs", icolors=None, x0=None):
        """BiCGSTAB of bicgstab.c:24-128 -> (x, stat, iters, resnorm, hist)."""
        bn, blk = s["bn"], s["blk"]
        kind = {"none": 0, "blusgs": 1, "pblusgs": 2, "bilu": 3, "ilu": 4}[pc]
        d = self.precon_diag(s) if kind in (1, 2) else np.zeros(1)
        fv = self.bilu_factor(s) if kind == 3 else self.ilu_factor(s) if kind == 4 else np.zeros(1)
        ic = _i32(icolors) if icolors is not None else np.zeros(1, dtype=np.int32)
        x = np.zeros(bn * blk) if x0 is None else _f64(x0).copy()
        it, res = c_int(), c_double()
        hist = np.zeros(max(maxiter, 1))
        st = self.L.oracle_bicgstab(bn, blk, P(_i32(s["rowptr"])), P(_i32(s["colidx"])), P(_f64(s["values"])),
                                    kind, len(ic) - 1, P(ic), P(_i32(s["diagslots"])), P(d), P(fv), maxiter, tol,
                                    P(x), P(_f64(b)), byref(it), byref(res), P(hist))
        return x, st, it.value, res.value, hist[:maxiter]


# ---------------------------------------------------------------------------
# the reference library compiled from its own sources
# ---------------------------------------------------------------------------
class Ref:
    def __init__(self, fast: bool = False):
        sfx = "_fast" if fast else ""
        self.lus = ctypes.CDLL(os.path.join(REF, f"liblusgs_ref{sfx}.so"))
        self.kry = ctypes.CDLL(os.path.join(REF, f"libkrylov_ref{sfx}.so"))
        H = POINTER(c_void_p)
        for n, a in {
            "UCFDFlowSysCreate": [H, _I, _I, _I, _I, _I, _I] + [_P] * 7,
            "UCFDFlowSysSetElement": [H, _I, _I, _I] + [_P] * 7,
            "UCFDFlowSysDestroy": [H],
            "UCFDFlowSysSetLUSGS": [H, _P, _P],
            "UCFDFlowSysSetBLUSGS": [H, _P, _P],
            "UCFDLUSGS_Pack": [_P, _I, _D, _D],
            "UCFDLUSGS_Update": [_P, _I],
            "UCFDLUSGS_NSPrepare": [_P, _D],
            "UCFDLUSGS_RANSPrepare": [_P, _D],
            "UCFDLUSGS_NSLowerSweep": [_P, _D],
            "UCFDLUSGS_NSUpperSweep": [_P, _D],
            "UCFDLUSGS_RANSLowerSweep": [_P, _D],
            "UCFDLUSGS_RANSUpperSweep": [_P, _D],
            "UCFDBLUSGS_Pack": [_P, _I, _D],
            "UCFDBLUSGS_KWSST_Pack": [_P, _I, _D, _D],
            "UCFDBLUSGS_SA_Pack": [_P, _I, _D, _D],
            "UCFDBLUSGS_NSPrepare": [_P],
            "UCFDBLUSGS_RANSPrepare": [_P],
            "UCFDBLUSGS_NSLowerSweep": [_P],
            "UCFDBLUSGS_NSUpperSweep": [_P],
            "UCFDBLUSGS_RANSLowerSweep": [_P],
            "UCFDBLUSGS_RANSUpperSweep": [_P],
            "UCFDBLUSGS_SubResidual": [_P, _I],
            "UCFDBLUSGS_Update": [_P, _I],
            "UCFDBLUSGS_Reset": [_P],
        }.items():
            f = getattr(self.lus, n)
            f.restype = _I
            f.argtypes = a
        for n, a in {
            "UCFDMatCreateBSR": [H, _I, _I, _P, _P, _P],
            "UCFDMatMult": [_D, _P, _P, _D, _P],
            "UCFDMatDestroy": [H],
            "UCFDPreconCreatefromArrays": [H, _P, _P, _P, _P],
            "UCFDPreconSetBLUSGS": [H, _I, _I],
            "UCFDPreconSetPBLUSGS": [H, _I, _I, _I, _P],
            "UCFDPreconPrepare": [_P],
            "UCFDPreconDestroy": [H],
            "UCFDSolverCreateGMRES": [H, _I, _I, _I, _D],
            "UCFDSolverCreateBICGSTAB": [H, _I, _I, _D],
            "UCFDPreconSetBILU": [H, _I, _I],
            "UCFDPreconSetPBILU": [H, _I, _I, _I, _P],
            "UCFDPreconSetILU": [H, _I],
            "UCFDSolve": [_P, _P, _P, _P, _P],
            "UCFDSolverGetResult": [_P, POINTER(c_int), POINTER(c_int), POINTER(c_double)],
            "UCFDSolverTraceResidualHistory": [_P],
            "UCFDSolverGetResidualHistory": [_P, _P],
            "UCFDSolverDestroy": [H],
        }.items():
            f = getattr(self.kry, n)
            f.restype = _I
            f.argtypes = a

    def _sys(self, fs, nelem=1):
        h = c_void_p()
        keep = [_i32(fs["rowptr"]), _i32(fs["colidx"]), _i32(fs["slots"]),
                np.ascontiguousarray(fs["sides"], dtype=np.int8), _f64(fs["face_area"]), _f64(fs["face_normal"]),
                _f64(fs["rcp_vol"])]
        self.lus.UCFDFlowSysCreate(byref(h), fs["nlocal"], fs["nvars"], fs["nfvars"], fs.get("ndims", 3),
                                   fs["nfaces"], nelem, *[P(a) for a in keep])
        return h, keep

    def flowsys_lusgs_step(self, fs, upts, rhs, dt, dsrc, fspr, tfspr=None, kappa=1.0, a0=0.0, turb_factor=1.0,
                           rans=False, nsteps=1):
        h, keep = self._sys(fs)
        upts = _f64(upts).copy()
        rhs, dt, dsrc, fspr = _f64(rhs), _f64(dt), _f64(dsrc), _f64(fspr)
        tf = _f64(tfspr) if tfspr is not None else None
        ids = _i32(fs["cell_ids"])
        neles = dt.shape[0]
        res = np.zeros_like(upts)
        vol = np.ones(neles)
        self.lus.UCFDFlowSysSetLUSGS(byref(h), P(fspr), P(tf))
        self.lus.UCFDFlowSysSetElement(byref(h), 0, neles, 6, P(ids), P(upts), P(rhs), P(dt), P(dsrc), P(vol),
                                       P(res))
        for _ in range(nsteps):
            self.lus.UCFDLUSGS_Pack(h, 0, turb_factor, a0)
            self.lus.UCFDLUSGS_NSPrepare(h, kappa)
            self.lus.UCFDLUSGS_NSLowerSweep(h, kappa)
            self.lus.UCFDLUSGS_NSUpperSweep(h, kappa)
            if rans:
                self.lus.UCFDLUSGS_RANSPrepare(h, kappa)
                self.lus.UCFDLUSGS_RANSLowerSweep(h, kappa)
                self.lus.UCFDLUSGS_RANSUpperSweep(h, kappa)
            self.lus.UCFDLUSGS_Update(h, 0)
        self.lus.UCFDFlowSysDestroy(byref(h))
        return upts

    def flowsys_blusgs(self, fs, rhs, dt, jmat, vol, upts, nsweeps=1, a0=0.0):
        h, keep = self._sys(fs)
        upts = _f64(upts).copy()
        rhs, dt, jmat, vol = _f64(rhs), _f64(dt), _f64(jmat), _f64(vol)
        ids = _i32(fs["cell_ids"])
        neles = dt.shape[0]
        res = np.zeros_like(upts)
        dsrc = np.zeros_like(upts)
        self.lus.UCFDFlowSysSetBLUSGS(byref(h), P(jmat), None)
        self.lus.UCFDFlowSysSetElement(byref(h), 0, neles, 6, P(ids), P(upts), P(rhs), P(dt), P(dsrc), P(vol),
                                       P(res))
        self.lus.UCFDBLUSGS_Pack(h, 0, a0)
        self.lus.UCFDBLUSGS_NSPrepare(h)
        self.lus.UCFDBLUSGS_Reset(h)
        for _ in range(nsweeps):
            self.lus.UCFDBLUSGS_NSLowerSweep(h)
            self.lus.UCFDBLUSGS_NSUpperSweep(h)
            self.lus.UCFDBLUSGS_SubResidual(h, 0)
        self.lus.UCFDBLUSGS_Update(h, 0)
        self.lus.UCFDFlowSysDestroy(byref(h))
        return upts, res

    def blusgs_phases(self, fs, rhs, dt, jmat, vol, upts, a0=0.0):
        """The reference's own FlowSys BLU-SGS calls one by one: see
        BlusgsPhases."""
        return _RefBlusgsPhases(self, fs, rhs, dt, jmat, vol, upts, a0)

    def bsr_spmv(self, s, x, alpha=1.0, beta=0.0, y=None):
        h = c_void_p()
        rp, ci, v = _i32(s["rowptr"]), _i32(s["colidx"]), _f64(s["values"])
        self.kry.UCFDMatCreateBSR(byref(h), s["bn"], s["blk"], P(rp), P(ci), P(v))
        y = np.zeros(s["bn"] * s["blk"]) if y is None else _f64(y).copy()
        x = _f64(x)
        self.kry.UCFDMatMult(alpha, h, P(x), beta, P(y))
        self.kry.UCFDMatDestroy(byref(h))
        return y

    def gmres(self, s, b, m=30, maxiter=50, tol=1e-10):
        """Natural-order BLU-SGS preconditioned GMRES of the reference."""
        A, pc, sv = c_void_p(), c_void_p(), c_void_p()
        rp, ci, v, ds = _i32(s["rowptr"]), _i32(s["colidx"]), _f64(s["values"]), _i32(s["diagslots"])
        self.kry.UCFDMatCreateBSR(byref(A), s["bn"], s["blk"], P(rp), P(ci), P(v))
        self.kry.UCFDPreconCreatefromArrays(byref(pc), P(rp), P(ci), P(ds), P(v))
        self.kry.UCFDPreconSetBLUSGS(byref(pc), s["bn"], s["blk"])
        self.kry.UCFDPreconPrepare(pc)
        n = s["bn"] * s["blk"]
        self.kry.UCFDSolverCreateGMRES(byref(sv), n, m, maxiter, tol)
        self.kry.UCFDSolverTraceResidualHistory(sv)
        x = np.zeros(n)
        b = _f64(b)
        self.kry.UCFDSolve(sv, pc, A, P(x), P(b))
        st, it, res = c_int(), c_int(), c_double()
        self.kry.UCFDSolverGetResult(sv, byref(st), byref(it), byref(res))
        hist = np.zeros(maxiter)
        self.kry.UCFDSolverGetResidualHistory(sv, P(hist))
        self.kry.UCFDSolverDestroy(byref(sv))
        self.kry.UCFDPreconDestroy(byref(pc))
        self.kry.UCFDMatDestroy(byref(A))
        return x, st.value, it.value, res.value, hist

    def _precon(self, s, pc, v, icolors=None):
        """A reference preconditioner on arrays (v is modified in place by
        the ILU-type prepares, as in the reference)."""
        h = c_void_p()
        keep = [_i32(s["rowptr"]), _i32(s["colidx"]), _i32(s["diagslots"])]
        self.kry.UCFDPreconCreatefromArrays(byref(h), P(keep[0]), P(keep[1]), P(keep[2]), P(v))
        if pc == "blusgs":
            self.kry.UCFDPreconSetBLUSGS(byref(h), s["bn"], s["blk"])
        elif pc == "bilu":
            self.kry.UCFDPreconSetBILU(byref(h), s["bn"], s["blk"])
        elif pc == "pbilu":
            ic = _i32(icolors)
            keep.append(ic)
            self.kry.UCFDPreconSetPBILU(byref(h), s["bn"], s["blk"], len(ic) - 1, P(ic))
            # pbilu.c:20 shares one column map (iw) among the OpenMP threads of a
            # colour, so its result is only defined with a single thread
            gomp = ctypes.CDLL("libgomp.so.1")
            nt = gomp.omp_get_max_threads()
            gomp.omp_set_num_threads(1)
            try:
                self.kry.UCFDPreconPrepare(h)
            finally:
                gomp.omp_set_num_threads(nt)
            return h, keep
        elif pc == "ilu":
            self.kry.UCFDPreconSetILU(byref(h), s["bn"])
        else:
            raise ValueError(pc)
        self.kry.UCFDPreconPrepare(h)
        return h, keep

    def ilu_factor(self, s, pc="bilu", icolors=None):
        """The values array after the reference's ILU-type Prepare."""
        v = _f64(s["values"]).copy()
        h, keep = self._precon(s, pc, v, icolors)
        self.kry.UCFDPreconDestroy(byref(h))
        return v

    def bicgstab(self, s, b, maxiter=50, tol=1e-10, pc="blusgs", icolors=None):
        """BiCGSTAB of the reference with a preconditioner on a copy of the
        values (the matrix keeps the originals)."""
        A, sv = c_void_p(), c_void_p()
        rp, ci, v = _i32(s["rowptr"]), _i32(s["colidx"]), _f64(s["values"])
        self.kry.UCFDMatCreateBSR(byref(A), s["bn"], s["blk"], P(rp), P(ci), P(v))
        pv = v.copy()
        pc_h, keep = self._precon(s, pc, pv, icolors)
        n = s["bn"] * s["blk"]
        self.kry.UCFDSolverCreateBICGSTAB(byref(sv), n, maxiter, tol)
        self.kry.UCFDSolverTraceResidualHistory(sv)
        x = np.zeros(n)
        b = _f64(b)
        self.kry.UCFDSolve(sv, pc_h, A, P(x), P(b))
        st, it, res = c_int(), c_int(), c_double()
        self.kry.UCFDSolverGetResult(sv, byref(st), byref(it), byref(res))
        hist = np.zeros(maxiter)
        self.kry.UCFDSolverGetResidualHistory(sv, P(hist))
        self.kry.UCFDSolverDestroy(byref(sv))
        self.kry.UCFDPreconDestroy(byref(pc_h))
        self.kry.UCFDMatDestroy(byref(A))
        return x, st.value, it.value, res.value, hist


# ---------------------------------------------------------------------------
# the reference's own GPU BSR matvec (oracle/_ref/cusparsemat.cubin)
# ---------------------------------------------------------------------------
REF_CUBIN = os.path.join(REF, "cusparsemat.cubin")


def ref_cuda_available() -> bool:
    return os.path.exists(REF_CUBIN)


class RefCudaBSR:
    """_SpMV_CUDABSR<blk> of src/krylov/matrix/cusparsemat.cu:74-115,
    compiled from the reference source for sm_103a by oracle/Makefile, loaded
    with the CUDA driver API and launched as SpMV_CUDABSR does
    (cusparsemat.cu:118-139: (bn + TPB - 1) / TPB blocks of TPB = 128
    threads, config.h:62-64).  Arguments are device pointers (integers);
    the caller's CUDA context must be current (any torch CUDA call makes
    it so)."""

    TPB = 128

    def __init__(self, blk: int = 5):
        self.cu = ctypes.CDLL("libcuda.so.1")
        cu = self.cu
        for n in ("cuModuleLoad", "cuModuleGetFunction", "cuLaunchKernel", "cuCtxGetCurrent", "cuModuleUnload"):
            getattr(cu, n).restype = c_int
        ctx = c_void_p()
        self._check(cu.cuCtxGetCurrent(byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context (initialise CUDA first, e.g. with torch)")
        self.mod = c_void_p()
        self._check(cu.cuModuleLoad(byref(self.mod), REF_CUBIN.encode()), "cuModuleLoad")
        self.fn = c_void_p()
        # the entry name nvcc gives the template instance (printed by ptxas -v)
        name = f"_Z13_SpMV_CUDABSRILi{blk}EEvdiPKiS1_PKdS3_dPd".encode()
        self._check(cu.cuModuleGetFunction(byref(self.fn), self.mod, name), "cuModuleGetFunction")

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def spmv(self, alpha, bn, rowptr, colidx, values, x, beta, y, stream=0):
        """y = alpha A x + beta y (all pointers device addresses)."""
        a, b = c_double(alpha), c_double(beta)
        n = c_int(bn)
        ptrs = [c_void_p(rowptr), c_void_p(colidx), c_void_p(values), c_void_p(x)]
        yp = c_void_p(y)
        params = (c_void_p * 8)(ctypes.addressof(a), ctypes.addressof(n), *[ctypes.addressof(q) for q in ptrs],
                                ctypes.addressof(b), ctypes.addressof(yp))
        grid = (bn + self.TPB - 1) // self.TPB
        self._check(self.cu.cuLaunchKernel(self.fn, grid, 1, 1, self.TPB, 1, 1, 0, c_void_p(stream), params, None),
                    "cuLaunchKernel")

    def close(self):
        if self.mod:
            self.cu.cuModuleUnload(self.mod)
            self.mod = c_void_p()


# ---------------------------------------------------------------------------
# one BLU-SGS pseudo-time step, call by call
# ---------------------------------------------------------------------------
class BlusgsPhases:
    """One FlowSys BLU-SGS step split into its calls, as a CFD code makes
    them (blusgs.c:17-57 pack, 200-270 prepare, 431-440 reset, 273-373
    sweeps, 161-197 sub-residual, 126-155 update): ``pack_prepare()``,
    ``reset()``, then ``lower()`` / ``upper()`` / ``sub_residual()`` per
    sweep pair, then ``update()``.  ``upts`` is updated in a copy
    (``self.upts``); ``self.res`` holds the last sub-residual."""

    def close(self):
        pass


class _PortBlusgsPhases(BlusgsPhases):
    def __init__(self, port, fs, rhs, dt, jmat, vol, upts, a0):
        L = port.L
        self.L = L
        N, nv, nfv, nF = fs["nlocal"], fs["nvars"], fs["nfvars"], fs["nfaces"]
        self.N, self.nv, self.nfv, self.nF, self.a0 = N, nv, nfv, nF, a0
        self.neles = dt.shape[0]
        self.ids = _i32(fs["cell_ids"])
        self.rp, self.ci, self.sl = _i32(fs["rowptr"]), _i32(fs["colidx"]), _i32(fs["slots"])
        self.sd = np.ascontiguousarray(fs["sides"], dtype=np.int8)
        self.fa, self.rv = _f64(fs["face_area"]), _f64(fs["rcp_vol"])
        self.rhs, self.dt, self.jmat, self.vol = _f64(rhs), _f64(dt), _f64(jmat), _f64(vol)
        self.upts = _f64(upts).copy()
        self.rrhs = np.zeros(N * nv)
        self.diag = np.zeros(N * nfv * nfv)
        self.du = np.zeros(N * nv)
        self.dup = np.zeros(N * nv)
        self.res = np.zeros((nv, self.neles))

    def pack_prepare(self):
        L = self.L
        L.oracle_blusgs_pack(self.N, self.neles, self.nv, self.nfv, self.a0, P(self.ids), P(self.rhs), P(self.dt),
                             P(self.rrhs), P(self.diag))
        L.oracle_blusgs_prepare(self.N, self.nfv, self.nF, P(self.rp), P(self.sl), P(self.sd), P(self.fa),
                                P(self.rv), P(self.diag), P(self.jmat))

    def reset(self):
        self.du[:] = 0.0
        self.dup[:] = 0.0

    def _g(self):
        return (P(self.rp), P(self.ci), P(self.sd), P(self.sl), P(self.fa), P(self.rv), P(self.rrhs), P(self.diag),
                P(self.jmat), P(self.du))

    def lower(self):
        self.L.oracle_blusgs_lower(0, self.nfv, self.N, self.nv, self.nF, *self._g())

    def upper(self):
        self.L.oracle_blusgs_upper(0, self.nfv, self.N, self.nv, self.nF, *self._g())

    def sub_residual(self):
        self.L.oracle_blusgs_sub_residual(self.N, self.neles, self.nv, P(self.ids), P(self.vol), P(self.du),
                                          P(self.dup), P(self.res))

    def update(self):
        self.L.oracle_blusgs_update(self.N, self.neles, self.nv, P(self.ids), P(self.du), P(self.upts))


class _RefBlusgsPhases(BlusgsPhases):
    def __init__(self, ref, fs, rhs, dt, jmat, vol, upts, a0):
        self.lus = ref.lus
        self.h, self.keep = ref._sys(fs)
        self.a0 = a0
        self.upts = _f64(upts).copy()
        self.rhs, self.dt, self.jmat, self.vol = _f64(rhs), _f64(dt), _f64(jmat), _f64(vol)
        self.ids = _i32(fs["cell_ids"])
        self.res = np.zeros_like(self.upts)
        self.dsrc = np.zeros_like(self.upts)
        self.lus.UCFDFlowSysSetBLUSGS(byref(self.h), P(self.jmat), None)
        self.lus.UCFDFlowSysSetElement(byref(self.h), 0, self.dt.shape[0], 6, P(self.ids), P(self.upts),
                                       P(self.rhs), P(self.dt), P(self.dsrc), P(self.vol), P(self.res))

    def pack_prepare(self):
        self.lus.UCFDBLUSGS_Pack(self.h, 0, self.a0)
        self.lus.UCFDBLUSGS_NSPrepare(self.h)

    def reset(self):
        self.lus.UCFDBLUSGS_Reset(self.h)

    def lower(self):
        self.lus.UCFDBLUSGS_NSLowerSweep(self.h)

    def upper(self):
        self.lus.UCFDBLUSGS_NSUpperSweep(self.h)

    def sub_residual(self):
        self.lus.UCFDBLUSGS_SubResidual(self.h, 0)

    def update(self):
        self.lus.UCFDBLUSGS_Update(self.h, 0)

    def close(self):
        if self.h:
            self.lus.UCFDFlowSysDestroy(byref(self.h))
            self.h = c_void_p()


# ---------------------------------------------------------------------------
# colored array layout -> FlowSys layout (the colour-renumbered mesh)
# ---------------------------------------------------------------------------
def legacy_to_flowsys(c: dict, icolor, nfvars: int = 5, ndims: int = 3) -> dict:
    """FlowSys arrays equal to the colored array API on a colour-renumbered
    mesh: rank k = position of the cell in icolor, rowptr = nf*k, one CSR
    entry per cell face (self entries at the boundary), slots = f*N + cell,
    sides = +1, face_area = fnorm_vol, rcp_vol = 1, face_normal[d][f*N+i] =
    vec_fnorm[f][d][i].  With kappa = 1, a0 = 0, dsrc = 0 and the element
    cell_ids = new rank of each cell, the reference's natural-order FlowSys
    sweeps perform exactly the colored sweeps' arithmetic."""
    N, nf = c["neles"], c["nface"]
    icolor = np.asarray(icolor, dtype=np.int64)
    newid = np.empty(N, dtype=np.int64)
    newid[icolor] = np.arange(N)
    nei = np.asarray(c["nei_ele"], dtype=np.int64)
    rowptr = (np.arange(N + 1) * nf).astype(np.int32)
    colidx = newid[nei[:, icolor]].T.reshape(-1).astype(np.int32)          # [k][f]
    slots = (np.arange(nf)[None, :] * N + icolor[:, None]).reshape(-1).astype(np.int32)
    sides = np.ones(N * nf, dtype=np.int8)
    face_area = np.ascontiguousarray(np.asarray(c["fnorm_vol"]).reshape(-1))
    vec = np.asarray(c["vec_fnorm"])                                        # [f][d][i]
    face_normal = np.ascontiguousarray(vec.transpose(1, 0, 2).reshape(ndims, nf * N))
    return dict(nlocal=N, nvars=c["nvars"], nfvars=nfvars, ndims=ndims, nfaces=nf * N, rowptr=rowptr,
                colidx=colidx, slots=slots, sides=sides, face_area=face_area, face_normal=face_normal,
                rcp_vol=np.ones(N), cell_ids=newid.astype(np.int32),
                fspr=np.ascontiguousarray(np.asarray(c["fspr"]).reshape(-1)))
