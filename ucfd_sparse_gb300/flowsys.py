"""Python mirror of the FlowSys API (``src/lusgs/include/ucfdlusgs.h``).

Method names follow the reference C functions with the ``UCFDFlowSys`` /
``UCFDLUSGS_`` / ``UCFDBLUSGS_`` prefixes dropped; arguments keep their
meaning and order.  Arrays are numpy arrays or torch tensors (host or CUDA)
and are kept alive by the object, since the library keeps their pointers
as the reference does.
"""
from __future__ import annotations

from ctypes import byref, c_double, c_int, c_void_p

from .lib import PREC_FP32, PREC_FP64, PREC_FP64_FMA, LaunchConfig, call, load, ptr

__all__ = ["FlowSys", "PREC_FP64", "PREC_FP64_FMA", "PREC_FP32"]


class FlowSys:
    def __init__(self, nlocal, nvars, nfvars, ndims, nfaces, nelem, rowptr, colidx, slots, sides, face_area,
                 face_normal, rcp_vol):
        load()
        self._h = c_void_p()
        self._keep = [rowptr, colidx, slots, sides, face_area, face_normal, rcp_vol]
        call("UCFDFlowSysCreate", byref(self._h), nlocal, nvars, nfvars, ndims, nfaces, nelem, ptr(rowptr),
             ptr(colidx), ptr(slots), ptr(sides), ptr(face_area), ptr(face_normal), ptr(rcp_vol))
        self.nlocal, self.nvars, self.nfvars, self.ndims = nlocal, nvars, nfvars, ndims
        self.nfaces = nfaces
        self.precision = PREC_FP64
        self.kind = None

    @classmethod
    def from_dict(cls, fs: dict, nelem: int = 1):
        return cls(fs["nlocal"], fs["nvars"], fs.get("nfvars", 5), 3, fs["nfaces"], nelem, fs["rowptr"],
                   fs["colidx"], fs["slots"], fs["sides"], fs["face_area"], fs["face_normal"], fs["rcp_vol"])

    # ---- common ----------------------------------------------------------
    def set_element(self, eidx, neles, nface, cell_ids, uptsb, rhs, dt, dsrc, vol, resid_out):
        self._keep += [cell_ids, uptsb, rhs, dt, dsrc, vol, resid_out]
        call("UCFDFlowSysSetElement", byref(self._h), eidx, neles, nface, ptr(cell_ids), ptr(uptsb), ptr(rhs),
             ptr(dt), ptr(dsrc), ptr(vol), ptr(resid_out))

    def destroy(self):
        if self._h:
            call("UCFDFlowSysDestroy", byref(self._h))
            self._h = c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    # ---- extensions --------------------------------------------------------
    def set_coloring(self, color):
        self._keep.append(color)
        call("UCFDFlowSysSetColoring", self._h, ptr(color))

    def color_greedy(self) -> int:
        n = c_int()
        call("UCFDFlowSysColorGreedy", self._h, byref(n))
        return n.value

    def levels(self) -> int:
        n = c_int()
        call("UCFDFlowSysGetLevels", self._h, byref(n))
        return n.value

    def set_precision(self, prec: int):
        call("UCFDFlowSysSetPrecision", self._h, prec)
        self.precision = prec

    def set_launch(self, threads: int):
        call("UCFDFlowSysSetLaunch", self._h, threads)

    def launch_config(self) -> dict:
        cfg = LaunchConfig()
        call("UCFDFlowSysGetLaunchConfig", self._h, byref(cfg))
        return cfg.as_dict()

    def set_launch_config(self, threads_per_block=0, sweep_variant=0, run_mode=0, **_ignored):
        cfg = LaunchConfig(threads_per_block, sweep_variant, run_mode, 0.0)
        call("UCFDFlowSysSetLaunchConfig", self._h, byref(cfg))

    def autotune(self, reps: int = 5, cache: str | bool | None = None) -> dict:
        """Times the launch candidates (``UCFDFlowSysAutotune``) and keeps the
        fastest.  With ``cache`` (a path, or True for the default file) the
        choice is looked up in / stored to the JSON cache of ``autotune.py``."""
        from . import autotune as _at
        return _at.tune(self, reps=reps, cache=cache)

    def set_stream(self, stream_ptr: int | None, asynchronous: bool = False):
        call("UCFDFlowSysSetStream", self._h, stream_ptr, 1 if asynchronous else 0)

    # ---- scalar LU-SGS -------------------------------------------------------
    def set_lusgs(self, fspr, tfspr=None):
        self.kind = "lusgs"
        self._keep += [fspr, tfspr]
        call("UCFDFlowSysSetLUSGS", byref(self._h), ptr(fspr), ptr(tfspr))

    def lusgs_pack(self, eidx=0, turb_factor=1.0, a0=0.0):
        call("UCFDLUSGS_Pack", self._h, eidx, turb_factor, a0)

    def lusgs_update(self, eidx=0):
        call("UCFDLUSGS_Update", self._h, eidx)

    def lusgs_ns_prepare(self, kappa=1.0):
        call("UCFDLUSGS_NSPrepare", self._h, kappa)

    def lusgs_rans_prepare(self, kappa=1.0):
        call("UCFDLUSGS_RANSPrepare", self._h, kappa)

    def lusgs_ns_lower(self, kappa=1.0):
        call("UCFDLUSGS_NSLowerSweep", self._h, kappa)

    def lusgs_ns_upper(self, kappa=1.0):
        call("UCFDLUSGS_NSUpperSweep", self._h, kappa)

    def lusgs_rans_lower(self, kappa=1.0):
        call("UCFDLUSGS_RANSLowerSweep", self._h, kappa)

    def lusgs_rans_upper(self, kappa=1.0):
        call("UCFDLUSGS_RANSUpperSweep", self._h, kappa)

    # both systems per call: the values of the NS call followed by the RANS call
    def lusgs_nsrans_prepare(self, kappa=1.0):
        call("UCFDLUSGS_NSRANSPrepare", self._h, kappa)

    def lusgs_nsrans_lower(self, kappa=1.0):
        call("UCFDLUSGS_NSRANSLowerSweep", self._h, kappa)

    def lusgs_nsrans_upper(self, kappa=1.0):
        call("UCFDLUSGS_NSRANSUpperSweep", self._h, kappa)

    def lusgs_run(self, niter, kappa=1.0, rans=False, mode=0, resid=None):
        call("UCFDLUSGS_Run", self._h, niter, kappa, 1 if rans else 0, mode, ptr(resid))

    # ---- block LU-SGS -------------------------------------------------------
    def set_blusgs(self, jmat, tjmat=None):
        self.kind = "blusgs"
        self._keep += [jmat, tjmat]
        call("UCFDFlowSysSetBLUSGS", byref(self._h), ptr(jmat), ptr(tjmat))

    def blusgs_pack(self, eidx=0, a0=0.0):
        call("UCFDBLUSGS_Pack", self._h, eidx, a0)

    def blusgs_kwsst_pack(self, eidx=0, turb_factor=1.0, a0=0.0):
        call("UCFDBLUSGS_KWSST_Pack", self._h, eidx, turb_factor, a0)

    def blusgs_sa_pack(self, eidx=0, turb_factor=1.0, a0=0.0):
        call("UCFDBLUSGS_SA_Pack", self._h, eidx, turb_factor, a0)

    def blusgs_update(self, eidx=0):
        call("UCFDBLUSGS_Update", self._h, eidx)

    def blusgs_sub_residual(self, eidx=0):
        call("UCFDBLUSGS_SubResidual", self._h, eidx)

    def blusgs_ns_prepare(self):
        call("UCFDBLUSGS_NSPrepare", self._h)

    def blusgs_rans_prepare(self):
        call("UCFDBLUSGS_RANSPrepare", self._h)

    def blusgs_ns_lower(self):
        call("UCFDBLUSGS_NSLowerSweep", self._h)

    def blusgs_ns_upper(self):
        call("UCFDBLUSGS_NSUpperSweep", self._h)

    def blusgs_rans_lower(self):
        call("UCFDBLUSGS_RANSLowerSweep", self._h)

    def blusgs_rans_upper(self):
        call("UCFDBLUSGS_RANSUpperSweep", self._h)

    def blusgs_reset(self):
        call("UCFDBLUSGS_Reset", self._h)

    def blusgs_solve(self, rtol=1e-10, max_sweeps=500, inner_sweeps=10):
        n, r = c_int(), c_double()
        call("UCFDBLUSGS_Solve", self._h, rtol, max_sweeps, inner_sweeps, byref(n), byref(r))
        return n.value, r.value

    def blusgs_residual(self) -> float:
        r = c_double()
        call("UCFDBLUSGS_Residual", self._h, byref(r))
        return r.value
