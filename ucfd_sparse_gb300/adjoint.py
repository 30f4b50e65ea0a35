"""Differentiable colored LU-SGS step (torch.autograd.Function).

``lusgs_step(rhs, dt, fspr, mesh, upts)`` returns dQ of one colored LU-SGS
step -- pre, lower sweep colour by colour, upper sweep in reverse colour
order (the array API of the reference, README.md:37-50) -- and its backward
runs the hand-written transposed sweeps of ``UCFDColoredStepAdjoint``
(upper sweep transposed, then lower sweep transposed, then the diagonal),
giving gradients with respect to rhs, dt and fspr.  Geometry and the
current state upts are treated as constants.  float64 tensors use the
bit-exact FP64 kernels, float32 tensors the FP32 ones.
"""
from __future__ import annotations

import numpy as np
import torch

from .lib import PREC_FP32, PREC_FP64, call, load, ptr

__all__ = ["ColoredMesh", "ColoredLUSGSStep", "lusgs_step"]


class ColoredMesh:
    """Connectivity, geometry and colouring of the array layout, on the GPU.

    nei_ele/fnorm_vol [nface, neles], vec_fnorm [nface, ndims, neles];
    icolor lists the cells colour by colour, ranges the exclusive end of
    each colour."""

    def __init__(self, nei_ele, fnorm_vol, vec_fnorm, icolor, ranges, nvars=5, nfvars=5, ndims=3,
                 device="cuda", dtype=torch.float64):
        load()
        nei = np.ascontiguousarray(nei_ele, dtype=np.int32)
        self.nface, self.neles = nei.shape
        rface = np.empty_like(nei)
        call("UCFDReverseFaces", self.neles, self.nface, ptr(nei), ptr(rface))
        icolor = np.ascontiguousarray(icolor, dtype=np.int32)
        lcolor = np.empty(self.neles, dtype=np.int32)
        start = 0
        for c, end in enumerate(ranges):
            lcolor[icolor[start:end]] = c + 1
            start = end
        i32 = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)
        self.nei = i32(nei)
        self.rface = i32(rface)
        self.icolor = i32(icolor)
        self.lcolor = i32(lcolor)
        self.ranges = np.ascontiguousarray(ranges, dtype=np.int32)
        self.nvars, self.nfvars, self.ndims = nvars, nfvars, ndims
        self.device = device
        self._geo = {}
        self._fnv = np.ascontiguousarray(fnorm_vol, dtype=np.float64)
        self._vec = np.ascontiguousarray(vec_fnorm, dtype=np.float64)

    def geometry(self, dtype):
        if dtype not in self._geo:
            self._geo[dtype] = (torch.from_numpy(self._fnv).to(self.device, dtype),
                                torch.from_numpy(self._vec).to(self.device, dtype))
        return self._geo[dtype]


def _prec(dtype, fma=False):
    if dtype == torch.float32:
        return PREC_FP32
    if dtype == torch.float64:
        return 1 if fma else PREC_FP64
    raise TypeError(f"unsupported dtype {dtype}")


class ColoredLUSGSStep(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rhs, dt, fspr, mesh: ColoredMesh, upts):
        dtype = rhs.dtype
        N, nf = mesh.neles, mesh.nface
        fnv, vec = mesh.geometry(dtype)
        rhs, dt, fspr, upts = (t.contiguous() for t in (rhs, dt, fspr, upts))
        diag = torch.empty(N, dtype=dtype, device=rhs.device)
        dub = torch.zeros_like(rhs)
        dq = torch.zeros_like(rhs)
        stream = torch.cuda.current_stream(rhs.device).cuda_stream
        call("UCFDColoredStep", _prec(dtype), N, nf, mesh.nvars, mesh.nfvars, mesh.ndims, ptr(mesh.nei),
             ptr(mesh.icolor), len(mesh.ranges), ptr(mesh.ranges), ptr(mesh.lcolor), 1.0, ptr(fnv), ptr(vec),
             ptr(fspr), ptr(dt), ptr(upts), ptr(rhs), ptr(diag), ptr(dub), ptr(dq), stream)
        ctx.mesh = mesh
        ctx.save_for_backward(dt, fspr, upts, diag, dub, dq)
        return dq

    @staticmethod
    def backward(ctx, gdq):
        mesh = ctx.mesh
        dt, fspr, upts, diag, dub, dq = ctx.saved_tensors
        dtype = dq.dtype
        N, nf = mesh.neles, mesh.nface
        fnv, vec = mesh.geometry(dtype)
        gdq = gdq.contiguous()
        grhs = torch.empty_like(dq)
        gdt = torch.empty_like(dt)
        gfspr = torch.empty_like(fspr)
        work = torch.empty((2 * mesh.nfvars + 1) * N, dtype=dtype, device=dq.device)
        stream = torch.cuda.current_stream(dq.device).cuda_stream
        call("UCFDColoredStepAdjoint", _prec(dtype), N, nf, mesh.nvars, mesh.nfvars, mesh.ndims, ptr(mesh.nei),
             ptr(mesh.rface), ptr(mesh.icolor), len(mesh.ranges), ptr(mesh.ranges), ptr(mesh.lcolor), 1.0,
             ptr(fnv), ptr(vec), ptr(fspr), ptr(dt), ptr(upts), ptr(diag), ptr(dub), ptr(dq), ptr(gdq),
             ptr(grhs), ptr(gdt), ptr(gfspr), ptr(work), stream)
        return grhs, gdt, gfspr, None, None


def lusgs_step(rhs, dt, fspr, mesh: ColoredMesh, upts):
    """dQ of one colored LU-SGS step, differentiable in rhs, dt and fspr."""
    return ColoredLUSGSStep.apply(rhs, dt, fspr, mesh, upts)
