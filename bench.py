#!/usr/bin/env python
"""Benchmark of the block LU-SGS hot path on one GB300.

Workload (the 2.1M-cell hex configuration): 128^3 hexahedra on the unit
cube, interior nodes jittered by +-0.2h, cell numbering randomly permuted
(seed 0), greedy first-fit colouring, 5x5 face Jacobians A+ = sigma I + E,
A- = -sigma I + E (E ~ N(0, 0.05^2), sigma ~ U[0.5, 2]), FP64 diagonal-block
LU.  One step = one pseudo-time step of the FlowSys BLU-SGS API: Pack, NS
Prepare (FP64 LU), Reset, solve of the block system to a 1e-10 relative
residual, Update.  The solve runs FP32 sweeps inside FP64 iterative
refinement; the same step with plain FP64 sweeps is timed for comparison.

Metric: cell-updates/s, one cell-update = one cell visited by one symmetric
(lower + upper) sweep pair; value = cells * pairs / step time, summed over
ranks (replicas) for --gpus N.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LU-SGS cell-updates/s & HBM GB/s @2.1M cells; FP32+refine vs FP64 @1e-10"
UNIT = "cell-updates/s"
# DRAM bytes per cell update of the unrolled FP32 block sweep: ncu
# dram__bytes_read.sum + dram__bytes_write.sum over one lower + upper sweep
# pair on the 96^3 mesh (718.1 MB for 2 x 884,736 cell updates;
# profiles/fs_blusgs_sweep_96cubed.md)
SWEEP_TRAFFIC_PER_CELL = 405.8


# ---------------------------------------------------------------------------
# multi-rank plumbing (replicas: no data-path collective)
# ---------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(backend):
    import torch.distributed as dist
    ws, rank, _ = dist_env()
    if ws > 1 and not dist.is_initialized():
        dist.init_process_group(backend=backend)
    return dist if ws > 1 else None


def reduce_max(x: float, dist, device=None) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(x: float, dist, device=None) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(dist, device=None):
    if dist is not None:
        if device is not None and device.type == "cuda":
            dist.barrier(device_ids=[device.index])
        else:
            dist.barrier()


def repo_libraries_loaded():
    """Shared libraries of this repository mapped into the process (from
    /proc/self/maps): shows which native code an arm ran."""
    libs = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = line.split()[-1] if len(line.split()) >= 6 else ""
                if path.startswith(ROOT) and path.endswith(".so"):
                    libs.add(os.path.relpath(path, ROOT))
    except OSError:
        return None
    return sorted(libs)


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"ucfd_clocks_{os.getpid()}.csv")
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def make_case(m: int, seed: int = 0):
    from ucfd_sparse_gb300 import meshgen as mg
    return mg.blusgs_case(m, seed=seed)


def sweep_bytes(rowptr: np.ndarray, elt: int, B: int = 5) -> int:
    """Algorithmic bytes of one BLU-SGS sweep over all cells (the mean of a
    lower and an upper sweep) as the FP32 / FMA-mode kernels run it: per
    cell-face its neighbour index (4) in every sweep and its block (B*B*elt:
    M = D^-1 J fv, formed at Prepare) in the one sweep of the pair that
    updates that neighbour's side; per cell its right-hand side (D^-1 rhs),
    du read (as the neighbours' data, once) and written, and the stored
    other side's sums read and its own written."""
    nnz = int(rowptr[-1])
    N = rowptr.shape[0] - 1
    return nnz * 4 + (nnz * B * B * elt) // 2 + N * (5 * B * elt)


class Problem:
    """FlowSys objects on device-resident inputs (torch CUDA tensors)."""

    def __init__(self, case, colour, prec, stream, device, host_inputs=False):
        import torch

        from ucfd_sparse_gb300.flowsys import FlowSys
        self.case = case
        if host_inputs:
            conv = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        else:
            conv = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)
        m = {k: conv(case[k]) for k in ("rowptr", "colidx", "slots", "sides", "face_area", "face_normal",
                                         "rcp_vol")}
        self.S = FlowSys(case["nlocal"], 5, 5, 3, case["nfaces"], 1, m["rowptr"], m["colidx"], m["slots"],
                         m["sides"], m["face_area"], m["face_normal"], m["rcp_vol"])
        self.S.set_coloring(colour)
        self.S.set_precision(prec)
        if stream is not None and not host_inputs:
            self.S.set_stream(stream.cuda_stream, True)
        self.e = {k: conv(case[k]) for k in ("rhs", "dt", "cell_ids", "vol", "jmat")}
        self.e["upts"] = conv(np.array(case["upts"]))
        self.e["dsrc"] = conv(np.zeros_like(case["rhs"]))
        self.e["res"] = conv(np.zeros_like(case["rhs"]))
        e = self.e
        self.S.set_element(0, case["neles"], 6, e["cell_ids"], e["upts"], e["rhs"], e["dt"], e["dsrc"], e["vol"],
                           e["res"])
        self.S.set_blusgs(e["jmat"])
        self.nlev = self.S.levels()

    def tune(self, reps=3, cache=None):
        """Launch autotuner on the packed system (outside any timed region)."""
        S = self.S
        S.blusgs_pack(0, 0.0)
        S.blusgs_ns_prepare()
        cfg = S.autotune(reps=reps, cache=cache)
        cfg.pop("source", None)
        return cfg

    def step(self, rtol, max_pairs, inner, calls=None, copies=None):
        """One pseudo-time step; with `calls` (a dict) the host wall time of
        each C-ABI call is added to it (the calls on host inputs are
        synchronous, so this is each call's whole cost); with `copies` (a
        dict, transfer timing on) each call's timed host<->device copy
        milliseconds."""
        from ucfd_sparse_gb300 import lib as _lib
        S = self.S
        steps = (("pack", lambda: S.blusgs_pack(0, 0.0)), ("prepare", S.blusgs_ns_prepare),
                 ("reset", S.blusgs_reset), ("solve", lambda: S.blusgs_solve(rtol, max_pairs, inner)),
                 ("update", lambda: S.blusgs_update(0)))
        out = None
        for name, f in steps:
            x0 = _lib.transfer_stats() if copies is not None else None
            t = time.perf_counter()
            r = f()
            if calls is not None:
                calls[name] = calls.get(name, 0.0) + time.perf_counter() - t
            if copies is not None:
                x1 = _lib.transfer_stats()
                c = copies.setdefault(name, {"h2d_ms": 0.0, "h2d_bytes": 0.0, "d2h_ms": 0.0, "d2h_bytes": 0.0})
                for k in c:
                    c[k] += x1[k] - x0[k]
            if name == "solve":
                out = r
        return out

    def h2d_bytes(self):
        c = self.case
        return sum(np.asarray(c[k]).nbytes for k in ("rhs", "dt", "cell_ids", "jmat", "upts"))

    def d2h_bytes(self):
        return np.asarray(self.case["upts"]).nbytes


def launches_per_step(nlev, pairs, inner, mixed):
    outer = math.ceil(pairs / inner) if pairs else 0
    n = 1 + 2 + 1                                  # pack, prepare (jmat transpose + diagonal/LU), update
    n += 2                                         # initial residual + reduction
    n += outer * 2 + pairs * 2 * nlev              # residual per outer loop, sweeps
    if mixed:
        n += 2 + 2 * outer                         # conversions; per outer step x += delta and D^-1 r
    return n


# ---------------------------------------------------------------------------
# CPU baseline (the oracle: the reference's CPU path restated, or the
# reference itself where it was compiled on this machine)
# ---------------------------------------------------------------------------
def headline_config(args, N, ncolors, ws):
    """The workload of the headline line (both arms)."""
    return {"workload": f"BLU-SGS 5x5 face Jacobians, {args.mesh}^3 jittered (+-0.2h) randomly permuted "
                        f"hex ({N} cells), greedy colouring in {args.coloring} order ({ncolors} colours), "
                        f"solve to rtol {args.rtol:g} per pseudo-time step", "cells": N, "colors": ncolors,
            "coloring": args.coloring, "inner_sweeps": args.inner, "fp64_check_every": args.check,
            "l2": "inputs larger than L2 (no flush needed)", "parallelism": f"replicas x{ws}"}


# Sweep pairs the headline solve needs per pseudo-time step on this workload:
# the FP32-sweep + FP64-refinement solve and the plain FP64 solve both reach
# the 1e-10 relative residual at 40 pairs (the GPU arm reports its own count
# as pairs_per_step).  The CPU legs compose a step of this many pairs.
PAIRS_PER_STEP = 40


def cpu_impl():
    """The reference's CPU code for the BLU-SGS step: the reference library
    compiled from its own sources (oracle/_ref, -O3 -ffast-math as its
    Makefile.inc) where it was built on this machine, else the oracle's
    restatement built with the same flags."""
    from oracle import oracle as orc
    if orc.ref_available():
        return orc.Ref(fast=True), "reference"
    return orc.Port(fast=True), "port"


def colour_renumbered(case):
    """The mesh renumbered colour by colour (greedy first-fit in index
    order, computed by the oracle so that no product library is loaded).  A
    natural-order sweep of the result is the coloured sweep the GPU runs."""
    from oracle import oracle as orc
    from ucfd_sparse_gb300 import meshgen as mg
    ic, rg, _ = orc.Port(fast=True).greedy_coloring_csr(case["rowptr"], case["colidx"])
    new = np.empty(case["nlocal"], dtype=np.int64)
    new[ic] = np.arange(case["nlocal"])
    return mg.renumber_flowsys(case, new), rg


def compose_cpu_step(t_prepare, t_update, t_lower, t_upper_sub, pairs=PAIRS_PER_STEP):
    """Seconds of one pseudo-time step of `pairs` sweep pairs from the timed
    pieces: Pack + NSPrepare + Reset, Update, and per pair a lower sweep and
    an upper sweep + SubResidual (blusgs.c's call sequence)."""
    return t_prepare + t_update + pairs * (t_lower + t_upper_sub)


def cpu_baseline(case, br=None):
    """A bounded sample of the reference's CPU path on the full mesh (about
    25 s on 16 Arm cores): Pack + NSPrepare + Reset, one lower sweep, one
    upper sweep + SubResidual, Update, each timed, composed into a step of
    PAIRS_PER_STEP pairs.  The reference FlowSys is serial (src/lusgs has
    no OpenMP), so one core does the work."""
    if br is None:
        br, _ = colour_renumbered(case)
    impl, kind = cpu_impl()
    ph = impl.blusgs_phases(br, case["rhs"], case["dt"], case["jmat"], case["vol"], case["upts"])
    tic = time.perf_counter
    t0 = tic(); ph.pack_prepare(); ph.reset(); t_prep = tic() - t0
    t0 = tic(); ph.lower(); t_low = tic() - t0
    t0 = tic(); ph.upper(); ph.sub_residual(); t_up = tic() - t0
    t0 = tic(); ph.update(); t_upd = tic() - t0
    ph.close()
    step = compose_cpu_step(t_prep, t_upd, t_low, t_up)
    N = case["nlocal"]
    return {"value": N * PAIRS_PER_STEP / step, "unit": UNIT, "cores": 1, "kind": kind,
            "sample": f"FP64 on all {N} cells of the colour-renumbered mesh: Pack+NSPrepare+Reset, one lower "
                      f"sweep, one upper sweep+SubResidual and Update timed once each and composed into a step "
                      f"of {PAIRS_PER_STEP} pairs, the GPU arm's unit; serial, as the reference FlowSys",
            "seconds": {"prepare": t_prep, "lower": t_low, "upper_subresidual": t_up, "update": t_upd,
                        "composed_step": step}}


def lusgs_cpu_baseline(c, iters=1):
    """One bounded sample of the reference's scalar LU-SGS CPU path on the
    same mesh: `iters` pseudo-time iterations of Pack, NS + RANS Prepare,
    lower and upper sweeps (natural order, as lusgs.c) and Update.  The
    reference FlowSys is serial (src/lusgs has no OpenMP): one core."""
    impl, kind = cpu_impl()
    dsrc = np.zeros_like(c["rhs"])
    t0 = time.perf_counter()
    impl.flowsys_lusgs_step(c, c["upts"], c["rhs"], c["dt"], dsrc, c["fspr"], c["tfspr"], rans=True, nsteps=iters)
    sec = time.perf_counter() - t0
    N = c["nlocal"]
    return {"value": N * iters / sec, "unit": UNIT, "cores": 1, "kind": kind, "seconds": sec,
            "sample": f"{iters} iteration(s) of Pack+NS/RANS Prepare+lower/upper sweeps+Update on all {N} cells, "
                      f"FP64; serial natural-order sweeps as in lusgs.c"}


def krylov_cpu_baseline(s, icolors, tol):
    """The reference's CPU GMRES(30) and BiCGSTAB with the coloured BLU-SGS
    preconditioner (OpenMP SpMV / preconditioner as in the reference) on a
    BSR system, to the absolute tolerance tol: seconds and iterations."""
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    port = orc.Port(fast=True)
    out = {"kind": "port", "cores": threads}
    t0 = time.perf_counter()
    _, st, it, res, _ = port.gmres(s, s["rhs"], m=30, maxiter=100, tol=tol, pc="pblusgs", icolors=icolors)
    out["gmres"] = {"s": time.perf_counter() - t0, "stat": st, "restarts": it, "resid": res}
    t0 = time.perf_counter()
    _, st, it, res, _ = port.bicgstab(s, s["rhs"], maxiter=200, tol=tol, pc="pblusgs", icolors=icolors)
    out["bicgstab"] = {"s": time.perf_counter() - t0, "stat": st, "iters": it, "resid": res}
    return out


def run_reference(args):
    """The reference's own CPU path (cpu_impl) on the headline workload.

    The unit is the GPU arm's: a pseudo-time step of PAIRS_PER_STEP sweep
    pairs, cell-updates/s = cells x pairs / step time.  A whole step takes
    about ten minutes on the host cores, so each timed step is a bounded
    sample of it: one sweep over all cells, lower sweeps on even steps and
    upper sweep + SubResidual on odd ones (the serial sweep of the colour-
    renumbered mesh, as the reference runs it).  Pack + NSPrepare + Reset are
    timed before the warm-up sweeps and Update after the timed ones; the step
    time is composed from those and the medians of the sampled sweeps."""
    ws, rank, _ = dist_env()
    dist = dist_init("gloo")
    if rank != 0:
        barrier(dist)
        return
    if args.coloring != "index":
        print(json.dumps({"impl": "reference", "unavailable": "the CPU legs colour in index order only "
                                                              "(--coloring index)"}))
        barrier(dist)
        return
    case = make_case(args.mesh)
    N = case["nlocal"]
    br, rg = colour_renumbered(case)
    impl, kind = cpu_impl()
    ph = impl.blusgs_phases(br, case["rhs"], case["dt"], case["jmat"], case["vol"], case["upts"])
    tic = time.perf_counter
    t0 = tic()
    ph.pack_prepare()
    ph.reset()
    t_prep = tic() - t0
    for w in range(args.warmup):
        (ph.lower if w % 2 == 0 else ph.upper)()
    lows, ups, samples = [], [], []
    for k in range(args.steps):
        t0 = tic()
        if k % 2 == 0:
            ph.lower()
        else:
            ph.upper()
            ph.sub_residual()
        dt_ = tic() - t0
        samples.append(dt_)
        (lows if k % 2 == 0 else ups).append(dt_)
    if not ups:                       # --steps 1: one upper sweep + SubResidual, untimed as a step
        t0 = tic()
        ph.upper()
        ph.sub_residual()
        ups.append(tic() - t0)
    t0 = tic()
    ph.update()
    t_upd = tic() - t0
    ph.close()
    t_low, t_up = statistics.median(lows), statistics.median(ups)
    step = compose_cpu_step(t_prep, t_upd, t_low, t_up)
    val = N * PAIRS_PER_STEP / step
    sample = (f"FP64 on all {N} cells of the colour-renumbered mesh, serial as the reference FlowSys (src/lusgs has "
              f"no OpenMP); each timed step one sweep (lower on even steps, upper + SubResidual on odd); step of "
              f"{PAIRS_PER_STEP} pairs composed as Pack+NSPrepare+Reset ({t_prep:.2f} s) + Update ({t_upd:.3f} s) "
              f"+ {PAIRS_PER_STEP} x (median lower {t_low:.2f} s of {len(lows)} + median upper+SubResidual "
              f"{t_up:.2f} s of {len(ups)}) = {step:.1f} s")
    out = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(samples) * 1e3,
           "ms_per_step_is": "mean duration of a timed sample (one sweep); the composed step is composed_step_s",
           "composed_step_s": step, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": headline_config(args, N, len(rg), ws),
           "cpu_baseline": {"value": val, "unit": UNIT, "cores": 1, "kind": kind, "sample": sample},
           "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "libraries_loaded": repo_libraries_loaded()}
    print(json.dumps(out))
    barrier(dist)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gpu(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    dist = dist_init("nccl")
    from ucfd_sparse_gb300 import _build, lib
    _build.build()
    lib.load()
    from ucfd_sparse_gb300 import coloredlusgs as cl

    case = make_case(args.mesh, seed=args.seed + rank)
    N = case["nlocal"]
    ic, rg, lc = cl.greedy_coloring_csr(case["rowptr"], case["colidx"], order=args.coloring)
    stream = torch.cuda.Stream(device=device)
    P32 = Problem(case, lc, 2, stream, device)
    P64 = Problem(case, lc, 1, stream, device)
    nlev = P32.nlev
    tuned = {}
    if not args.no_autotune:
        tuned = {"fp32": P32.tune(cache=args.autotune_cache), "fp64_fma": P64.tune(cache=args.autotune_cache)}

    def timed(P, steps, warm, inner, tag):
        for _ in range(warm):
            P.step(args.rtol, args.max_pairs, inner)
        torch.cuda.synchronize()
        barrier(dist, device)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        pairs_all, rels = [], []
        torch.cuda.nvtx.range_push(tag)  # a profiler can select the timed launches by this range
        ev0.record(stream)
        for _ in range(steps):
            p, r = P.step(args.rtol, args.max_pairs, inner)
            pairs_all.append(p)
            rels.append(r)
        ev1.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        barrier(dist, device)
        ms = ev0.elapsed_time(ev1) / steps
        return reduce_max(ms, dist, device), pairs_all, rels

    with ClockSampler(local) as clk:
        ms32, pairs32, rel32 = timed(P32, args.steps, args.warmup, args.inner, "timed_fp32")
    clocks = clk.summary()
    ms64, pairs64, rel64 = timed(P64, max(2, args.steps // 2), max(args.warmup, 3), args.check, "timed_fp64")
    pairs_mean = statistics.mean(pairs32)
    value_rank = N * pairs_mean / (ms32 * 1e-3)
    value = reduce_sum(value_rank, dist, device) if dist else value_rank

    # ---- dominant kernel: the FP32 sweep (roofline) -------------------------
    P32.S.blusgs_pack(0, 0.0)
    P32.S.blusgs_ns_prepare()
    P32.S.blusgs_reset()
    torch.cuda.synchronize()
    nk = 20
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(nk):
        P32.S.blusgs_ns_lower()
        P32.S.blusgs_ns_upper()
    ev1.record(stream)
    torch.cuda.synchronize()
    sweep_ms = ev0.elapsed_time(ev1) / (2 * nk)
    # the FP64 (fused multiply-add) sweep the same way
    P64.S.blusgs_pack(0, 0.0)
    P64.S.blusgs_ns_prepare()
    P64.S.blusgs_reset()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(nk):
        P64.S.blusgs_ns_lower()
        P64.S.blusgs_ns_upper()
    ev1.record(stream)
    torch.cuda.synchronize()
    sweep64_ms = ev0.elapsed_time(ev1) / (2 * nk)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    bytes_sweep64 = sweep_bytes(case["rowptr"], 8, 5)
    bytes_sweep = sweep_bytes(case["rowptr"], 4, 5)
    achieved = bytes_sweep / (sweep_ms * 1e-3) / 1e9
    launch_bytes = bytes_sweep / nlev
    cfg32 = P32.S.launch_config()
    kname = {0: "fs_blusgs_sweep_kernel<float,5,6>", 1: "fs_blusgs_sweep_kernel<float,5,0>",
             2: "fs_blusgs_sweep_bulk_kernel<5,6,2>", 3: "fs_blusgs_sweep_bulk_kernel<5,6,1>",
             4: "fs_blusgs_sweep_kernel<float,5,6,true>"}.get(cfg32["sweep_variant"], "fs_blusgs_sweep_kernel")
    # DRAM bytes per cell update from ncu (dram__bytes_read.sum + write) of
    # the unrolled FP32 sweep on the 64^3 case, scaled to this launch's cells
    traffic = (SWEEP_TRAFFIC_PER_CELL * N / nlev if SWEEP_TRAFFIC_PER_CELL and cfg32["sweep_variant"] in (0, 4)
               else None)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": kname, "threads_per_block": cfg32["threads_per_block"],
                "algorithmic_bytes_per_launch": launch_bytes, "launch_ms": sweep_ms / nlev,
                "traffic_source": f"ncu 96^3 capture of a sweep pair, {SWEEP_TRAFFIC_PER_CELL} B per cell update, "
                                  "scaled by cells per launch",
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6.8 TB/s",
                "pair_ms": 2 * sweep_ms,
                "algorithmic_bytes_per_cell_update": bytes_sweep / N,
                "bytes_note": "split-sum sweeps: every neighbour index each sweep, each face block once per "
                              "lower+upper pair (in the sweep that updates its side), 5 vectors per cell"}

    # ---- error of one step against the FP64 arithmetic of the oracle --------
    # (UCFD_PREC_FP64 runs the reference's operation order, bit-identical to
    # the oracle; each step solves the same system, so the per-step
    # increments dQ = upts_after - upts_before compare directly)
    def step_increment(P, inner):
        u0 = P.e["upts"].clone()
        P.step(args.rtol, args.max_pairs, inner)
        torch.cuda.synchronize()
        return P.e["upts"] - u0

    P0 = Problem(case, lc, 0, stream, device)
    dq0 = step_increment(P0, args.check)
    del P0
    torch.cuda.empty_cache()
    dq0_max = float(dq0.abs().max())
    err = {"err_vs_fp64": float((step_increment(P32, args.inner) - dq0).abs().max()) / dq0_max,
           "fp64_fma_err_vs_fp64": float((step_increment(P64, args.check) - dq0).abs().max()) / dq0_max,
           "definition": "max|dQ - dQ_fp64| / max|dQ_fp64| over all cells and variables, one pseudo-time step "
                         "solved to rtol, dQ_fp64 from UCFD_PREC_FP64 (the oracle's arithmetic)"}
    del dq0

    # ---- end to end through the C-ABI with pinned host buffers -------------
    Ph = Problem(case, lc, 2, None, device, host_inputs=True)
    if tuned:
        Ph.S.set_launch_config(**tuned["fp32"])
    for _ in range(max(1, args.warmup // 2)):
        Ph.step(args.rtol, args.max_pairs, args.inner)
    torch.cuda.synchronize()
    barrier(dist, device)
    t0 = time.perf_counter()
    pe = []
    calls = {}
    for _ in range(args.steps):
        pe.append(Ph.step(args.rtol, args.max_pairs, args.inner, calls)[0])
    torch.cuda.synchronize()
    e2e_s = reduce_max((time.perf_counter() - t0) / args.steps, dist, device)
    # the same steps again with the library's host<->device copies timed by
    # CUDA events (each timed copy waits for itself), then once more untimed:
    # where the time of the host-input calls goes, and whether the host link
    # changed speed meanwhile
    from ucfd_sparse_gb300 import lib as _lib
    xfer_calls, xfer_copies = {}, {}
    _lib.transfer_timing(True)
    t1 = time.perf_counter()
    for _ in range(args.steps):
        Ph.step(args.rtol, args.max_pairs, args.inner, xfer_calls, xfer_copies)
    torch.cuda.synchronize()
    xfer_s = (time.perf_counter() - t1) / args.steps
    xfer = _lib.transfer_stats()
    _lib.transfer_timing(False)
    t2 = time.perf_counter()
    for _ in range(args.steps):
        Ph.step(args.rtol, args.max_pairs, args.inner)
    torch.cuda.synchronize()
    again_s = (time.perf_counter() - t2) / args.steps
    K = args.steps
    xfer_out = {"ms_per_step": xfer_s * 1e3, "untimed_again_ms_per_step": again_s * 1e3,
                "h2d_ms_per_step": xfer["h2d_ms"] / K,
                "h2d_bytes_per_step": xfer["h2d_bytes"] / K,
                "h2d_GBps": xfer["h2d_bytes"] / max(xfer["h2d_ms"], 1e-9) / 1e6,
                "d2h_ms_per_step": xfer["d2h_ms"] / K,
                "d2h_bytes_per_step": xfer["d2h_bytes"] / K,
                "ms_per_call": {k: v * 1e3 / K for k, v in xfer_calls.items()},
                "copies_per_call": {k: {"h2d_ms": v["h2d_ms"] / K, "h2d_MB": v["h2d_bytes"] / K / 1e6,
                                        "d2h_ms": v["d2h_ms"] / K, "d2h_MB": v["d2h_bytes"] / K / 1e6}
                                    for k, v in xfer_copies.items()},
                "how": "CUDA events around every host<->device copy the library makes, the same steps repeated; "
                       "then the steps once more without timing"}
    # staged copies of the face Jacobians (UCFD_HOST_STAGE) against reading
    # them in place from pinned host memory in the Prepare kernels
    # (UCFD_HOST_MAP): steps alternate between the two, so both see the same
    # phases of the host link
    host_access0 = _lib.host_array_access()
    per_mode = {0: [], 1: []}
    calls_mode = {0: {}, 1: {}}
    for _ in range(args.steps):
        for mode in (0, 1):
            _lib.set_host_array_access(mode)
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            Ph.step(args.rtol, args.max_pairs, args.inner, calls_mode[mode])
            torch.cuda.synchronize()
            per_mode[mode].append(time.perf_counter() - t3)
    _lib.set_host_array_access(host_access0)
    other_access = {("UCFD_HOST_MAP" if m else "UCFD_HOST_STAGE"):
                    {"median_ms_per_step": statistics.median(v) * 1e3, "ms_per_step": [x * 1e3 for x in v],
                     "ms_per_call": {k: x * 1e3 / K for k, x in calls_mode[m].items()}}
                    for m, v in per_mode.items()}
    other_access["how"] = "steps alternating between the two modes, each timed alone (wall clock, synchronised)"
    # the same pinned jmat copied alone (torch copy, one transfer): the host link's rate for it
    jdev = torch.empty(Ph.e["jmat"].shape, dtype=Ph.e["jmat"].dtype, device=device)
    torch.cuda.synchronize()
    tj = time.perf_counter()
    jdev.copy_(Ph.e["jmat"], non_blocking=True)
    torch.cuda.synchronize()
    jmat_gbps = Ph.e["jmat"].numel() * 8 / (time.perf_counter() - tj) / 1e9
    del jdev
    e2e_val = reduce_sum(N * statistics.mean(pe) / e2e_s, dist, device) if dist else N * statistics.mean(pe) / e2e_s

    out = None
    if rank == 0:
        cpu = cpu_baseline(case) if ws == 1 else None
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms32, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 sweeps + f64 refinement/LU/residual", "data": "synthetic",
            "config": headline_config(args, N, len(rg), ws),
            "pairs_per_step": pairs_mean, "relres": max(rel32),
            "fp64": {"ms_per_step": ms64, "pairs_per_step": statistics.mean(pairs64), "relres": max(rel64),
                     "value": N * statistics.mean(pairs64) / (ms64 * 1e-3),
                     "sweep_ms": sweep64_ms, "sweep_GBps": bytes_sweep64 / (sweep64_ms * 1e-3) / 1e9,
                     "sweep_frac": bytes_sweep64 / (sweep64_ms * 1e-3) / 1e9 / peak,
                     "sweep_kernel": "fs_blusgs_sweep_kernel<double,5,6,true> (FP64 with fused multiply-adds)"},
            "speedup_fp32_refined_vs_fp64": ms64 / ms32,
            "err_vs_fp64": err["err_vs_fp64"], "error": err,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": Ph.h2d_bytes(),
                    "d2h_bytes_per_step": Ph.d2h_bytes(), "ms_per_step": e2e_s * 1e3,
                    "ms_per_call": {k: v * 1e3 / args.steps for k, v in calls.items()},
                    "jmat_copy_GBps": jmat_gbps, "copies_timed": xfer_out,
                    "host_array_access": "UCFD_HOST_MAP" if host_access0 == 1 else "UCFD_HOST_STAGE",
                    "host_array_access_compared": other_access},
            "gpu_launches": launches_per_step(nlev, int(round(pairs_mean)), args.inner, True) * args.steps,
            "clocks": clocks,
            "launch": tuned or "defaults (--no-autotune)",
        }
        print(json.dumps(out))
    barrier(dist, device)
    return out


# ---------------------------------------------------------------------------
# secondary workloads (one JSON line each; the default run is the BLU-SGS one)
# ---------------------------------------------------------------------------
def _events(stream):
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def lusgs_iter_bytes(rowptr, elt, nfv=5, nt=1, both=False):
    """Algorithmic bytes of one scalar LU-SGS pseudo-time iteration per
    UCFDLUSGS_Run (NS + RANS prepare, lower and upper sweeps, update), FlowSys
    layout: per face its index, area, spectral radius and (once, in the sweep
    where it is active) its normal; per cell the packed diagonal, the state
    and increment of every variable read/written once.  both: the loop's
    one-pass kernels (one prepare and one sweep per direction for both
    systems), which read each face's index and area once per kernel."""
    nnz = int(rowptr[-1])
    N = rowptr.shape[0] - 1
    nv = nfv + nt
    if both:
        per_face = (4 + 3 * elt) + 2 * (4 + 3 * elt) + 3 * elt    # prepare, 2 sweeps, normal once
        per_cell = 2 * nv * elt                                    # du = rhs copy
        per_cell += elt + 2 * nv * elt                             # rcp_vol, diag from base
        per_cell += 2 * (elt + nfv * elt + 3 * nv * elt)           # sweeps: rv, u, du own r/w + nbr, diag
        per_cell += 3 * nv * elt                                   # u += du
        return nnz * per_face + N * per_cell
    per_face = (4 + 2 * elt) * 2 + (4 + 3 * elt + 2 * elt)   # NS prepare + sweeps
    per_face += (4 + 2 * elt) + (4 + 3 * elt + 2 * elt)      # RANS prepare + sweeps
    per_cell = 2 * nv * elt                                    # du = rhs copy
    per_cell += elt + 2 * nfv * elt + elt + 2 * nt * elt       # rcp_vol, diag from base (NS, RANS)
    per_cell += 2 * (elt + 5 * elt + 3 * nfv * elt)            # NS sweeps: rv, u, du own r/w + nbr, diag
    per_cell += 2 * (elt + 5 * elt + 3 * nt * elt)             # RANS sweeps
    per_cell += 3 * nv * elt                                   # u += du
    return nnz * per_face + N * per_cell


def nsrans_sweep_bytes(rowptr, nfv=5, nt=1, elt=4):
    """Algorithmic bytes of one sweep of both scalar systems (the loop's
    one-pass kernel): per cell-face the neighbour index, area, both spectral
    radii and the normal; per cell rcp_vol, the mean-flow state values the
    fluxes read, du of every variable (own and neighbours' once), du written
    and diag -- 264 B per hex cell in FP32."""
    nnz = int(rowptr[-1])
    N = rowptr.shape[0] - 1
    nv = nfv + nt
    return nnz * (4 + (3 + 3) * elt) + N * (elt + nfv * elt + 3 * nv * elt)


def run_lusgs(args):
    """Steady pseudo-time loop: jittered, permuted hex, nvars = 5 + 1 RANS,
    FP32 state, greedy colouring; args.iters iterations as a captured CUDA
    graph (mode 0) and with persistent grid-synchronised sweeps (mode 1)."""
    import torch

    from ucfd_sparse_gb300 import _build, lib
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    from ucfd_sparse_gb300.flowsys import FlowSys
    _build.build()
    lib.load()
    m = args.mesh
    t0 = time.perf_counter()
    c = mg.lusgs_flowsys_case(m, nvars=6, seed=args.seed, rhs_scale=1e-3)
    gen_s = time.perf_counter() - t0
    N = c["nlocal"]
    ic, rg, lc = cl.greedy_coloring_csr(c["rowptr"], c["colidx"])
    dev = torch.device("cuda:0")
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    g = {k: T(c[k]) for k in ("rowptr", "colidx", "slots", "sides", "face_area", "face_normal", "rcp_vol", "fspr",
                              "tfspr", "dt", "rhs", "cell_ids", "vol")}
    up = T(c["upts"])
    stream = torch.cuda.Stream(device=dev)
    res = {}
    for mode in (0, 1):
        S = FlowSys(N, 6, 5, 3, c["nfaces"], 1, g["rowptr"], g["colidx"], g["slots"], g["sides"], g["face_area"],
                    g["face_normal"], g["rcp_vol"])
        S.set_coloring(lc)
        S.set_precision(2)
        S.set_stream(stream.cuda_stream, True)
        uu = up.clone()
        S.set_element(0, N, 6, g["cell_ids"], uu, g["rhs"], g["dt"], torch.zeros_like(uu), g["vol"],
                      torch.zeros_like(uu))
        S.set_lusgs(g["fspr"], g["tfspr"])
        S.lusgs_pack(0, 1.0, 0.0)
        if args.sweep_variant is not None:
            S.set_launch_config(threads_per_block=256, sweep_variant=args.sweep_variant, run_mode=mode)
            res.setdefault("launch", S.launch_config())
        elif not args.no_autotune:
            tuned = S.autotune(reps=2, cache=args.autotune_cache)  # block size x register build (state restored)
            tuned.pop("source", None)
            res.setdefault("launch", tuned)
        hist = np.zeros(args.iters)
        S.lusgs_run(3, 1.0, True, mode, None)          # warm-up (graph capture / occupancy query)
        S.lusgs_pack(0, 1.0, 0.0)
        torch.cuda.synchronize()
        e0, e1 = _events(stream)
        with ClockSampler(0) as clk:
            e0.record(stream)
            S.lusgs_run(args.iters, 1.0, True, mode, None)
            e1.record(stream)
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        S.lusgs_pack(0, 1.0, 0.0)
        S.lusgs_run(args.iters, 1.0, True, mode, hist)
        res[mode] = dict(ms=ms, clocks=clk.summary(), resid_first=float(hist[0]), resid_last=float(hist[-1]))
        # scalar sweep kernel alone (per-level launches): NS lower sweep, the
        # tuned launch and every variant at 256 threads
        if mode == 0:
            S.lusgs_ns_prepare(1.0)
            S.lusgs_rans_prepare(1.0)

            def lower_ms(sweep=S.lusgs_ns_lower):
                sweep(1.0)
                torch.cuda.synchronize()
                e0, e1 = _events(stream)
                e0.record(stream)
                for _ in range(10):
                    sweep(1.0)
                e1.record(stream)
                torch.cuda.synchronize()
                return e0.elapsed_time(e1) / 10

            res["sweep_ms"] = lower_ms()
            res["sweep_launch"] = S.launch_config()
            # the loop's sweep with the turbulence system: both systems in one
            # pass (one thread per cell), or the RANS sweep after the NS sweep
            res["rans_sweep_ms"] = lower_ms(S.lusgs_rans_lower)
            S.lusgs_nsrans_prepare(1.0)  # the packed face data the loop's sweep reads
            res["nsrans_sweep_ms"] = lower_ms(S.lusgs_nsrans_lower)
            cand = {}
            for var in (0, 1, 2, 3, 5):
                S.set_launch_config(threads_per_block=256, sweep_variant=var)
                cand[f"v{var}/b256"] = lower_ms()
            for tpb in (64, 128):
                S.set_launch_config(threads_per_block=tpb, sweep_variant=5)
                cand[f"v5/b{tpb}"] = lower_ms()
            res["sweep_candidates_ms"] = cand
        del S
    # error of the FP32 loop against the FP64 arithmetic of the oracle
    # (UCFD_PREC_FP64): args.iters iterations of each from the same state
    finals = {}
    for prec in (2, 0):
        S = FlowSys(N, 6, 5, 3, c["nfaces"], 1, g["rowptr"], g["colidx"], g["slots"], g["sides"], g["face_area"],
                    g["face_normal"], g["rcp_vol"])
        S.set_coloring(lc)
        S.set_precision(prec)
        S.set_stream(stream.cuda_stream, True)
        uu = up.clone()
        S.set_element(0, N, 6, g["cell_ids"], uu, g["rhs"], g["dt"], torch.zeros_like(uu), g["vol"],
                      torch.zeros_like(uu))
        S.set_lusgs(g["fspr"], g["tfspr"])
        if prec == 2 and res.get("launch"):
            S.set_launch_config(**res["launch"])
        S.lusgs_pack(0, 1.0, 0.0)
        S.lusgs_run(args.iters, 1.0, True, 0, None)
        S.lusgs_update(0)                           # the device-resident state back to uu
        torch.cuda.synchronize()
        finals[prec] = uu
        del S
    change = float((finals[0] - up).abs().max())
    err_lusgs = float((finals[2] - finals[0]).abs().max()) / change
    del finals
    torch.cuda.empty_cache()
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    # the loop sweeps both systems in one pass with one thread per cell
    both = res["sweep_launch"]["sweep_variant"] <= 2
    bytes_iter = lusgs_iter_bytes(c["rowptr"], 4, both=both)
    best = min(res[0]["ms"], res[1]["ms"])
    rp = c["rowptr"]
    nnz = int(rp[-1])
    # NS sweep algorithmic bytes, every array element once at storage precision:
    # per cell-face neighbour index, area, spectral radius, 3 normal components;
    # per cell rcp_vol and 4 x nvars state values (u and du of neighbours as
    # other cells' own data, du read and written, diag) -- 228 B/cell on hex
    ns_bytes = nnz * (4 + (2 + 3) * 4) + N * (4 + 4 * 5 * 4)
    both_bytes = nsrans_sweep_bytes(rp)
    sweep_bytes_, sweep_ms_ = (both_bytes, res["nsrans_sweep_ms"]) if both else (ns_bytes, res["sweep_ms"])
    out = {"workload": "lusgs", "metric": METRIC, "unit": UNIT,
           "config": {"workload": f"scalar LU-SGS pseudo-time loop, {m}^3 jittered permuted hex ({N} cells), "
                                  f"nvars 5 + 1 RANS, FP32, greedy colouring ({len(rg)} colours), "
                                  f"{args.iters} iterations", "cells": N, "colors": len(rg)},
           "value": N * args.iters / (best * 1e-3),
           "graph": {"ms": res[0]["ms"], "cell_updates_per_s": N * args.iters / (res[0]["ms"] * 1e-3),
                     "GBps": bytes_iter * args.iters / (res[0]["ms"] * 1e-3) / 1e9},
           "persistent": {"ms": res[1]["ms"], "cell_updates_per_s": N * args.iters / (res[1]["ms"] * 1e-3),
                          "GBps": bytes_iter * args.iters / (res[1]["ms"] * 1e-3) / 1e9},
           "bytes_per_cell_iteration": bytes_iter / N,
           "roofline": {"bound": "hbm",
                        "kernel": ("scalar_sweep_both_kernel<float,6,5,3> (both systems, lower sweep)" if both else
                                   "scalar_sweep_faces_kernel<float,6,5,3,false>"
                                   if res["sweep_launch"]["sweep_variant"] == 5 else
                                   "scalar_sweep_pair_kernel<float,6,5,3,false>"
                                   if res["sweep_launch"]["sweep_variant"] in (3, 4) else
                                   "scalar_sweep_kernel<float,6,5,3,false>"),
                        "launch": res["sweep_launch"],
                        "achieved": sweep_bytes_ / (sweep_ms_ * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": sweep_bytes_ / (sweep_ms_ * 1e-3) / 1e9 / peak,
                        "sweep_ms": sweep_ms_, "algorithmic_bytes_per_sweep": sweep_bytes_},
           "ns_sweep": {"kernel": "NS lower sweep alone (UCFDLUSGS_NSLowerSweep)", "ms": res["sweep_ms"],
                        "GBps": ns_bytes / (res["sweep_ms"] * 1e-3) / 1e9,
                        "frac": ns_bytes / (res["sweep_ms"] * 1e-3) / 1e9 / peak,
                        "algorithmic_bytes": ns_bytes, "candidates_ms": res["sweep_candidates_ms"]},
           "nsrans_sweep": {"ms": res["nsrans_sweep_ms"], "separate_ns_plus_rans_ms":
                            res["sweep_ms"] + res["rans_sweep_ms"], "rans_ms": res["rans_sweep_ms"],
                            "algorithmic_bytes": both_bytes},
           "loop_frac_of_peak": bytes_iter * args.iters / (best * 1e-3) / 1e9 / peak,
           "resid_fp64": [res[0]["resid_first"], res[0]["resid_last"]],
           "err_vs_fp64": err_lusgs,
           "err_definition": f"max|U_fp32 - U_fp64| / max|U_fp64 - U_0| after {args.iters} iterations of the graph "
                             f"loop from the same state, U_fp64 from UCFD_PREC_FP64 (the oracle's arithmetic)",
           "clocks": res[0]["clocks"], "generation_s": gen_s, "launch": res.get("launch")}
    if args.cpu_iters > 0:
        del g, up
        torch.cuda.empty_cache()
        # a bounded sample: the serial sweeps take over a minute per iteration at 256^3
        cm = min(m, args.cpu_mesh or 128)
        cc = c if cm == m else mg.lusgs_flowsys_case(cm, nvars=6, seed=args.seed, rhs_scale=1e-3)
        out["cpu_baseline"] = lusgs_cpu_baseline(cc, iters=args.cpu_iters)
    print(json.dumps(out))


def run_gmres(args):
    """GMRES(30) with the coloured BLU-SGS preconditioner on the Kuhn-tet
    BSR 5x5 system, to a 1e-10 relative residual: FP64 with fused
    multiply-adds (the `fp64` entry) and mixed (FP32 matvec + FP32
    preconditioner inside FP64 Arnoldi/refinement); BiCGSTAB (FP64) with the
    coloured BLU-SGS and the coloured block ILU(0)."""
    import torch

    from ucfd_sparse_gb300 import _build, lib
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    from ucfd_sparse_gb300.krylov import Precon, Solver, SpMat
    _build.build()
    lib.load()

    def coloured_case(mesh):
        s0 = mg.bsr_case(mesh, seed=args.seed)
        tab = np.where(s0["nei"] >= 0, s0["nei"], np.arange(s0["bn"])[None, :]).astype(np.int32)
        ic, rg, lc = cl.greedy_coloring(tab)
        new = np.empty(s0["bn"], dtype=np.int64)
        new[ic] = np.arange(s0["bn"])
        return mg.renumber_bsr(s0, new), rg

    t0 = time.perf_counter()
    s, rg = coloured_case(args.mesh)
    gen_s = time.perf_counter() - t0
    bn = s["bn"]
    n = bn * 5
    dev = torch.device("cuda:0")
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d = {k: T(s[k]) for k in ("rowptr", "colidx", "values", "diagslots", "rhs")}
    icolors = np.array([0] + rg, dtype=np.int32)
    A = SpMat(bn, 5, d["rowptr"], d["colidx"], d["values"], cuda=True)
    tol = 1e-10 * float(np.linalg.norm(s["rhs"]))
    nnzb = int(s["rowptr"][-1])
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    res = {}
    xs = {}
    for prec in (1, 2):
        pc = Precon(d["rowptr"], d["colidx"], d["diagslots"], d["values"])
        pc.set_pblusgs(bn, 5, len(rg), icolors, cuda=True)
        pc.set_precision(prec)
        pc.prepare()
        torch.cuda.synchronize()
        t = time.perf_counter()
        pc.prepare()  # structure cached: values gathered and factorised on the device
        torch.cuda.synchronize()
        reprep_ms = (time.perf_counter() - t) * 1e3
        sv = Solver(n, 30, 100, tol, cuda=True)
        sv.set_precision(prec)
        x = torch.zeros(n, dtype=torch.float64, device=dev)
        sv.solve(pc, A, x, d["rhs"])  # warm-up
        x.zero_()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("gmres_fp64" if prec == 1 else "gmres_mixed")
        t = time.perf_counter()
        sv.solve(pc, A, x, d["rhs"])
        torch.cuda.synchronize()
        el = time.perf_counter() - t
        torch.cuda.nvtx.range_pop()
        st, it, r = sv.result()
        res[prec] = dict(s=el, stat=st, restarts=it, resid=r / (tol / 1e-10), arnoldi=sv.arnoldi_steps(),
                         prepare_ms=reprep_ms)
        xs[prec] = x.clone()
        # preconditioner apply alone
        w = torch.randn(n, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(10):
            pc.apply(w)
        torch.cuda.synchronize()
        res[prec]["precon_ms"] = (time.perf_counter() - t) / 10 * 1e3
        # algorithmic bytes of one apply: every off-diagonal block and its column
        # once, the diagonal LU in both sweeps, the block vector in and out per sweep
        r = 8 if prec == 1 else 4
        pb = (nnzb - bn) * (4 + 25 * r) + bn * (2 * 25 * r + 2 * 2 * 5 * r)
        res[prec]["precon_GBps"] = pb / (res[prec]["precon_ms"] * 1e-3) / 1e9
        res[prec]["precon_frac"] = res[prec]["precon_GBps"] / peak
        del pc, sv
    # FP64 (FMA) GMRES ending a cycle once its residual estimate is low enough
    # (UCFDSolverSetCycleExit) instead of the reference's full 30-step cycle
    pc = Precon(d["rowptr"], d["colidx"], d["diagslots"], d["values"])
    pc.set_pblusgs(bn, 5, len(rg), icolors, cuda=True)
    pc.set_precision(1)
    pc.prepare()
    sv = Solver(n, 30, 100, tol, cuda=True)
    sv.set_precision(1)
    sv.set_cycle_exit(True)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    sv.solve(pc, A, x, d["rhs"])  # warm-up
    x.zero_()
    torch.cuda.synchronize()
    t = time.perf_counter()
    sv.solve(pc, A, x, d["rhs"])
    torch.cuda.synchronize()
    el = time.perf_counter() - t
    st, it, r = sv.result()
    res["fp64_cycle_exit"] = dict(s=el, stat=st, restarts=it, resid=r / (tol / 1e-10), arnoldi=sv.arnoldi_steps())
    xs["fp64_cycle_exit"] = x.clone()
    del pc, sv
    # the solution of the FP64 arithmetic of the oracle (UCFD_PREC_FP64: the
    # reference's operation order in the matvec and preconditioner), untimed
    pc = Precon(d["rowptr"], d["colidx"], d["diagslots"], d["values"])
    pc.set_pblusgs(bn, 5, len(rg), icolors, cuda=True)
    pc.set_precision(0)
    pc.prepare()
    sv = Solver(n, 30, 100, tol, cuda=True)
    sv.set_precision(0)
    x0 = torch.zeros(n, dtype=torch.float64, device=dev)
    sv.solve(pc, A, x0, d["rhs"])
    x0max = float(x0.abs().max())
    for key in (1, 2, "fp64_cycle_exit"):
        res[key]["err_vs_fp64"] = float((xs[key] - x0).abs().max()) / x0max
    del pc, sv, x0, xs
    torch.cuda.empty_cache()
    # BiCGSTAB (FP64) with the coloured BLU-SGS and the coloured block ILU(0)
    bic = {}
    for pc_kind in ("pblusgs", "pbilu"):
        pvals = d["values"].clone() if pc_kind == "pbilu" else d["values"]  # ILU prepare writes the factors
        pc = Precon(d["rowptr"], d["colidx"], d["diagslots"], pvals)
        t = time.perf_counter()
        if pc_kind == "pbilu":
            pc.set_pbilu(bn, 5, len(rg), icolors, cuda=True)
        else:
            pc.set_pblusgs(bn, 5, len(rg), icolors, cuda=True)
        pc.prepare()
        torch.cuda.synchronize()
        prep_s = time.perf_counter() - t
        # Prepare again on fresh values (same structure: cached, values
        # gathered and factorised on the device)
        if pc_kind == "pbilu":
            pvals.copy_(d["values"])
        torch.cuda.synchronize()
        t = time.perf_counter()
        pc.prepare()
        torch.cuda.synchronize()
        reprep_ms = (time.perf_counter() - t) * 1e3
        sv = Solver(n, 0, 200, tol, kind="bicgstab")
        x = torch.zeros(n, dtype=torch.float64, device=dev)
        sv.solve(pc, A, x, d["rhs"])  # warm-up
        x.zero_()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("bicgstab_" + pc_kind)
        t = time.perf_counter()
        sv.solve(pc, A, x, d["rhs"])
        torch.cuda.synchronize()
        el = time.perf_counter() - t
        torch.cuda.nvtx.range_pop()
        st, it, r = sv.result()
        bic[pc_kind] = dict(s=el, stat=st, iters=it, resid=r / (tol / 1e-10), first_prepare_s=prep_s,
                            prepare_ms=reprep_ms)
        del pc, sv, pvals
        torch.cuda.empty_cache()
    # SpMV kernel alone: FP64 in the reference's order, FP64 with fused
    # multiply-adds, FP32 values; beside them the reference's own GPU kernel
    # (_SpMV_CUDABSR<5>, cusparsemat.cu:74-139) compiled from its source
    from ucfd_sparse_gb300.lib import PREC_FP32, PREC_FP64, PREC_FP64_FMA
    x = torch.randn(n, dtype=torch.float64, device=dev)
    y = torch.zeros(n, dtype=torch.float64, device=dev)
    sp = {}
    for prec in (PREC_FP64, PREC_FP64_FMA, PREC_FP32):
        A.mult(1.0, x, 0.0, y, precision=prec)
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(20):
            A.mult(1.0, x, 0.0, y, precision=prec)
        torch.cuda.synchronize()
        sp[prec] = (time.perf_counter() - t) / 20 * 1e3
    b64 = nnzb * (4 + 25 * 8) + bn * (40 + 40)
    b32 = nnzb * (4 + 25 * 4) + bn * (40 + 40)
    ref_spmv = None
    from oracle import oracle as orc
    if orc.ref_cuda_available():
        R = orc.RefCudaBSR(5)
        cs = torch.cuda.current_stream(dev)
        yr = torch.zeros_like(y)
        launch = lambda: R.spmv(1.0, bn, d["rowptr"].data_ptr(), d["colidx"].data_ptr(), d["values"].data_ptr(),
                                x.data_ptr(), 0.0, yr.data_ptr(), cs.cuda_stream)
        launch()
        torch.cuda.synchronize()
        e0, e1 = _events(cs)
        e0.record(cs)
        for _ in range(20):
            launch()
        e1.record(cs)
        torch.cuda.synchronize()
        ref_ms = e0.elapsed_time(e1) / 20
        A.mult(1.0, x, 0.0, y, precision=PREC_FP64_FMA)
        agree = float((yr - y).abs().max() / y.abs().max())
        R.close()
        ref_spmv = {"kernel": "_SpMV_CUDABSR<5> of cusparsemat.cu, built from the reference source for sm_103a "
                              "(oracle/Makefile), launched as its SpMV_CUDABSR (128 threads, one per block row)",
                    "ms": ref_ms, "GBps": b64 / (ref_ms * 1e-3) / 1e9, "frac": b64 / (ref_ms * 1e-3) / 1e9 / peak,
                    "speedup_of_fp64_fma": ref_ms / sp[PREC_FP64_FMA], "speedup_of_fp64": ref_ms / sp[PREC_FP64],
                    "max_rel_diff_vs_fp64_fma": agree}
    out = {"workload": "gmres", "unit": "s to 1e-10",
           "config": {"workload": f"GMRES(30) + coloured BLU-SGS, Kuhn tets of a {args.mesh}^3 box ({bn} cells, "
                                  f"5x5 BSR, {nnzb} blocks), {len(rg)} colours, tol 1e-10 relative", "cells": bn},
           "fp64": res[1], "mixed": res[2], "speedup_mixed_vs_fp64": res[1]["s"] / res[2]["s"],
           "fp64_cycle_exit": res["fp64_cycle_exit"],
           "speedup_mixed_vs_fp64_cycle_exit": res["fp64_cycle_exit"]["s"] / res[2]["s"],
           "err_vs_fp64": res[2]["err_vs_fp64"],
           "err_definition": "max|x - x_fp64| / max|x_fp64|, x_fp64 the GMRES solution with UCFD_PREC_FP64 "
                             "(the oracle's arithmetic) to the same tolerance",
           "spmv": {"fp64_ms": sp[PREC_FP64], "fp32_ms": sp[PREC_FP32], "fp64_fma_ms": sp[PREC_FP64_FMA],
                    "fp64_GBps": b64 / (sp[PREC_FP64] * 1e-3) / 1e9, "fp32_GBps": b32 / (sp[PREC_FP32] * 1e-3) / 1e9,
                    "fp64_fma_GBps": b64 / (sp[PREC_FP64_FMA] * 1e-3) / 1e9,
                    "peak": peak, "fp64_frac": b64 / (sp[PREC_FP64] * 1e-3) / 1e9 / peak,
                    "fp64_fma_frac": b64 / (sp[PREC_FP64_FMA] * 1e-3) / 1e9 / peak,
                    "fp32_frac": b32 / (sp[PREC_FP32] * 1e-3) / 1e9 / peak,
                    "reference_gpu_kernel": ref_spmv},
           "bicgstab_fp64": bic,
           "generation_s": gen_s}
    del A, d, x, y
    torch.cuda.empty_cache()
    # the reference's CPU solvers beside the GPU ones, on a smaller system of
    # the same construction (the full one takes minutes on the host cores)
    if args.cpu_mesh is None:
        args.cpu_mesh = 48
    if args.cpu_mesh > 0:
        sc, rgc = coloured_case(args.cpu_mesh)
        icc = np.array([0] + rgc, dtype=np.int32)
        tolc = 1e-10 * float(np.linalg.norm(sc["rhs"]))
        cpu = krylov_cpu_baseline(sc, icc, tolc)
        dc = {k: T(sc[k]) for k in ("rowptr", "colidx", "values", "diagslots", "rhs")}
        Ac = SpMat(sc["bn"], 5, dc["rowptr"], dc["colidx"], dc["values"], cuda=True)
        gpu = {}
        for kind in ("gmres", "bicgstab"):
            pc = Precon(dc["rowptr"], dc["colidx"], dc["diagslots"], dc["values"])
            pc.set_pblusgs(sc["bn"], 5, len(rgc), icc, cuda=True)
            pc.prepare()
            sv = Solver(sc["bn"] * 5, 30, 100 if kind == "gmres" else 200, tolc, cuda=True, kind=kind)
            xc = torch.zeros(sc["bn"] * 5, dtype=torch.float64, device=dev)
            sv.solve(pc, Ac, xc, dc["rhs"])  # warm-up
            xc.zero_()
            torch.cuda.synchronize()
            t = time.perf_counter()
            sv.solve(pc, Ac, xc, dc["rhs"])
            torch.cuda.synchronize()
            gpu[kind] = {"s": time.perf_counter() - t, "stat": sv.result()[0], "iters": sv.result()[1]}
            del pc, sv
        out["cpu_baseline"] = dict(cpu, sample=f"FP64 GMRES(30) and BiCGSTAB with the coloured BLU-SGS to 1e-10 "
                                                f"relative on Kuhn tets of a {args.cpu_mesh}^3 box ({sc['bn']} cells)",
                                   gpu_same_system=gpu)
    print(json.dumps(out))


def run_colored(args):
    """The reference's own array API (colored LU-SGS step) on the 32^3 box,
    FP64, args.iters steps: host numpy arrays (staged by the library) and
    device tensors, against the oracle's CPU step."""
    import torch

    from oracle import oracle as orc
    from ucfd_sparse_gb300 import _build, lib
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    _build.build()
    lib.load()
    m = args.mesh
    c = mg.lusgs_case(m)
    icolor = cl.make_coloring(m, m, m)
    ranges = [(m ** 3 + 1) // 2, m ** 3]
    c["lcolor"] = mg.colors_from_icolor(icolor, ranges)
    N = c["neles"]
    out = {"workload": "colored", "unit": UNIT, "config": {"workload": f"colored LU-SGS array API, {m}^3 box, "
                                                                       f"checkerboard, FP64, {args.iters} steps",
                                                           "cells": N}}
    for where in ("host", "device"):
        if where == "device":
            cc = dict(c, **{k: torch.from_numpy(np.ascontiguousarray(c[k])).cuda() for k in
                            ("nei_ele", "fnorm_vol", "vec_fnorm", "fspr", "dt", "upts", "rhs", "lcolor")})
            ic = torch.from_numpy(icolor).cuda()
            diag = torch.zeros(N, dtype=torch.float64, device="cuda")
            dub = torch.zeros_like(cc["rhs"])
        else:
            cc = dict(c, upts=c["upts"].copy(), rhs=c["rhs"].copy())
            ic, diag, dub = icolor, np.zeros(N), np.zeros_like(c["rhs"])
        cl.colored_step(cc, ic, ranges, diag, dub)
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(args.iters):
            cl.colored_step(cc, ic, ranges, diag, dub)
        torch.cuda.synchronize()
        el = time.perf_counter() - t
        out[where] = {"s_per_step": el / args.iters, "cell_updates_per_s": N * args.iters / el}
    p = orc.Port(fast=True)
    t = time.perf_counter()
    p.legacy_step(c, icolor, ranges, c["lcolor"], nsteps=args.iters)
    el = time.perf_counter() - t
    out["cpu_port"] = {"s_per_step": el / args.iters, "cell_updates_per_s": N * args.iters / el,
                       "threads": os.cpu_count()}
    print(json.dumps(out))


def run_adjoint(args):
    """Differentiable colored LU-SGS step (C4 shape: jittered, permuted hex,
    greedy colouring): forward alone and forward + backward (the transposed
    sweeps giving d/d rhs, dt, fspr), FP64 and FP32, CUDA events over
    args.steps calls after args.warmup; beside it the reference's CPU
    forward step (the adjoint has no reference counterpart)."""
    import torch

    from oracle import oracle as orc
    from ucfd_sparse_gb300 import _build, lib
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    from ucfd_sparse_gb300.adjoint import ColoredMesh, lusgs_step
    _build.build()
    lib.load()
    m = args.mesh
    c = mg.lusgs_case(m, jitter=0.2, permute=True, seed=args.seed)
    N = c["neles"]
    icolor, ranges, lcolor = cl.greedy_coloring(c["nei_ele"])
    mesh = ColoredMesh(c["nei_ele"], c["fnorm_vol"], c["vec_fnorm"], icolor, ranges)
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    out = {"workload": "adjoint", "unit": UNIT,
           "config": {"workload": f"differentiable colored LU-SGS step, {m}^3 jittered permuted hex ({N} cells), "
                                  f"greedy colouring ({len(ranges)} colours), gradients w.r.t. rhs, dt, fspr",
                      "cells": N, "colors": len(ranges)}}
    for dt_ in (torch.float64, torch.float32):
        T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt_)
        x = {k: T(c[k]).requires_grad_(True) for k in ("rhs", "dt", "fspr")}
        up = T(c["upts"])
        g = torch.randn(c["rhs"].shape, dtype=dt_, device=dev)
        res = {}
        for mode in ("forward", "forward_backward"):
            def once():
                if mode == "forward":
                    with torch.no_grad():
                        lusgs_step(x["rhs"], x["dt"], x["fspr"], mesh, up)
                else:
                    for v in x.values():
                        v.grad = None
                    (lusgs_step(x["rhs"], x["dt"], x["fspr"], mesh, up) * g).sum().backward()
            for _ in range(max(args.warmup, 3)):
                once()
            torch.cuda.synchronize()
            e0, e1 = _events(stream)
            e0.record(stream)
            for _ in range(args.steps):
                once()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            res[mode] = {"ms": ms, "cell_updates_per_s": N / (ms * 1e-3)}
        out["fp64" if dt_ == torch.float64 else "fp32"] = res
    # the reference's CPU forward step on the same arrays
    c["lcolor"] = mg.colors_from_icolor(icolor, ranges)
    port = orc.Port(fast=True)
    t = time.perf_counter()
    port.legacy_step(c, icolor, ranges, c["lcolor"], nsteps=1)
    el = time.perf_counter() - t
    out["cpu_baseline"] = {"value": N / el, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                           "sample": f"one colored LU-SGS forward step (pre, lower and upper sweeps by colour, "
                                     f"update), FP64, on all {N} cells"}
    print(json.dumps(out))


def run_kernels(args):
    """The BLU-SGS pieces of one pseudo-time step timed one by one on a
    single FP32 system (device-resident inputs): Pack + NSPrepare, one
    lower+upper sweep pair over all colours, and the FP64 true residual.
    Small meshes of this workload are the ncu capture cases."""
    import torch

    from ucfd_sparse_gb300 import _build, lib
    from ucfd_sparse_gb300 import coloredlusgs as cl
    _build.build()
    lib.load()
    case = make_case(args.mesh, seed=args.seed)
    N = case["nlocal"]
    ic, rg, lc = cl.greedy_coloring_csr(case["rowptr"], case["colidx"], order=args.coloring)
    device = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=device)
    prec = 1 if args.fp64 else 2
    P = Problem(case, lc, prec, stream, device)
    S = P.S
    tuned = P.tune(cache=args.autotune_cache) if not args.no_autotune else None
    if args.sweep_variant is not None:
        S.blusgs_pack(0, 0.0)
        S.blusgs_ns_prepare()
        S.set_launch_config(threads_per_block=256, sweep_variant=args.sweep_variant)
        tuned = S.launch_config()
    S.blusgs_reset()

    def timed(fn, reps):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = _events(stream)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def prep():
        S.blusgs_pack(0, 0.0)
        S.blusgs_ns_prepare()

    def pair():
        S.blusgs_ns_lower()
        S.blusgs_ns_upper()

    reps = max(args.steps, 3)
    prep_ms = timed(prep, reps)
    # every launch candidate of the sweep (unless one variant was asked
    # for), then the chosen one
    candidates = {}
    cand_list = ((64, 0), (128, 0), (256, 0), (64, 1), (256, 1), (0, 2), (0, 3), (64, 4), (128, 4), (256, 4))
    if args.sweep_variant is not None:
        cand_list = ()
    for tpb, var in cand_list:
        if prec != 2 and var in (2, 3):
            continue                      # bulk-copy kernels are FP32-only
        S.set_launch_config(threads_per_block=tpb, sweep_variant=var)
        candidates[f"v{var}/b{tpb}"] = timed(pair, max(10, 2 * reps))
    if tuned:
        S.set_launch_config(**tuned)
    pair_ms = timed(pair, max(20, 4 * reps))
    S.blusgs_solve(0.0, 1, 1)                    # one refinement step: x (FP64) != 0 from here on
    res_ms = timed(S.blusgs_residual, reps)      # includes its host read-back
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    nnz = int(case["rowptr"][-1])
    nF = int(case["nfaces"])
    elt = 8 if prec != 2 else 4
    sw = 2 * sweep_bytes(case["rowptr"], elt, 5)
    # Prepare: jmat read twice (transpose in, face records out) + written once,
    # face records read per cell-face (the diagonal half in the first pass,
    # the off-diagonal half in the second), the sweep blocks D^-1 J fv written
    # once, J64 (FP32 mode) / D / LU written, ELL index arrays read per pass
    jb = 25 * elt
    prep_b = (nF * 400 * 3 + nnz * (400 + jb + (200 if prec == 2 else 0) + 2 * (4 + 4 + 1 + 8))
              + N * (200 + 25 * elt + 8 + 8))
    res_b = nnz * (4 + 8 + 200) + N * (8 + 200 + 40 + 40 + 20)
    out = {"workload": "kernels", "unit": "ms", "config": {
        "workload": f"BLU-SGS 5x5 {'FP64 (FMA)' if prec != 2 else 'FP32'} pieces, {args.mesh}^3 jittered permuted "
                    f"hex ({N} cells, {nF} faces), "
                    f"{len(rg)} colours", "cells": N, "colors": len(rg)},
        "launch": tuned,
        "prepare": {"ms": prep_ms, "GBps": prep_b / (prep_ms * 1e-3) / 1e9, "bytes": prep_b},
        "sweep_pair": {"ms": pair_ms, "GBps": sw / (pair_ms * 1e-3) / 1e9, "frac": sw / (pair_ms * 1e-3) / 1e9 / peak,
                       "bytes": sw},
        "residual_fp64": {"ms": res_ms, "GBps": res_b / (res_ms * 1e-3) / 1e9, "bytes": res_b},
        "sweep_pair_candidates_ms": candidates,
        "peak": peak}
    print(json.dumps(out))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mesh", type=int, default=None,
                    help="box size (default per workload: blusgs/kernels 128, lusgs 256, gmres 96, colored 32, "
                         "adjoint 64)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--rtol", type=float, default=1e-10)
    ap.add_argument("--inner", type=int, default=20, help="FP32 sweep pairs per FP64 refinement step")
    ap.add_argument("--check", type=int, default=20,
                    help="FP64 solve: pairs between residual checks (as many as the FP32 solve's --inner)")
    ap.add_argument("--max-pairs", type=int, default=400)
    ap.add_argument("--ref-pairs", type=int, default=1)
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch configuration")
    ap.add_argument("--sweep-variant", type=int, default=None,
                    help="lusgs / kernels workloads: this sweep variant at 256 threads instead of the autotuned "
                         "launch (a profiler then sees one known kernel)")
    ap.add_argument("--fp64", action="store_true", help="kernels workload: the FP64 (fused multiply-add) system")
    ap.add_argument("--autotune-cache", default=None,
                    help="JSON file of launch choices: reused when it holds one for the system, else written "
                         "(a profiled run can then repeat the choices of an unprofiled one)")
    ap.add_argument("--coloring", default="index", choices=["index", "bfs"],
                    help="greedy colouring visiting cells by index or in breadth-first order")
    ap.add_argument("--workload", default="blusgs",
                    choices=["blusgs", "lusgs", "gmres", "colored", "kernels", "adjoint"],
                    help="blusgs: the headline line; the others measure the remaining configurations")
    ap.add_argument("--iters", type=int, default=200, help="iterations of the lusgs/colored workloads")
    ap.add_argument("--cpu-mesh", type=int, default=None,
                    help="box of the smaller system the reference's CPU path runs on (gmres: 48, 0 skips; "
                         "lusgs: at most 128)")
    ap.add_argument("--cpu-iters", type=int, default=1,
                    help="lusgs workload: pseudo-time iterations of the reference's CPU path (0: skip)")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        args.warmup = 3
    if args.mesh is None:
        args.mesh = {"lusgs": 256, "gmres": 96, "colored": 32, "adjoint": 64}.get(args.workload, 128)
    if args.sweep_variant is not None:
        args.no_autotune = True
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "lusgs":
        run_lusgs(args)
    elif args.workload == "gmres":
        run_gmres(args)
    elif args.workload == "colored":
        run_colored(args)
    elif args.workload == "kernels":
        run_kernels(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
