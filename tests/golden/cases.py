"""Seeded parity cases shared by the golden generator and the tests.

Each case is rebuilt from its seed by ucfd_sparse_gb300.meshgen (pure
numpy, platform-independent arithmetic), so only outputs are stored.
"""
from __future__ import annotations

import hashlib

import numpy as np

from ucfd_sparse_gb300 import meshgen as mg

BOXES = [(4, 3, 5), (5, 5, 5), (3, 1, 2)]

# colored array LU-SGS: name -> meshgen arguments and step count
LEGACY = {
    "leg8": dict(m=8, jitter=0.0, permute=False, coloring="checker", nsteps=1),
    "leg32": dict(m=32, jitter=0.0, permute=False, coloring="checker", nsteps=10),
    "legjp6": dict(m=6, jitter=0.2, permute=True, coloring="greedy", nsteps=3),
    "legjp12rans": dict(m=12, jitter=0.2, permute=True, coloring="greedy", nsteps=2, nvars=6),
}

FLOWSYS = {
    "fs5": dict(m=5, seed=0, kappa=1.3, a0=0.7, turb_factor=1.5, nsteps=2),
    "fs9": dict(m=9, seed=4, kappa=1.0, a0=0.0, turb_factor=1.0, nsteps=1),
}

BLUSGS = {
    "blu6": dict(m=6, seed=0, nsweeps=3),
    "blu10": dict(m=10, seed=2, nsweeps=2),
}

KRYLOV = {
    "kry4": dict(mesh=4, seed=0, m=30),
    "kry6": dict(mesh=6, seed=1, m=10),
}


def input_hash(d: dict) -> str:
    h = hashlib.sha256()
    for k in sorted(d):
        v = d[k]
        if isinstance(v, np.ndarray):
            h.update(k.encode())
            h.update(np.ascontiguousarray(v).tobytes())
    return h.hexdigest()


def legacy_case(m, jitter, permute, coloring, nsteps, nvars=5, seed=0):
    c = mg.lusgs_case(m, nvars=nvars, jitter=jitter, permute=permute, seed=seed)
    if coloring == "checker":
        icolor = mg.box_coloring(m, m, m)
        ranges = [int((m ** 3 + 1) // 2), m ** 3]
        lcolor = mg.colors_from_icolor(icolor, ranges)
    else:
        icolor, ranges, lcolor = mg.greedy_coloring_np(c["nei_ele"])
    c["lcolor"] = lcolor.astype(np.int32)
    return c, icolor.astype(np.int32), [int(r) for r in ranges], c["lcolor"]


def flowsys_case(m, seed, **_):
    """Jittered, permuted hex FlowSys mesh with nvars = 6 (5 flow + 1 turb)."""
    b = mg.blusgs_case(m, nvars=6, seed=seed)
    b["nfvars"] = 5
    rng = np.random.default_rng(seed + 11)
    N, nF = b["nlocal"], b["nfaces"]
    upts = mg.free_stream(6, N)
    upts[5] = rng.uniform(0.1, 1.0, N)
    inp = dict(upts=upts, rhs=rng.standard_normal((6, N)), dt=rng.uniform(1e-3, 1e-2, N),
               dsrc=rng.uniform(0.0, 1.0, (6, N)), fspr=rng.uniform(0.5, 2.0, nF), tfspr=rng.uniform(0.5, 2.0, nF),
               rowptr=b["rowptr"], colidx=b["colidx"])
    return b, inp


def blusgs_case(m, seed, **_):
    return mg.blusgs_case(m, seed=seed)


def bsr_case(mesh, seed, **_):
    return mg.bsr_case(mesh, seed=seed)


def spmv_x(s):
    return np.random.default_rng(7).standard_normal(s["bn"] * s["blk"])


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
