"""Generate the golden vectors of tests/golden/ from the reference itself.

Run where a UCFD_SPARSE source tree exists:
    python tests/golden/make_golden.py <reference_root>
(or with UCFD_REFERENCE_SRC set to that root)

* box connectivity and the checkerboard come from importing the reference
  example module examples/utils/pbutils.py;
* every numerical fixture comes from the reference library compiled from
  its own sources (oracle/Makefile -> oracle/_ref, FP64, -O2,
  -ffp-contract=off), driven through its public C API.
The inputs are regenerated from seeds by ucfd_sparse_gb300.meshgen, so the
fixtures store only outputs (plus a hash of the inputs, to detect drift).
Large outputs are stored as SHA-256 digests of their bytes: the pinned
oracle reproduces them bit for bit.
"""
from __future__ import annotations

import hashlib
import importlib.util
import json
import os
import sys

import numpy as np

# one OpenMP thread: the reference's reductions then sum in index order, as
# the restatement does (set before the reference library is loaded)
os.environ["OMP_NUM_THREADS"] = "1"

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
OUT = os.path.dirname(os.path.abspath(__file__))

from oracle import oracle as orc  # noqa: E402
from tests.golden import cases  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main(ref_root: str) -> None:
    os.environ["UCFD_REFERENCE_SRC"] = ref_root
    orc.REF_SRC = ref_root
    assert orc.build_ref(), "reference sources not found"
    ref = orc.Ref()
    spec = importlib.util.spec_from_file_location("pbutils", os.path.join(ref_root, "examples", "utils",
                                                                          "pbutils.py"))
    pb = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pb)

    meta = {}
    arrays = {}

    # ---- pbutils connectivity / checkerboard --------------------------------
    for (m, n, l) in cases.BOXES:
        arrays[f"nei_{m}_{n}_{l}"] = np.asarray(pb.make_nei_ele(m, n, l), dtype=np.int32)
        arrays[f"col_{m}_{n}_{l}"] = np.asarray(pb.make_coloring(m, n, l), dtype=np.int32)
    m = 32
    meta["nei_32_sha"] = sha(np.asarray(pb.make_nei_ele(m, m, m), dtype=np.int32))
    meta["col_32_sha"] = sha(np.asarray(pb.make_coloring(m, m, m), dtype=np.int32))

    # ---- colored LU-SGS through the reference FlowSys on the colour-renumbered mesh
    for name, kw in cases.LEGACY.items():
        c, icolor, ranges, lcolor = cases.legacy_case(**kw)
        fs = orc.legacy_to_flowsys(c, icolor)
        up = ref.flowsys_lusgs_step(fs, c["upts"], c["rhs"], c["dt"], np.zeros_like(c["rhs"]), fs["fspr"],
                                    nsteps=kw["nsteps"])
        meta[f"{name}_in"] = cases.input_hash(c)
        if c["neles"] <= 4096:
            arrays[f"{name}_upts"] = up
        meta[f"{name}_upts_sha"] = sha(up)

    # ---- FlowSys scalar LU-SGS, natural order, NS + RANS
    for name, kw in cases.FLOWSYS.items():
        fs, inp = cases.flowsys_case(**kw)
        up = ref.flowsys_lusgs_step(fs, inp["upts"], inp["rhs"], inp["dt"], inp["dsrc"], inp["fspr"], inp["tfspr"],
                                    kappa=kw["kappa"], a0=kw["a0"], turb_factor=kw["turb_factor"], rans=True,
                                    nsteps=kw["nsteps"])
        meta[f"{name}_in"] = cases.input_hash(inp)
        arrays[f"{name}_upts"] = up
        meta[f"{name}_upts_sha"] = sha(up)

    # ---- FlowSys BLU-SGS
    for name, kw in cases.BLUSGS.items():
        b = cases.blusgs_case(**kw)
        up, res = ref.flowsys_blusgs(b, b["rhs"], b["dt"], b["jmat"], b["vol"], b["upts"], nsweeps=kw["nsweeps"])
        meta[f"{name}_in"] = cases.input_hash({k: b[k] for k in ("rhs", "dt", "jmat", "upts", "rowptr", "colidx")})
        arrays[f"{name}_upts"] = up
        arrays[f"{name}_resid"] = res
        meta[f"{name}_upts_sha"] = sha(up)

    # ---- Krylov: BSR SpMV and BLU-SGS-preconditioned GMRES
    for name, kw in cases.KRYLOV.items():
        s = cases.bsr_case(**kw)
        x = cases.spmv_x(s)
        y = ref.bsr_spmv(s, x, 1.5, -0.5, x)
        meta[f"{name}_in"] = cases.input_hash({k: s[k] for k in ("values", "rowptr", "colidx", "rhs")})
        arrays[f"{name}_spmv"] = y
        tol = 1e-10 * float(np.linalg.norm(s["rhs"]))
        xs, st, it, res, hist = ref.gmres(s, s["rhs"], m=kw["m"], maxiter=20, tol=tol)
        arrays[f"{name}_gmres_x"] = xs
        meta[f"{name}_gmres"] = dict(stat=st, iters=it, resid=res, tol=tol)
        # block ILU(0) factors (bilu.c), BiCGSTAB with BLU-SGS and with BILU
        meta[f"{name}_bilu_sha"] = sha(ref.ilu_factor(s, "bilu"))
        for pc in ("blusgs", "bilu"):
            xb, st, it, res, hist = ref.bicgstab(s, s["rhs"], maxiter=20, tol=tol, pc=pc)
            arrays[f"{name}_bicgstab_{pc}_x"] = xb
            meta[f"{name}_bicgstab_{pc}"] = dict(stat=st, iters=it, resid=res, tol=tol,
                                                 hist=[float(h) for h in hist[:it + 1]])

    np.savez_compressed(os.path.join(OUT, "golden.npz"), **arrays)
    with open(os.path.join(OUT, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrote", len(arrays), "arrays,", len(meta), "entries")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("UCFD_REFERENCE_SRC")
    if not root:
        sys.exit("usage: python tests/golden/make_golden.py <root of the UCFD_SPARSE source tree> "
                 "(or set UCFD_REFERENCE_SRC)")
    main(root)
