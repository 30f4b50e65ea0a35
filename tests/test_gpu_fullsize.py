"""Size-independent properties at the full workload sizes (GPU).

The oracle finishes only small cases; at full size the checks are
properties that hold whatever the size:

* C2  128^3 hex (2,097,152 cells), BLU-SGS: FP32 sweeps + FP64 refinement
  and plain FP64 sweeps both reach a 1e-10 relative residual, confirmed by
  the independent allocation-free residual, and agree with each other;
  every launch variant of the FP32 sweep gives the same sweep pair;
* C3  96^3 Kuhn tets (5,308,416 cells), GMRES(30) + coloured BLU-SGS: FP64
  and mixed precision reach the tolerance, and the true residual
  ||b - A x|| recomputed with the FP64 matvec confirms it;
* C4  64^3 hex, differentiable colored step: the adjoint passes the
  dot-product test against central differences of the forward step;
* C5  256^3 hex (16,777,216 cells), scalar LU-SGS loop NS + RANS: CUDA graph
  and persistent kernel give bit-identical states and residual histories.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda", 0)


def T(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def blusgs_system(case, lc, prec):
    from ucfd_sparse_gb300.flowsys import FlowSys
    m = {k: T(case[k]) for k in ("rowptr", "colidx", "slots", "sides", "face_area", "face_normal", "rcp_vol")}
    S = FlowSys(case["nlocal"], 5, 5, 3, case["nfaces"], 1, m["rowptr"], m["colidx"], m["slots"], m["sides"],
                m["face_area"], m["face_normal"], m["rcp_vol"])
    S.set_coloring(lc)
    S.set_precision(prec)
    e = {k: T(case[k]) for k in ("rhs", "dt", "cell_ids", "vol", "jmat")}
    e["upts"] = T(np.array(case["upts"]))
    e["dsrc"] = torch.zeros_like(e["rhs"])
    e["res"] = torch.zeros_like(e["rhs"])
    S.set_element(0, case["neles"], 6, e["cell_ids"], e["upts"], e["rhs"], e["dt"], e["dsrc"], e["vol"], e["res"])
    S.set_blusgs(e["jmat"])
    S._fullsize_keep = (m, e)
    S.blusgs_pack(0, 0.0)
    S.blusgs_ns_prepare()
    S.blusgs_reset()
    return S, e


def noalloc_relres(S):
    from ctypes import byref, c_double
    from ucfd_sparse_gb300.lib import call
    r = c_double()
    call("UCFDBLUSGS_ResidualNoAlloc", S._h, byref(r))
    return r.value


def test_c2_blusgs_full_size(ucfd):
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    case = mg.blusgs_case(128, seed=0)
    assert case["nlocal"] == 2097152
    ic, rg, lc = cl.greedy_coloring_csr(case["rowptr"], case["colidx"])
    sols = {}
    for prec in (2, 1):
        S, e = blusgs_system(case, lc, prec)
        pairs, rel = S.blusgs_solve(1e-10, 400, 20)
        assert rel <= 1e-10, (prec, pairs, rel)
        assert S.blusgs_residual() <= 1e-10
        assert noalloc_relres(S) <= 1e-10
        S.blusgs_update(0)
        sols[prec] = (e["upts"] - T(case["upts"])).cpu().numpy()
        del S, e
        torch.cuda.empty_cache()
    d32, d64 = sols[2], sols[1]
    assert np.abs(d32 - d64).max() <= 1e-7 * np.abs(d64).max()


def test_c2_sweep_variants_full_size(ucfd):
    """One FP32 sweep pair under every launch variant, bit for bit."""
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    case = mg.blusgs_case(128, seed=1)
    ic, rg, lc = cl.greedy_coloring_csr(case["rowptr"], case["colidx"])
    S, e = blusgs_system(case, lc, 2)
    outs = []
    for tpb, var in ((256, 0), (64, 1), (0, 2), (0, 3), (128, 4)):
        S.set_launch_config(threads_per_block=tpb, sweep_variant=var)
        S.blusgs_reset()
        S.blusgs_ns_lower()
        S.blusgs_ns_upper()
        S.blusgs_sub_residual(0)
        outs.append(e["res"].cpu().numpy().copy())
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])


def test_c3_gmres_full_size(ucfd):
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    from ucfd_sparse_gb300.krylov import Precon, Solver, SpMat
    s0 = mg.bsr_case(96, seed=0)
    assert s0["bn"] == 5308416
    tab = np.where(s0["nei"] >= 0, s0["nei"], np.arange(s0["bn"])[None, :]).astype(np.int32)
    ic, rg, lc = cl.greedy_coloring(tab)
    new = np.empty(s0["bn"], dtype=np.int64)
    new[ic] = np.arange(s0["bn"])
    s = mg.renumber_bsr(s0, new)
    del s0
    bn = s["bn"]
    n = bn * 5
    d = {k: T(s[k]) for k in ("rowptr", "colidx", "values", "diagslots", "rhs")}
    A = SpMat(bn, 5, d["rowptr"], d["colidx"], d["values"], cuda=True)
    bnorm = float(torch.linalg.norm(d["rhs"]))
    tol = 1e-10 * bnorm
    icolors = np.array([0] + rg, dtype=np.int32)
    for prec in (1, 2):
        pc = Precon(d["rowptr"], d["colidx"], d["diagslots"], d["values"])
        pc.set_pblusgs(bn, 5, len(rg), icolors, cuda=True)
        pc.set_precision(prec)
        pc.prepare()
        sv = Solver(n, 30, 100, tol, cuda=True)
        sv.set_precision(prec)
        x = torch.zeros(n, dtype=torch.float64, device=DEV)
        sv.solve(pc, A, x, d["rhs"])
        st, it, r = sv.result()
        assert st == 0 and r <= tol, (prec, st, it, r)
        # true residual with the FP64 matvec: r = b - A x
        y = d["rhs"].clone()
        A.mult(-1.0, x, 1.0, y)
        assert float(torch.linalg.norm(y)) <= 1.01 * tol
        del pc, sv, x, y
        torch.cuda.empty_cache()


def test_c4_adjoint_full_size(ucfd):
    """Dot-product test at 64^3: <g, J v> by central differences of the
    forward colored step against <J^T g, v> from the adjoint (FP64)."""
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    from ucfd_sparse_gb300.adjoint import ColoredMesh, lusgs_step
    c = mg.lusgs_case(64, jitter=0.2, permute=True, seed=0)
    icolor, ranges, lcolor = cl.greedy_coloring(c["nei_ele"])
    mesh = ColoredMesh(c["nei_ele"], c["fnorm_vol"], c["vec_fnorm"], icolor, ranges)
    rng = np.random.default_rng(11)
    x = {k: T(c[k]).requires_grad_(True) for k in ("rhs", "dt", "fspr")}
    v = {k: T(rng.standard_normal(c[k].shape) * np.abs(c[k]).mean()) for k in ("rhs", "dt", "fspr")}
    up = T(c["upts"])
    g = T(rng.standard_normal(c["rhs"].shape))
    (lusgs_step(x["rhs"], x["dt"], x["fspr"], mesh, up) * g).sum().backward()
    adj = sum(float((x[k].grad * v[k]).sum()) for k in x)
    h = 1e-6
    with torch.no_grad():
        fp = lusgs_step(*(x[k] + h * v[k] for k in ("rhs", "dt", "fspr")), mesh, up)
        fm = lusgs_step(*(x[k] - h * v[k] for k in ("rhs", "dt", "fspr")), mesh, up)
    fd = float(((fp - fm) * g).sum()) / (2 * h)
    assert abs(adj - fd) <= 1e-6 * max(abs(fd), 1e-30), (adj, fd)


def test_c5_lusgs_loop_full_size(ucfd):
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    from ucfd_sparse_gb300.flowsys import FlowSys
    c = mg.lusgs_flowsys_case(256, nvars=6, seed=0, rhs_scale=1e-3)
    N = c["nlocal"]
    assert N == 16777216
    ic, rg, lc = cl.greedy_coloring_csr(c["rowptr"], c["colidx"])
    g = {k: T(c[k]) for k in ("rowptr", "colidx", "slots", "sides", "face_area", "face_normal", "rcp_vol", "fspr",
                              "tfspr", "dt", "rhs", "cell_ids", "vol")}
    out = {}
    for mode in (0, 1):
        S = FlowSys(N, 6, 5, 3, c["nfaces"], 1, g["rowptr"], g["colidx"], g["slots"], g["sides"], g["face_area"],
                    g["face_normal"], g["rcp_vol"])
        S.set_coloring(lc)
        S.set_precision(2)
        up = T(c["upts"])
        S.set_element(0, N, 6, g["cell_ids"], up, g["rhs"], g["dt"], torch.zeros_like(up), g["vol"],
                      torch.zeros_like(up))
        S.set_lusgs(g["fspr"], g["tfspr"])
        S.lusgs_pack(0, 1.0, 0.0)
        hist = np.zeros(3)
        S.lusgs_run(3, 1.0, True, mode, hist)
        S.lusgs_update(0)
        out[mode] = (up.cpu().numpy(), hist)
        del S, up
        torch.cuda.empty_cache()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert np.all(np.isfinite(out[0][1])) and out[0][1][0] > 0
