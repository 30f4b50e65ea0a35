"""The full workload sizes (GPU): parity with the oracle and
size-independent properties.

Parity: the CUDA path in its FP64 mode (UCFD_PREC_FP64, the reference's
operation order) against the oracle's CPU restatement on the same seeded
inputs, bit for bit, on the benchmark meshes:

* C2  128^3 jittered, permuted hex (2,097,152 cells), BLU-SGS 5x5: Pack,
  NSPrepare, Reset, one lower + upper sweep pair, SubResidual, Update in
  greedy colour order, against the reference call sequence on the colour-
  renumbered mesh (blusgs.c:17-57, 126-155, 161-197, 200-270, 273-373);
* C3  Kuhn tets of a 96^3 box (5,308,416 cells), BSR 5x5: one matvec
  (sparsemat.c:57-101) and one coloured BLU-SGS preconditioner apply
  (precon/blusgs.c:7-100 on the colour-ordered matrix);
* C5  256^3 jittered, permuted hex (16,777,216 cells), scalar LU-SGS NS +
  1-equation RANS: one pseudo-time iteration (lusgs.c:8-321) in colour
  order; the FP32 path's error against it is bounded as well.
The oracle's sweeps are serial, as the reference's: about a minute of CPU for
C5 and half a minute for C2.

Properties that hold whatever the size:

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

# FP32 sweeps against the FP64 arithmetic, one C5 iteration:
# max|dU_fp32 - dU_fp64| <= C5_FP32_BOUND * max|dU_fp64|
C5_FP32_BOUND = 1e-4


def T(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def renumber_by_colour(case):
    """Greedy colouring of a FlowSys mesh and the mesh renumbered colour by
    colour (on which the oracle's natural-order sweeps are the coloured
    sweeps) -> (renumbered case, lcolor, colour range ends)."""
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    ic, rg, lc = cl.greedy_coloring_csr(case["rowptr"], case["colidx"])
    new = np.empty(case["nlocal"], dtype=np.int64)
    new[ic] = np.arange(case["nlocal"])
    return mg.renumber_flowsys(case, new), lc, rg


# the meshes take a minute each to generate: once per module
@pytest.fixture(scope="module")
def c2():
    from ucfd_sparse_gb300 import meshgen as mg
    case = mg.blusgs_case(128, seed=0)
    assert case["nlocal"] == 2097152
    br, lc, rg = renumber_by_colour(case)
    return case, br, lc, rg


@pytest.fixture(scope="module")
def c3():
    """The C3 system renumbered colour by colour and its colour offsets."""
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    s0 = mg.bsr_case(96, seed=0)
    assert s0["bn"] == 5308416
    tab = np.where(s0["nei"] >= 0, s0["nei"], np.arange(s0["bn"])[None, :]).astype(np.int32)
    ic, rg, lc = cl.greedy_coloring(tab)
    new = np.empty(s0["bn"], dtype=np.int64)
    new[ic] = np.arange(s0["bn"])
    return mg.renumber_bsr(s0, new), rg


@pytest.fixture(scope="module")
def c5():
    from ucfd_sparse_gb300 import meshgen as mg
    c = mg.lusgs_flowsys_case(256, nvars=6, seed=0, rhs_scale=1e-3)
    assert c["nlocal"] == 16777216
    br, lc, rg = renumber_by_colour(c)
    return c, br, lc, rg


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


def test_c2_blusgs_full_size(c2, ucfd):
    case, _, lc, _ = c2
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


def test_c3_gmres_full_size(c3, ucfd):
    from ucfd_sparse_gb300.krylov import Precon, Solver, SpMat
    s, rg = c3
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


def test_c5_lusgs_loop_full_size(c5, ucfd):
    from ucfd_sparse_gb300.flowsys import FlowSys
    c, _, lc, _ = c5
    N = c["nlocal"]
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


# ---------------------------------------------------------------------------
# parity with the oracle at full size
# ---------------------------------------------------------------------------
def flowsys(case, nvars, lc, prec):
    from ucfd_sparse_gb300.flowsys import FlowSys
    m = {k: T(case[k]) for k in ("rowptr", "colidx", "slots", "sides", "face_area", "face_normal", "rcp_vol")}
    S = FlowSys(case["nlocal"], nvars, 5, 3, case["nfaces"], 1, m["rowptr"], m["colidx"], m["slots"], m["sides"],
                m["face_area"], m["face_normal"], m["rcp_vol"])
    S.set_coloring(lc)
    S.set_precision(prec)
    return S


def test_c2_blusgs_fp64_bitexact_full_size(c2, port, ucfd):
    case, br, lc, rg = c2
    assert len(rg) == 7
    S = flowsys(case, 5, lc, 0)
    e = {k: T(case[k]) for k in ("rhs", "dt", "cell_ids", "vol", "jmat")}
    e["upts"] = T(np.array(case["upts"]))
    e["res"] = torch.zeros_like(e["rhs"])
    S.set_element(0, case["neles"], 6, e["cell_ids"], e["upts"], e["rhs"], e["dt"], torch.zeros_like(e["rhs"]),
                  e["vol"], e["res"])
    S.set_blusgs(e["jmat"])
    S.blusgs_pack(0, 0.0)
    S.blusgs_ns_prepare()
    S.blusgs_reset()
    S.blusgs_ns_lower()
    S.blusgs_ns_upper()
    S.blusgs_sub_residual(0)
    S.blusgs_update(0)
    got_up, got_res = e["upts"].cpu().numpy(), e["res"].cpu().numpy()
    S.destroy()
    del S, e
    torch.cuda.empty_cache()
    up, _, res, _ = port.flowsys_blusgs(br, case["rhs"], case["dt"], case["jmat"], case["vol"], case["upts"],
                                        nsweeps=1)
    np.testing.assert_array_equal(got_up, up)
    np.testing.assert_array_equal(got_res, res)
    assert np.abs(up - case["upts"]).max() > 0


def test_c3_spmv_and_coloured_blusgs_fp64_bitexact_full_size(c3, port, ucfd):
    from ucfd_sparse_gb300.krylov import Precon, SpMat
    s, rg = c3
    bn = s["bn"]
    icolors = np.array([0] + rg, dtype=np.int32)
    rng = np.random.default_rng(21)
    x = rng.standard_normal(bn * 5)
    b = rng.standard_normal(bn * 5)
    d = {k: T(s[k]) for k in ("rowptr", "colidx", "values", "diagslots")}
    A = SpMat(bn, 5, d["rowptr"], d["colidx"], d["values"], cuda=True)
    y = torch.zeros(bn * 5, dtype=torch.float64, device=DEV)
    A.mult(1.0, T(x), 0.0, y)
    got_y = y.cpu().numpy()
    pc = Precon(d["rowptr"], d["colidx"], d["diagslots"], d["values"])
    pc.set_pblusgs(bn, 5, len(rg), icolors, cuda=True)
    pc.set_precision(0)
    pc.prepare()
    xb = T(b)
    pc.apply(xb)
    got_pc = xb.cpu().numpy()
    del A, pc, d, y, xb
    torch.cuda.empty_cache()
    np.testing.assert_array_equal(got_y, port.bsr_spmv(s, x))
    np.testing.assert_array_equal(got_pc, port.precon_apply(s, b, icolors=icolors))


def test_c5_lusgs_iteration_full_size(c5, port, ucfd):
    """One NS + RANS iteration, FP64 bit for bit (one thread per cell and one
    thread per active face); FP32 within C5_FP32_BOUND."""
    c, br, lc, rg = c5
    N = c["nlocal"]
    g = {k: T(c[k]) for k in ("fspr", "tfspr", "dt", "rhs", "cell_ids", "vol")}
    got = {}
    for prec, var in ((0, 0), (0, 5), (2, 0), (2, 5)):
        S = flowsys(c, 6, lc, prec)
        S.set_launch_config(threads_per_block=256, sweep_variant=var)
        up = T(c["upts"])
        S.set_element(0, N, 6, g["cell_ids"], up, g["rhs"], g["dt"], torch.zeros_like(up), g["vol"],
                      torch.zeros_like(up))
        S.set_lusgs(g["fspr"], g["tfspr"])
        S.lusgs_pack(0, 1.0, 0.0)
        S.lusgs_ns_prepare(1.0)
        S.lusgs_ns_lower(1.0)
        S.lusgs_ns_upper(1.0)
        S.lusgs_rans_prepare(1.0)
        S.lusgs_rans_lower(1.0)
        S.lusgs_rans_upper(1.0)
        S.lusgs_update(0)
        got[prec, var] = up.cpu().numpy()
        S.destroy()
        del S, up
        torch.cuda.empty_cache()
    del g
    torch.cuda.empty_cache()
    ref = port.flowsys_lusgs_step(br, c["upts"], c["rhs"], c["dt"], np.zeros_like(c["rhs"]), c["fspr"],
                                  c["tfspr"], rans=True, nsteps=1)[0]
    np.testing.assert_array_equal(got[0, 0], ref)
    # one thread per active face: the same terms in the same order
    np.testing.assert_array_equal(got[0, 5], ref)
    np.testing.assert_array_equal(got[2, 5], got[2, 0])
    d64 = ref - c["upts"]
    err = np.abs((got[2, 0] - c["upts"]) - d64).max() / np.abs(d64).max()
    print(f"C5 FP32 iteration: max|dU32 - dU64| / max|dU64| = {err:.3e}")
    assert err <= C5_FP32_BOUND, err
