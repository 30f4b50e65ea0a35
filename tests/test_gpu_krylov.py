"""GPU parity of the Krylov path: BSR SpMV, BLU-SGS preconditioners (natural
and coloured) and GMRES(m), against the oracle."""
import numpy as np
import pytest
import torch

from tests.golden import cases

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def colour_renumbered(s):
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    tab = np.where(s["nei"] >= 0, s["nei"], np.arange(s["bn"])[None, :]).astype(np.int32)
    ic, rg, lc = cl.greedy_coloring(tab)
    new = np.empty(s["bn"], dtype=np.int64)
    new[ic] = np.arange(s["bn"])
    return mg.renumber_bsr(s, new), [0] + rg


@pytest.mark.parametrize("name", sorted(cases.KRYLOV))
@pytest.mark.parametrize("on_device", [False, True])
def test_spmv_bitexact(name, on_device, golden, ucfd):
    from ucfd_sparse_gb300.krylov import SpMat
    meta, arr = golden
    s = cases.bsr_case(**cases.KRYLOV[name])
    conv = dev if on_device else np.ascontiguousarray
    A = SpMat(s["bn"], s["blk"], conv(s["rowptr"]), conv(s["colidx"]), conv(s["values"]), cuda=on_device)
    x = cases.spmv_x(s)
    y = conv(x.copy())
    A.mult(1.5, conv(x), -0.5, y)
    y = y.cpu().numpy() if on_device else y
    np.testing.assert_array_equal(y, arr[f"{name}_spmv"])


@pytest.mark.parametrize("fp32", [False, True])
def test_spmv_beta_zero_does_not_read_y(fp32, port, ucfd):
    """y = A x with beta = 0 over a y full of NaN: y is not read (the
    product equals the oracle's with a zero y)."""
    from ucfd_sparse_gb300.krylov import SpMat
    s = cases.bsr_case(mesh=4, seed=5)
    A = SpMat(s["bn"], s["blk"], dev(s["rowptr"]), dev(s["colidx"]), dev(s["values"]), cuda=True)
    x = cases.spmv_x(s)
    y = torch.full((x.size,), float("nan"), dtype=torch.float64, device="cuda")
    A.mult(2.0, dev(x), 0.0, y, fp32=fp32)
    got = y.cpu().numpy()
    ref = port.bsr_spmv(s, x, alpha=2.0, beta=0.0, y=np.zeros_like(x))
    assert np.isfinite(got).all()
    if fp32:
        assert np.abs(got - ref).max() <= 2e-6 * np.abs(ref).max()
    else:
        np.testing.assert_array_equal(got, ref)


def test_spmv_fp32_values(golden, ucfd):
    from ucfd_sparse_gb300.krylov import SpMat
    meta, arr = golden
    s = cases.bsr_case(**cases.KRYLOV["kry6"])
    A = SpMat(s["bn"], s["blk"], s["rowptr"], s["colidx"], s["values"])
    x = cases.spmv_x(s)
    y = x.copy()
    A.mult(1.5, x, -0.5, y, fp32=True)
    ref = arr["kry6_spmv"]
    assert np.abs(y - ref).max() <= 2e-6 * np.abs(ref).max()


@pytest.mark.parametrize("coloured", [False, True])
def test_precon_apply_bitexact(coloured, port, ucfd):
    from ucfd_sparse_gb300.krylov import Precon
    s0 = cases.bsr_case(mesh=5, seed=3)
    s, ic = colour_renumbered(s0)
    b = np.random.default_rng(5).standard_normal(s["bn"] * 5)
    pc = Precon(s["rowptr"], s["colidx"], s["diagslots"], s["values"])
    if coloured:
        pc.set_pblusgs(s["bn"], 5, len(ic) - 1, np.array(ic, dtype=np.int32))
    else:
        pc.set_blusgs(s["bn"], 5)
    pc.prepare()
    x = b.copy()
    pc.apply(x)
    ref = port.precon_apply(s, b, icolors=ic if coloured else None)
    np.testing.assert_array_equal(x, ref)
    assert pc.levels() <= len(ic) - 1


def test_precon_natural_order_unrenumbered(port, ucfd):
    """Natural-order BLU-SGS on a matrix whose numbering is not colour-major:
    level scheduling reproduces the sequential sweep exactly."""
    from ucfd_sparse_gb300.krylov import Precon
    s = cases.bsr_case(mesh=4, seed=8)
    b = np.random.default_rng(6).standard_normal(s["bn"] * 5)
    pc = Precon(s["rowptr"], s["colidx"], s["diagslots"], s["values"])
    pc.set_blusgs(s["bn"], 5)
    pc.prepare()
    assert pc.levels() > 4
    x = dev(b)
    pc.apply(x)
    np.testing.assert_array_equal(x.cpu().numpy(), port.precon_apply(s, b))


@pytest.mark.parametrize("name", sorted(cases.KRYLOV))
def test_gmres_matches_oracle(name, golden, port, ucfd):
    from ucfd_sparse_gb300.krylov import Precon, Solver, SpMat
    meta, arr = golden
    kw = cases.KRYLOV[name]
    s = cases.bsr_case(**kw)
    g = meta[f"{name}_gmres"]
    A = SpMat(s["bn"], 5, s["rowptr"], s["colidx"], s["values"])
    pc = Precon(s["rowptr"], s["colidx"], s["diagslots"], s["values"])
    pc.set_blusgs(s["bn"], 5)
    pc.prepare()
    sv = Solver(s["bn"] * 5, kw["m"], 20, g["tol"])
    sv.trace()
    x = np.zeros(s["bn"] * 5)
    sv.solve(pc, A, x, s["rhs"])
    st, it, res = sv.result()
    assert (st, it) == (g["stat"], g["iters"])
    ref = arr[f"{name}_gmres_x"]
    assert np.abs(x - ref).max() <= 1e-10 * np.abs(ref).max()
    assert res <= g["tol"]


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_gmres_coloured_and_mixed_reach_1e10(prec, port, ucfd):
    from ucfd_sparse_gb300.krylov import Precon, Solver, SpMat
    s0 = cases.bsr_case(mesh=8, seed=2)
    s, ic = colour_renumbered(s0)
    n = s["bn"] * 5
    d = {k: dev(s[k]) for k in ("rowptr", "colidx", "values", "diagslots", "rhs")}
    A = SpMat(s["bn"], 5, d["rowptr"], d["colidx"], d["values"], cuda=True)
    pc = Precon(d["rowptr"], d["colidx"], d["diagslots"], d["values"])
    pc.set_pblusgs(s["bn"], 5, len(ic) - 1, np.array(ic, dtype=np.int32), cuda=True)
    pc.set_precision(prec)
    pc.prepare()
    tol = 1e-10 * float(np.linalg.norm(s["rhs"]))
    sv = Solver(n, 30, 50, tol, cuda=True)
    sv.set_precision(prec)
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    sv.solve(pc, A, x, d["rhs"])
    st, it, res = sv.result()
    assert st == 0 and res <= tol
    xr, st_o, it_o, res_o, _ = port.gmres(s, s["rhs"], m=30, maxiter=50, tol=tol, pc="pblusgs", icolors=ic)
    assert st_o == 0
    assert np.abs(x.cpu().numpy() - xr).max() <= 1e-8 * np.abs(xr).max()


@pytest.mark.parametrize("prec", [0, 1])
def test_gmres_cycle_exit(prec, port, ucfd):
    """UCFDSolverSetCycleExit: the FP64 GMRES ends its cycle once the residual
    estimate is low enough -- fewer Arnoldi steps than the reference's full
    cycle, the same status, at most one more restart check, the true
    residual within tol and the solution within 1e-8 of the oracle's."""
    from ucfd_sparse_gb300.krylov import Precon, Solver, SpMat
    s0 = cases.bsr_case(mesh=8, seed=2)
    s, ic = colour_renumbered(s0)
    n = s["bn"] * 5
    d = {k: dev(s[k]) for k in ("rowptr", "colidx", "values", "diagslots", "rhs")}
    A = SpMat(s["bn"], 5, d["rowptr"], d["colidx"], d["values"], cuda=True)
    pc = Precon(d["rowptr"], d["colidx"], d["diagslots"], d["values"])
    pc.set_pblusgs(s["bn"], 5, len(ic) - 1, np.array(ic, dtype=np.int32), cuda=True)
    pc.set_precision(prec)
    pc.prepare()
    tol = 1e-10 * float(np.linalg.norm(s["rhs"]))
    steps, xs = {}, {}
    for on in (False, True):
        sv = Solver(n, 30, 50, tol, cuda=True)
        sv.set_precision(prec)
        sv.set_cycle_exit(on)
        x = torch.zeros(n, dtype=torch.float64, device="cuda")
        sv.solve(pc, A, x, d["rhs"])
        st, it, res = sv.result()
        assert st == 0 and res <= tol
        steps[on] = (it, sv.arnoldi_steps())
        xs[on] = x.cpu().numpy()
        y = d["rhs"].clone()
        A.mult(-1.0, x, 1.0, y)
        assert float(torch.linalg.norm(y)) <= 1.01 * tol
    xr, st_o, it_o, res_o, _ = port.gmres(s, s["rhs"], m=30, maxiter=50, tol=tol, pc="pblusgs", icolors=ic)
    assert steps[False][0] == it_o
    assert steps[True][0] <= it_o + 1           # at most one extra restart check
    assert steps[True][1] < steps[False][1]
    assert np.abs(xs[True] - xr).max() <= 1e-8 * np.abs(xr).max()


# ---- block / scalar ILU(0) and BiCGSTAB -----------------------------------------
def scalar_case(s):
    """A CSR matrix (blk 1) on the BSR pattern: the (0, 0) entry of each block."""
    v = np.ascontiguousarray(np.asarray(s["values"]).reshape(-1, s["blk"], s["blk"])[:, 0, 0])
    return dict(s, blk=1, values=v)


@pytest.mark.parametrize("kind", ["bilu", "pbilu", "ilu"])
def test_ilu_factors_and_apply_bitexact(kind, port, ucfd):
    """Prepare factorises on the GPU (FP64, level by level) and, as the
    reference does, overwrites the caller's values with the factors: bit for
    bit the oracle's (bilu.c / ilu.c); the apply equals the oracle's."""
    from ucfd_sparse_gb300.krylov import Precon
    s0 = cases.bsr_case(mesh=5, seed=4)
    s, ic = colour_renumbered(s0) if kind == "pbilu" else (s0, None)
    if kind == "ilu":
        s = scalar_case(s)
    vals = np.array(s["values"], dtype=np.float64)
    pc = Precon(s["rowptr"], s["colidx"], s["diagslots"], vals)
    if kind == "bilu":
        pc.set_bilu(s["bn"], s["blk"])
    elif kind == "pbilu":
        pc.set_pbilu(s["bn"], s["blk"], len(ic) - 1, ic)
    else:
        pc.set_ilu(s["bn"])
    pc.prepare()
    fv = port.ilu_factor(s) if kind == "ilu" else port.bilu_factor(s)
    np.testing.assert_array_equal(vals, fv)
    b = np.random.default_rng(7).standard_normal(s["bn"] * s["blk"])
    x = b.copy()
    pc.apply(x)
    ref = port.ilu_apply(s, fv, b) if kind == "ilu" else port.bilu_apply(s, fv, b)
    np.testing.assert_array_equal(x, ref)
    if kind == "bilu":
        assert pc.levels() > 2   # natural order: level-scheduled


def test_bilu_fp32_apply_close(port, ucfd):
    from ucfd_sparse_gb300.krylov import Precon
    s = cases.bsr_case(mesh=5, seed=8)
    vals = np.array(s["values"], dtype=np.float64)
    pc = Precon(s["rowptr"], s["colidx"], s["diagslots"], vals)
    pc.set_bilu(s["bn"], s["blk"])
    pc.set_precision(2)
    pc.prepare()
    b = np.random.default_rng(3).standard_normal(s["bn"] * 5)
    x = b.copy()
    pc.apply(x)
    ref = port.bilu_apply(s, port.bilu_factor(s), b)
    assert np.abs(x - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("name", sorted(cases.KRYLOV))
@pytest.mark.parametrize("pc_kind", ["blusgs", "bilu"])
@pytest.mark.parametrize("on_device", [False, True])
def test_bicgstab_matches_reference(name, pc_kind, on_device, golden, ucfd):
    """BiCGSTAB (bicgstab.c) on the GPU: the reference's status, iteration
    count and residual history; the solution within 1e-10 of the
    reference's (the device reductions sum in another order)."""
    from ucfd_sparse_gb300.krylov import Precon, Solver, SpMat
    meta, arr = golden
    s = cases.bsr_case(**cases.KRYLOV[name])
    g = meta[f"{name}_bicgstab_{pc_kind}"]
    conv = dev if on_device else np.ascontiguousarray
    A = SpMat(s["bn"], s["blk"], conv(s["rowptr"]), conv(s["colidx"]), conv(s["values"]), cuda=on_device)
    pvals = conv(np.array(s["values"], dtype=np.float64))
    pc = Precon(conv(s["rowptr"]), conv(s["colidx"]), conv(s["diagslots"]), pvals)
    if pc_kind == "bilu":
        pc.set_bilu(s["bn"], s["blk"])
    else:
        pc.set_blusgs(s["bn"], s["blk"])
    pc.prepare()
    n = s["bn"] * s["blk"]
    sv = Solver(n, 0, 20, g["tol"], kind="bicgstab")
    sv.trace()
    x = conv(np.zeros(n))
    sv.solve(pc, A, x, conv(s["rhs"]))
    st, it, res = sv.result()
    assert (st, it) == (g["stat"], g["iters"])
    np.testing.assert_allclose(sv.history()[:it + 1], g["hist"], rtol=1e-8)
    xh = x.cpu().numpy() if on_device else x
    ref = arr[f"{name}_bicgstab_{pc_kind}_x"]
    assert np.abs(xh - ref).max() <= 1e-10 * np.abs(ref).max()


def test_bicgstab_edge_cases(port, ucfd):
    """Iteration limit 0 (REACH_ITERMAX, no iteration), zero right-hand side
    (rho breakdown, status 3) and a limit that stops before convergence."""
    from ucfd_sparse_gb300.krylov import Precon, Solver, SpMat
    s = cases.bsr_case(mesh=4, seed=2)
    n = s["bn"] * 5
    A = SpMat(s["bn"], 5, s["rowptr"], s["colidx"], s["values"])
    pc = Precon(s["rowptr"], s["colidx"], s["diagslots"], np.array(s["values"]))
    pc.set_blusgs(s["bn"], 5)
    pc.prepare()
    for maxiter, b, want in ((0, s["rhs"], 2), (10, np.zeros(n), 3), (1, s["rhs"], 2)):
        sv = Solver(n, 0, maxiter, 1e-30, kind="bicgstab")
        x = np.zeros(n)
        sv.solve(pc, A, x, np.ascontiguousarray(b))
        st, it, res = sv.result()
        xo, sto, ito, reso, _ = port.bicgstab(s, b, maxiter=maxiter, tol=1e-30, pc="blusgs")
        assert (st, it) == (sto, ito) == (want, ito)
        assert np.abs(x - xo).max() <= 1e-10 * max(np.abs(xo).max(), 1e-300)


@pytest.mark.parametrize("pc_kind", ["pbilu", "pblusgs"])
def test_bicgstab_coloured_reaches_tolerance(pc_kind, port, ucfd):
    """Coloured preconditioners on a larger system: converged, and the true
    residual ||b - A x|| confirms the estimate."""
    from ucfd_sparse_gb300.krylov import Precon, Solver, SpMat
    s0 = cases.bsr_case(mesh=12, seed=9)
    s, ic = colour_renumbered(s0)
    n = s["bn"] * 5
    A = SpMat(s["bn"], 5, dev(s["rowptr"]), dev(s["colidx"]), dev(s["values"]), cuda=True)
    pc = Precon(dev(s["rowptr"]), dev(s["colidx"]), dev(s["diagslots"]), dev(np.array(s["values"])))
    if pc_kind == "pbilu":
        pc.set_pbilu(s["bn"], 5, len(ic) - 1, ic, cuda=True)
    else:
        pc.set_pblusgs(s["bn"], 5, len(ic) - 1, ic, cuda=True)
    pc.prepare()
    tol = 1e-10 * float(np.linalg.norm(s["rhs"]))
    sv = Solver(n, 0, 100, tol, kind="bicgstab")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    b = dev(s["rhs"])
    sv.solve(pc, A, x, b)
    st, it, res = sv.result()
    assert st == 0 and res < tol
    r = b.clone()
    A.mult(-1.0, x, 1.0, r)
    assert float(torch.linalg.norm(r)) <= 10 * tol


def _fill(dst, src):
    """Writes src into the caller-owned array dst in place (host or device)."""
    if isinstance(dst, torch.Tensor):
        dst.copy_(torch.from_numpy(np.ascontiguousarray(src)))
    else:
        np.copyto(dst, src)


@pytest.mark.parametrize("kind", ["pblusgs", "pbilu"])
@pytest.mark.parametrize("on_device", [False, True])
def test_reprepare_with_new_values(kind, on_device, port, ucfd):
    """A second Prepare after new values were written into the same array
    (structure unchanged: the structure built by the first Prepare is kept
    and only the values are gathered on the device) gives, bit for bit, the
    factors and apply of the oracle on the new values."""
    from ucfd_sparse_gb300.krylov import Precon
    s1, ic = colour_renumbered(cases.bsr_case(mesh=5, seed=3))
    s2, ic2 = colour_renumbered(cases.bsr_case(mesh=5, seed=11))
    for k in ("rowptr", "colidx", "diagslots"):
        np.testing.assert_array_equal(s1[k], s2[k])   # same mesh: same structure
    assert ic == ic2 and not np.array_equal(s1["values"], s2["values"])
    conv = dev if on_device else np.ascontiguousarray
    vals = conv(np.array(s1["values"], dtype=np.float64))
    pc = Precon(conv(s1["rowptr"]), conv(s1["colidx"]), conv(s1["diagslots"]), vals)
    icn = np.array(ic, dtype=np.int32)
    if kind == "pbilu":
        pc.set_pbilu(s1["bn"], 5, len(ic) - 1, icn)
    else:
        pc.set_pblusgs(s1["bn"], 5, len(ic) - 1, icn)
    b = np.random.default_rng(5).standard_normal(s1["bn"] * 5)
    for s in (s1, s2):
        _fill(vals, s["values"])
        pc.prepare()
        x = b.copy()
        pc.apply(x)
        if kind == "pbilu":
            fv = port.bilu_factor(s)
            got = vals.cpu().numpy() if on_device else vals
            np.testing.assert_array_equal(got, fv)
            ref = port.bilu_apply(s, fv, b)
        else:
            ref = port.precon_apply(s, b, icolors=ic)
        np.testing.assert_array_equal(x, ref)


@pytest.mark.parametrize("on_device", [False, True])
def test_reprepare_detects_structure_change(on_device, port, ucfd):
    """Another matrix of the same size written into the same rowptr /
    colidx / diagslots arrays changes their fingerprints: Prepare rebuilds
    the schedule and layout, and the apply is the oracle's on the new
    matrix."""
    from ucfd_sparse_gb300.krylov import Precon
    s0 = cases.bsr_case(mesh=4, seed=8)
    s1, _ = colour_renumbered(s0)
    assert s0["rowptr"][-1] == s1["rowptr"][-1] and not np.array_equal(s0["colidx"], s1["colidx"])
    conv = dev if on_device else np.ascontiguousarray
    arrs = {k: conv(np.array(s0[k])) for k in ("rowptr", "colidx", "diagslots", "values")}
    pc = Precon(arrs["rowptr"], arrs["colidx"], arrs["diagslots"], arrs["values"])
    pc.set_blusgs(s0["bn"], 5)
    b = np.random.default_rng(6).standard_normal(s0["bn"] * 5)
    for s in (s0, s1):
        for k in arrs:
            _fill(arrs[k], s[k])
        pc.prepare()
        x = b.copy()
        pc.apply(x)
        np.testing.assert_array_equal(x, port.precon_apply(s, b))


@pytest.mark.parametrize("on_device", [False, True])
def test_spmat_update_values(on_device, ucfd):
    """UCFDMatUpdateValues re-gathers the values on the device: the product
    equals a new matrix created on the new values, bit for bit, for the
    FP64 values and the FP32 copy; a changed structure is rebuilt."""
    from ucfd_sparse_gb300.krylov import SpMat
    s1 = cases.bsr_case(mesh=4, seed=1)
    s2 = cases.bsr_case(mesh=4, seed=2)
    s3, _ = colour_renumbered(s1)
    conv = dev if on_device else np.ascontiguousarray
    arrs = {k: conv(np.array(s1[k])) for k in ("rowptr", "colidx", "values")}
    A = SpMat(s1["bn"], 5, arrs["rowptr"], arrs["colidx"], arrs["values"], cuda=on_device)
    x = cases.spmv_x(s1)
    y = np.zeros_like(x)
    A.mult(1.0, x, 0.0, y, fp32=True)   # makes the FP32 copy, refreshed by updates
    for s in (s2, s3):
        for k in arrs:
            _fill(arrs[k], s[k])
        A.update_values()
        F = SpMat(s["bn"], 5, s["rowptr"], s["colidx"], s["values"])
        for fp32 in (False, True):
            y, yf = np.zeros_like(x), np.zeros_like(x)
            A.mult(1.0, x, 0.0, y, fp32=fp32)
            F.mult(1.0, x, 0.0, yf, fp32=fp32)
            np.testing.assert_array_equal(y, yf)


def _block_diagonal(bn, blk, seed):
    """A matrix with only diagonal blocks (no L or U entries at all)."""
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((bn, blk, blk)) * 0.1 + np.eye(blk) * 2.0
    idx = np.arange(bn, dtype=np.int32)
    return dict(bn=bn, blk=blk, rowptr=np.arange(bn + 1, dtype=np.int32), colidx=idx, diagslots=idx.copy(),
                values=np.ascontiguousarray(v.reshape(-1)), rhs=rng.standard_normal(bn * blk))


@pytest.mark.parametrize("bn", [1, 7])
@pytest.mark.parametrize("kind", ["blusgs", "pblusgs", "bilu", "ilu"])
def test_precon_without_off_diagonal_blocks(bn, kind, port, ucfd):
    """Block-diagonal systems (an empty strictly lower and upper part) and a
    single block row: Prepare, apply and SpMV equal the oracle bit for bit,
    and BiCGSTAB solves them."""
    from ucfd_sparse_gb300.krylov import Precon, Solver, SpMat
    s = _block_diagonal(bn, 1 if kind == "ilu" else 5, seed=bn)
    blk = s["blk"]
    vals = np.array(s["values"])
    pc = Precon(s["rowptr"], s["colidx"], s["diagslots"], vals)
    if kind == "blusgs":
        pc.set_blusgs(bn, blk)
    elif kind == "pblusgs":
        pc.set_pblusgs(bn, blk, 1, np.array([0, bn], dtype=np.int32))
    elif kind == "bilu":
        pc.set_bilu(bn, blk)
    else:
        pc.set_ilu(bn)
    pc.prepare()
    b = s["rhs"]
    x = b.copy()
    pc.apply(x)
    if kind in ("blusgs", "pblusgs"):
        ref = port.precon_apply(s, b, icolors=[0, bn] if kind == "pblusgs" else None)
    elif kind == "bilu":
        fv = port.bilu_factor(s)
        np.testing.assert_array_equal(vals, fv)
        ref = port.bilu_apply(s, fv, b)
    else:
        fv = port.ilu_factor(s)
        np.testing.assert_array_equal(vals, fv)
        ref = port.ilu_apply(s, fv, b)
    np.testing.assert_array_equal(x, ref)
    A = SpMat(bn, blk, s["rowptr"], s["colidx"], s["values"])
    y = np.zeros(bn * blk)
    A.mult(1.0, b, 0.0, y)
    np.testing.assert_array_equal(y, port.bsr_spmv(s, b))
    if kind != "ilu":
        pc2 = Precon(s["rowptr"], s["colidx"], s["diagslots"], np.array(s["values"]))
        pc2.set_blusgs(bn, blk)
        pc2.prepare()
        tol = 1e-12 * float(np.linalg.norm(b))
        sv = Solver(bn * blk, 0, 20, tol, kind="bicgstab")
        xs = np.zeros(bn * blk)
        sv.solve(pc2, A, xs, np.ascontiguousarray(b))
        assert sv.result()[0] == 0
        assert np.linalg.norm(port.bsr_spmv(s, xs) - b) <= 1e-10 * np.linalg.norm(b)


@pytest.mark.skipif(not __import__("oracle.oracle", fromlist=["x"]).ref_cuda_available(),
                    reason="the reference's GPU matvec was not compiled (oracle/_ref/cusparsemat.cubin)")
def test_reference_gpu_matvec_agrees(port, ucfd):
    """The reference's own _SpMV_CUDABSR<5> (cusparsemat.cu:74-139, built from
    its source), which the bench times beside this library's matvec, gives
    the oracle's product up to the rounding of fused multiply-adds, as does
    this library's FMA-mode product."""
    import torch

    from oracle.oracle import RefCudaBSR
    from ucfd_sparse_gb300.krylov import SpMat
    from ucfd_sparse_gb300.lib import PREC_FP64_FMA
    s = cases.bsr_case(mesh=6, seed=7)
    bn = s["bn"]
    x = cases.spmv_x(s)
    d = {k: dev(s[k]) for k in ("rowptr", "colidx", "values")}
    xd = dev(x)
    torch.cuda.synchronize()
    R = RefCudaBSR(5)
    yr = torch.zeros(bn * 5, dtype=torch.float64, device="cuda")
    R.spmv(1.0, bn, d["rowptr"].data_ptr(), d["colidx"].data_ptr(), d["values"].data_ptr(), xd.data_ptr(), 0.0,
           yr.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    R.close()
    A = SpMat(bn, 5, d["rowptr"], d["colidx"], d["values"], cuda=True)
    y = torch.zeros(bn * 5, dtype=torch.float64, device="cuda")
    A.mult(1.0, xd, 0.0, y, precision=PREC_FP64_FMA)
    ref = port.bsr_spmv(s, x)
    scale = np.abs(ref).max()
    assert np.abs(yr.cpu().numpy() - ref).max() <= 1e-13 * scale
    assert np.abs(y.cpu().numpy() - ref).max() <= 1e-13 * scale
