"""The oracle (oracle/ucfd_oracle.c) against the reference's own outputs.

Golden vectors were produced by the reference library compiled from its
sources (tests/golden/make_golden.py); the restatement must reproduce them
bit for bit.  Where the reference source tree is present, the oracle is
also compared with the freshly compiled reference on extra cases.
"""
import hashlib

import numpy as np
import pytest

from oracle import oracle as orc
from tests.golden import cases


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", sorted(cases.LEGACY))
def test_legacy_colored_matches_reference(name, golden, port):
    meta, arr = golden
    kw = cases.LEGACY[name]
    c, icolor, ranges, lcolor = cases.legacy_case(**kw)
    assert cases.input_hash(c) == meta[f"{name}_in"], "synthetic inputs drifted"
    nfv = 5
    up = port.legacy_step(c, icolor, ranges, lcolor, nsteps=kw["nsteps"], nfvars=nfv)[0]
    if kw.get("nvars", 5) > 5:
        # the reference FlowSys update adds every variable; the colored NS
        # step leaves the turbulence rows untouched, their du being rhs
        for _ in range(kw["nsteps"]):
            up[5:] += c["rhs"][5:]
    assert sha(up) == meta[f"{name}_upts_sha"]
    if f"{name}_upts" in arr.files:
        np.testing.assert_array_equal(up, arr[f"{name}_upts"])


@pytest.mark.parametrize("name", sorted(cases.FLOWSYS))
def test_flowsys_scalar_matches_reference(name, golden, port):
    meta, arr = golden
    kw = cases.FLOWSYS[name]
    fs, inp = cases.flowsys_case(**kw)
    assert cases.input_hash(inp) == meta[f"{name}_in"]
    up = port.flowsys_lusgs_step(fs, inp["upts"], inp["rhs"], inp["dt"], inp["dsrc"], inp["fspr"], inp["tfspr"],
                                 kappa=kw["kappa"], a0=kw["a0"], turb_factor=kw["turb_factor"], rans=True,
                                 nsteps=kw["nsteps"])[0]
    np.testing.assert_array_equal(up, arr[f"{name}_upts"])
    assert sha(up) == meta[f"{name}_upts_sha"]


@pytest.mark.parametrize("name", sorted(cases.BLUSGS))
def test_blusgs_matches_reference(name, golden, port):
    meta, arr = golden
    kw = cases.BLUSGS[name]
    b = cases.blusgs_case(**kw)
    up, du, res, _ = port.flowsys_blusgs(b, b["rhs"], b["dt"], b["jmat"], b["vol"], b["upts"], nsweeps=kw["nsweeps"])
    np.testing.assert_array_equal(up, arr[f"{name}_upts"])
    np.testing.assert_array_equal(res, arr[f"{name}_resid"])


@pytest.mark.parametrize("name", sorted(cases.KRYLOV))
def test_krylov_matches_reference(name, golden, port):
    meta, arr = golden
    kw = cases.KRYLOV[name]
    s = cases.bsr_case(**kw)
    assert cases.input_hash({k: s[k] for k in ("values", "rowptr", "colidx", "rhs")}) == meta[f"{name}_in"]
    x = cases.spmv_x(s)
    np.testing.assert_array_equal(port.bsr_spmv(s, x, 1.5, -0.5, x), arr[f"{name}_spmv"])
    g = meta[f"{name}_gmres"]
    xs, st, it, res, _ = port.gmres(s, s["rhs"], m=kw["m"], maxiter=20, tol=g["tol"])
    assert (st, it) == (g["stat"], g["iters"])
    # hypot/sqrt of libm may differ in the last bit between platforms
    np.testing.assert_allclose(xs, arr[f"{name}_gmres_x"], rtol=0, atol=1e-13 * np.abs(xs).max())
    assert res == pytest.approx(g["resid"], rel=1e-6, abs=1e-14)


def test_legacy_serial_equals_natural_flowsys(port):
    """The natural-order array sweeps equal the colored sweeps with one
    colour per cell (lusgs.c:184,236)."""
    c = cases.legacy_case(m=5, jitter=0.2, permute=True, coloring="greedy", nsteps=1)[0]
    up_s = port.legacy_serial_step(c)[0]
    N = c["neles"]
    ident = np.arange(N, dtype=np.int32)
    up_c = port.legacy_step(c, ident, list(range(1, N + 1)), ident + 1)[0]
    np.testing.assert_array_equal(up_s, up_c)


def test_pblusgs_equals_natural_on_colour_ordered_matrix(port):
    """Coloured BLU-SGS over contiguous colour ranges equals the natural
    order BLU-SGS of the colour-renumbered matrix (pblusgs.c with the diagonal
    block index fixed)."""
    from ucfd_sparse_gb300 import meshgen as mg
    s = mg.bsr_case(3, seed=3)
    icolor, ranges, lcolor = mg.greedy_coloring_np(np.where(s["nei"] >= 0, s["nei"],
                                                            np.arange(s["bn"])[None, :]))
    new = np.empty(s["bn"], dtype=np.int64)
    new[icolor] = np.arange(s["bn"])
    sc = mg.renumber_bsr(s, new)
    b = np.random.default_rng(2).standard_normal(sc["bn"] * 5)
    a = port.precon_apply(sc, b)
    c = port.precon_apply(sc, b, icolors=[0] + ranges)
    np.testing.assert_array_equal(a, c)


def test_blusgs_phases_equal_whole_step(port):
    """The call-by-call BLU-SGS driver the CPU timing legs use performs the
    same step as flowsys_blusgs (and, where the reference was compiled here,
    as the reference's own calls)."""
    b = cases.blusgs_case(m=6, seed=4)
    whole = port.flowsys_blusgs(b, b["rhs"], b["dt"], b["jmat"], b["vol"], b["upts"], nsweeps=3)
    impls = [port] + ([orc.Ref()] if orc.ref_available() else [])
    for impl in impls:
        ph = impl.blusgs_phases(b, b["rhs"], b["dt"], b["jmat"], b["vol"], b["upts"])
        ph.pack_prepare()
        ph.reset()
        for _ in range(3):
            ph.lower()
            ph.upper()
            ph.sub_residual()
        ph.update()
        np.testing.assert_array_equal(ph.upts, whole[0])
        np.testing.assert_array_equal(ph.res, whole[2])
        ph.close()


@pytest.mark.skipif(not orc.ref_available(), reason="reference source tree not present on this machine")
def test_port_vs_compiled_reference_extra(port):
    ref = orc.Ref()
    for m, jit, perm in [(7, 0.2, True), (16, 0.0, False)]:
        c, icolor, ranges, lcolor = cases.legacy_case(m=m, jitter=jit, permute=perm,
                                                      coloring="greedy" if perm else "checker", nsteps=2)
        up = port.legacy_step(c, icolor, ranges, lcolor, nsteps=2)[0]
        fs = orc.legacy_to_flowsys(c, icolor)
        upr = ref.flowsys_lusgs_step(fs, c["upts"], c["rhs"], c["dt"], np.zeros_like(c["rhs"]), fs["fspr"], nsteps=2)
        np.testing.assert_array_equal(up, upr)
    b = cases.blusgs_case(m=7, seed=9)
    a = port.flowsys_blusgs(b, b["rhs"], b["dt"], b["jmat"], b["vol"], b["upts"], nsweeps=4)
    r = ref.flowsys_blusgs(b, b["rhs"], b["dt"], b["jmat"], b["vol"], b["upts"], nsweeps=4)
    np.testing.assert_array_equal(a[0], r[0])
    np.testing.assert_array_equal(a[2], r[1])


@pytest.mark.parametrize("name", sorted(cases.KRYLOV))
def test_bilu_bicgstab_match_reference(name, golden, port):
    """Block ILU(0) factors (bilu.c) bit for bit; BiCGSTAB (bicgstab.c) with
    the BLU-SGS and the BILU preconditioner: same status, iteration count,
    solution and residual history as the reference."""
    meta, arr = golden
    s = cases.bsr_case(**cases.KRYLOV[name])
    fv = port.bilu_factor(s)
    assert cases.sha(fv) == meta[f"{name}_bilu_sha"]
    for pc in ("blusgs", "bilu"):
        g = meta[f"{name}_bicgstab_{pc}"]
        x, st, it, res, hist = port.bicgstab(s, s["rhs"], maxiter=20, tol=g["tol"], pc=pc)
        assert (st, it) == (g["stat"], g["iters"])
        np.testing.assert_array_equal(x, arr[f"{name}_bicgstab_{pc}_x"])
        np.testing.assert_allclose(hist[:it + 1], g["hist"], rtol=1e-14)


def test_pbilu_equals_natural_on_colour_ordered_matrix(port):
    """Coloured block ILU(0) (pbilu.c) equals the natural-order one on a
    colour-renumbered matrix: rows of one colour never reference each other."""
    from ucfd_sparse_gb300 import meshgen as mg
    s = mg.bsr_case(4, seed=5)
    icolor, ranges, lcolor = mg.greedy_coloring_np(np.where(s["nei"] >= 0, s["nei"],
                                                            np.arange(s["bn"])[None, :]))
    new = np.empty(s["bn"], dtype=np.int64)
    new[icolor] = np.arange(s["bn"])
    sc = mg.renumber_bsr(s, new)
    fv = port.bilu_factor(sc)
    if orc.ref_available():
        np.testing.assert_array_equal(fv, orc.Ref().ilu_factor(sc, "pbilu", [0] + [int(r) for r in ranges]))


def test_ilu_apply_inverts_its_factors(port):
    """Scalar ILU(0): the factors match the reference (ilu.c prepare) and
    the restated apply -- with the diagonal slot left out of the backward
    loop, unlike ilu.c:81 -- solves (L U) y = b exactly up to rounding."""
    from ucfd_sparse_gb300 import meshgen as mg
    s = mg.bsr_case(4, seed=6)
    ss = dict(s, blk=1, values=np.ascontiguousarray(np.asarray(s["values"]).reshape(-1, 5, 5)[:, 0, 0]))
    fv = port.ilu_factor(ss)
    if orc.ref_available():
        np.testing.assert_array_equal(fv, orc.Ref().ilu_factor(ss, "ilu"))
    n = ss["bn"]
    rp, ci, ds = ss["rowptr"], ss["colidx"], ss["diagslots"]
    Lm = np.eye(n)
    Um = np.zeros((n, n))
    for i in range(n):
        for j in range(rp[i], rp[i + 1]):
            if j < ds[i]:
                Lm[i, ci[j]] = fv[j]
            else:
                Um[i, ci[j]] = fv[j]
    y = np.random.default_rng(1).standard_normal(n)
    np.testing.assert_allclose(port.ilu_apply(ss, fv, Lm @ (Um @ y)), y, rtol=1e-10, atol=1e-12)
