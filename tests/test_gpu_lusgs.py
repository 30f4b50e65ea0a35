"""GPU parity of the scalar LU-SGS path (array API and FlowSys API) against
the oracle, through the C-ABI.  FP64 mode (no FMA contraction) must be
bit-identical; the FMA mode within 1e-12 (relative to max |value|)."""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.golden import cases

pytestmark = pytest.mark.gpu

REL_FMA = 1e-12


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def rel_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def run_colored_gpu(c, icolor, ranges, lcolor, nsteps, on_device, rans=False):
    from ucfd_sparse_gb300 import coloredlusgs as cl
    N = c["neles"]
    arrs = dict(nei_ele=c["nei_ele"].astype(np.int32), fnorm_vol=c["fnorm_vol"], vec_fnorm=c["vec_fnorm"],
                fspr=c["fspr"], dt=c["dt"], upts=c["upts"].copy(), rhs=c["rhs"].copy(), lcolor=lcolor)
    if on_device:
        arrs = {k: dev(v) for k, v in arrs.items()}
        ic = dev(icolor.astype(np.int32))
        diag = torch.zeros(N, dtype=torch.float64, device="cuda")
        dub = torch.zeros_like(arrs["rhs"])
    else:
        arrs = {k: np.ascontiguousarray(v) for k, v in arrs.items()}
        ic = icolor.astype(np.int32)
        diag = np.zeros(N)
        dub = np.zeros_like(c["rhs"])
    cc = dict(c, **arrs)
    for _ in range(nsteps):
        if on_device:
            arrs["rhs"].copy_(dev(c["rhs"]))
        else:
            arrs["rhs"][:] = c["rhs"]
        cl.colored_step(cc, ic, ranges, diag, dub, rans=rans)
    out = arrs["upts"]
    return out.cpu().numpy() if on_device else out


@pytest.mark.parametrize("name", sorted(cases.LEGACY))
@pytest.mark.parametrize("on_device", [True, False])
def test_colored_step_bitexact(name, on_device, port, ucfd):
    from ucfd_sparse_gb300 import coloredlusgs as cl
    kw = cases.LEGACY[name]
    c, icolor, ranges, lcolor = cases.legacy_case(**kw)
    cl.set_dims(c["nvars"], 5, 3)
    cl.set_precision(0)
    try:
        up = run_colored_gpu(c, icolor, ranges, lcolor, kw["nsteps"], on_device)
    finally:
        cl.set_dims(5, 5, 3)
    ref = port.legacy_step(c, icolor, ranges, lcolor, nsteps=kw["nsteps"])[0]
    np.testing.assert_array_equal(up, ref)


def test_colored_step_fma_mode_within_tolerance(port, ucfd):
    from ucfd_sparse_gb300 import coloredlusgs as cl
    c, icolor, ranges, lcolor = cases.legacy_case(**cases.LEGACY["leg32"])
    cl.set_precision(1)
    try:
        up = run_colored_gpu(c, icolor, ranges, lcolor, 10, True)
    finally:
        cl.set_precision(0)
    ref = port.legacy_step(c, icolor, ranges, lcolor, nsteps=10)[0]
    assert rel_err(up - c["upts"], ref - c["upts"]) < REL_FMA


def test_rans_colored_sweeps_bitexact(port, ucfd):
    from ucfd_sparse_gb300 import coloredlusgs as cl
    c, icolor, ranges, lcolor = cases.legacy_case(m=7, jitter=0.2, permute=True, coloring="greedy", nsteps=1,
                                                  nvars=6)
    cl.set_dims(6, 5, 3)
    try:
        up = run_colored_gpu(c, icolor, ranges, lcolor, 2, True, rans=True)
    finally:
        cl.set_dims(5, 5, 3)
    ref = port.legacy_step(c, icolor, ranges, lcolor, nsteps=2, rans=True)[0]
    np.testing.assert_array_equal(up, ref)


def test_serial_sweeps_bitexact(port, ucfd):
    """Natural-order array sweeps: level-scheduled on the GPU, identical to
    the sequential reference."""
    from ucfd_sparse_gb300 import coloredlusgs as cl
    c = cases.legacy_case(m=9, jitter=0.2, permute=True, coloring="greedy", nsteps=1)[0]
    N, nf = c["neles"], 6
    upts, rhs = c["upts"].copy(), c["rhs"].copy()
    dub, diag = np.zeros_like(rhs), np.zeros(N)
    nei = c["nei_ele"].astype(np.int32)
    cl.serial_pre_lusgs(N, nf, 1.0, c["fnorm_vol"], c["dt"], diag, c["fspr"])
    cl.ns_serial_lower_sweep(N, nf, nei, c["fnorm_vol"], c["vec_fnorm"], upts, rhs, dub, diag, c["fspr"])
    cl.ns_serial_upper_sweep(N, nf, nei, c["fnorm_vol"], c["vec_fnorm"], upts, rhs, dub, diag, c["fspr"])
    cl.lusgs_serial_ns_update(N, upts, rhs)
    ref = port.legacy_serial_step(c)
    np.testing.assert_array_equal(diag, ref[3])
    np.testing.assert_array_equal(dub, ref[2])
    np.testing.assert_array_equal(upts, ref[0])


def test_c_example_inplace_aliases(port, ucfd):
    """parallel_ns_* without rhs (omp3d.c:181-189): dub read and written in
    place, i.e. the FlowSys in-place form."""
    from ucfd_sparse_gb300 import lib
    c, icolor, ranges, lcolor = cases.legacy_case(**cases.LEGACY["legjp6"])
    N, nf = c["neles"], 6
    L = lib.load()
    upts, dub, diag = c["upts"].copy(), c["rhs"].copy(), np.zeros(N)
    nei = c["nei_ele"].astype(np.int32)
    P = lib.ptr
    lib.call_void("parallel_pre_lusgs", N, nf, 1.0, P(c["fnorm_vol"]), P(c["dt"]), P(diag), P(c["fspr"]))
    b = [0] + ranges
    for k in range(len(ranges)):
        lib.call_void("parallel_ns_lower_sweep", b[k], b[k + 1], N, nf, P(nei), P(icolor), P(lcolor),
                      P(c["fnorm_vol"]), P(c["vec_fnorm"]), P(upts), P(dub), P(diag), P(c["fspr"]))
    for k in reversed(range(len(ranges))):
        lib.call_void("parallel_ns_upper_sweep", b[k], b[k + 1], N, nf, P(nei), P(icolor), P(lcolor),
                      P(c["fnorm_vol"]), P(c["vec_fnorm"]), P(upts), P(dub), P(diag), P(c["fspr"]))
    lib.call_void("lusgs_parallel_ns_update", N, P(upts), P(dub))
    # oracle: same arithmetic with rhs aliased to dub
    o = port.L
    u2, d2, g2 = c["upts"].copy(), c["rhs"].copy(), np.zeros(N)
    fnv, vec, fs, dt = [np.ascontiguousarray(c[k]) for k in ("fnorm_vol", "vec_fnorm", "fspr", "dt")]
    Q = orc.P
    o.oracle_legacy_pre(N, nf, 1.0, Q(fnv), Q(dt), Q(g2), Q(fs))
    for k in range(len(ranges)):
        o.oracle_legacy_sweep(0, 0, b[k], b[k + 1], N, nf, 5, 5, 3, Q(nei), Q(icolor), Q(lcolor), Q(fnv), Q(vec),
                              Q(u2), Q(d2), Q(d2), Q(g2), Q(fs))
    for k in reversed(range(len(ranges))):
        o.oracle_legacy_sweep(1, 0, b[k], b[k + 1], N, nf, 5, 5, 3, Q(nei), Q(icolor), Q(lcolor), Q(fnv), Q(vec),
                              Q(u2), Q(d2), Q(d2), Q(g2), Q(fs))
    o.oracle_legacy_update(0, N, 5, 5, Q(u2), Q(d2))
    np.testing.assert_array_equal(upts, u2)


def test_edge_cases_and_errors(ucfd):
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import lib
    c, icolor, ranges, lcolor = cases.legacy_case(**cases.LEGACY["leg8"])
    N = c["neles"]
    dub, diag = np.zeros_like(c["rhs"]), np.ones(N)
    before = dub.copy()
    # empty colour range: no-op
    cl.ns_parallel_lower_sweep(5, 5, N, 6, c["nei_ele"], icolor, lcolor, c["fnorm_vol"], c["vec_fnorm"],
                               c["upts"], c["rhs"], dub, diag, c["fspr"])
    np.testing.assert_array_equal(dub, before)
    # reversed range -> error status, nothing written
    with pytest.raises(lib.UCFDError):
        cl.ns_parallel_lower_sweep(6, 5, N, 6, c["nei_ele"], icolor, lcolor, c["fnorm_vol"], c["vec_fnorm"],
                                   c["upts"], c["rhs"], dub, diag, c["fspr"])
    np.testing.assert_array_equal(dub, before)
    # unsupported variable count
    with pytest.raises(lib.UCFDError):
        cl.set_dims(9, 5, 3)
    # one-cell mesh (all faces point to itself)
    one = dict(neles=1, nface=6, nvars=5, nei_ele=np.zeros((6, 1), np.int32), fnorm_vol=np.ones((6, 1)),
               vec_fnorm=np.zeros((6, 3, 1)), fspr=np.ones((6, 1)), dt=np.array([0.1]),
               upts=c["upts"][:, :1].copy(), rhs=np.ones((5, 1)), lcolor=np.ones(1, np.int32))
    d1, g1 = np.zeros((5, 1)), np.zeros(1)
    cl.colored_step(one, np.zeros(1, np.int32), [1], g1, d1)
    assert g1[0] == 1 / 0.1 + 3.0
    np.testing.assert_array_equal(one["rhs"][:, 0], np.full(5, 1 / g1[0]))


# ---- FlowSys scalar LU-SGS --------------------------------------------------
def make_flowsys(fs, inp, prec=0, on_device=False, colored=None):
    from ucfd_sparse_gb300.flowsys import FlowSys
    conv = dev if on_device else np.ascontiguousarray
    m = {k: conv(fs[k]) for k in ("rowptr", "colidx", "slots", "sides", "face_area", "face_normal", "rcp_vol")}
    S = FlowSys(fs["nlocal"], fs["nvars"], fs["nfvars"], 3, fs["nfaces"], 1, m["rowptr"], m["colidx"], m["slots"],
                m["sides"], m["face_area"], m["face_normal"], m["rcp_vol"])
    if colored is not None:
        S.set_coloring(np.ascontiguousarray(colored, dtype=np.int32))
    S.set_precision(prec)
    e = {k: conv(inp[k]) for k in ("upts", "rhs", "dt", "dsrc")}
    e["upts"] = conv(np.array(inp["upts"]))
    e["ids"] = conv(fs["cell_ids"].astype(np.int32))
    e["vol"] = conv(np.ones(inp["dt"].shape[0]))
    e["res"] = conv(np.zeros_like(inp["upts"]))
    S.set_element(0, inp["dt"].shape[0], 6, e["ids"], e["upts"], e["rhs"], e["dt"], e["dsrc"], e["vol"], e["res"])
    S.set_lusgs(conv(inp["fspr"]), conv(inp["tfspr"]))
    return S, e


def flowsys_step(S, kw, nsteps):
    for _ in range(nsteps):
        S.lusgs_pack(0, kw["turb_factor"], kw["a0"])
        S.lusgs_ns_prepare(kw["kappa"])
        S.lusgs_ns_lower(kw["kappa"])
        S.lusgs_ns_upper(kw["kappa"])
        S.lusgs_rans_prepare(kw["kappa"])
        S.lusgs_rans_lower(kw["kappa"])
        S.lusgs_rans_upper(kw["kappa"])
        S.lusgs_update(0)


@pytest.mark.parametrize("name", sorted(cases.FLOWSYS))
@pytest.mark.parametrize("on_device", [False, True])
def test_flowsys_natural_order_bitexact(name, on_device, golden, port, ucfd):
    meta, arr = golden
    kw = cases.FLOWSYS[name]
    fs, inp = cases.flowsys_case(**kw)
    S, e = make_flowsys(fs, inp, on_device=on_device)
    assert S.levels() > 2
    flowsys_step(S, kw, kw["nsteps"])
    up = e["upts"].cpu().numpy() if on_device else e["upts"]
    np.testing.assert_array_equal(up, arr[f"{name}_upts"])


def test_flowsys_fp32_mode_error_bounded(port, ucfd):
    kw = cases.FLOWSYS["fs9"]
    fs, inp = cases.flowsys_case(**kw)
    ref = port.flowsys_lusgs_step(fs, inp["upts"], inp["rhs"], inp["dt"], inp["dsrc"], inp["fspr"], inp["tfspr"],
                                  rans=True)[0]
    S, e = make_flowsys(fs, inp, prec=2, on_device=True)
    flowsys_step(S, kw, 1)
    up = e["upts"].cpu().numpy()
    assert rel_err(up - inp["upts"], ref - inp["upts"]) < 1e-5


def test_flowsys_colored_equals_renumbered_natural(port, ucfd):
    """SetColoring sweeps colour by colour; equal to the natural order of the
    colour-renumbered mesh, bit for bit."""
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    kw = cases.FLOWSYS["fs9"]
    fs, inp = cases.flowsys_case(**kw)
    ic, rg, lc = cl.greedy_coloring_csr(fs["rowptr"], fs["colidx"])
    S, e = make_flowsys(fs, inp, colored=lc)
    assert S.levels() == len(rg)
    flowsys_step(S, kw, 1)
    new = np.empty(fs["nlocal"], dtype=np.int64)
    new[ic] = np.arange(fs["nlocal"])
    fr = mg.renumber_flowsys(fs, new)
    ref = port.flowsys_lusgs_step(fr, inp["upts"], inp["rhs"], inp["dt"], inp["dsrc"], inp["fspr"], inp["tfspr"],
                                  kappa=kw["kappa"], a0=kw["a0"], turb_factor=kw["turb_factor"], rans=True)[0]
    np.testing.assert_array_equal(e["upts"], ref)


def test_flowsys_invalid_colouring_rejected(ucfd):
    from ucfd_sparse_gb300 import lib
    fs, inp = cases.flowsys_case(**cases.FLOWSYS["fs5"])
    S, e = make_flowsys(fs, inp, colored=np.zeros(fs["nlocal"], np.int32))
    with pytest.raises(lib.UCFDError) as ex:
        S.lusgs_pack(0, 1.0, 0.0)
    assert ex.value.status == 2 and "colour" in str(ex.value)


@pytest.mark.parametrize("name", sorted(cases.FLOWSYS))
@pytest.mark.parametrize("mode", [0, 1])
def test_flowsys_run_loop_bitexact(name, mode, golden, ucfd):
    """UCFDLUSGS_Run with the turbulence system, FP64 mode, equals the
    reference's Pack / NSPrepare / NS lower / NS upper / RANSPrepare / RANS
    lower / RANS upper / Update repeated (the golden outputs) bit for bit.
    With one thread per cell the loop prepares both systems in one kernel
    and sweeps both in one launch per level (graph, mode 0) or in one
    cooperative launch per sweep (mode 1)."""
    meta, arr = golden
    kw = cases.FLOWSYS[name]
    fs, inp = cases.flowsys_case(**kw)
    S, e = make_flowsys(fs, inp, prec=0, on_device=True)
    S.set_launch_config(threads_per_block=128, sweep_variant=0, run_mode=mode)
    S.lusgs_pack(0, kw["turb_factor"], kw["a0"])
    S.lusgs_run(kw["nsteps"], kw["kappa"], rans=True, mode=mode)
    S.lusgs_update(0)
    np.testing.assert_array_equal(e["upts"].cpu().numpy(), arr[f"{name}_upts"])


@pytest.mark.parametrize("name", sorted(cases.FLOWSYS))
@pytest.mark.parametrize("variant", [0, 3])
def test_nsrans_calls_bitexact(name, variant, golden, ucfd):
    """NSRANSPrepare / NSRANSLowerSweep / NSRANSUpperSweep in place of the
    six NS and RANS calls: the golden outputs bit for bit, with the one-pass
    kernel (variant 0) and with the two sweeps one after the other
    (variant 3, two threads per cell)."""
    meta, arr = golden
    kw = cases.FLOWSYS[name]
    fs, inp = cases.flowsys_case(**kw)
    S, e = make_flowsys(fs, inp, prec=0, on_device=True)
    S.set_launch_config(threads_per_block=128, sweep_variant=variant)
    for _ in range(kw["nsteps"]):
        S.lusgs_pack(0, kw["turb_factor"], kw["a0"])
        S.lusgs_nsrans_prepare(kw["kappa"])
        S.lusgs_nsrans_lower(kw["kappa"])
        S.lusgs_nsrans_upper(kw["kappa"])
        S.lusgs_update(0)
    np.testing.assert_array_equal(e["upts"].cpu().numpy(), arr[f"{name}_upts"])


@pytest.mark.parametrize("prec", [1, 2])
def test_nsrans_calls_equal_separate_calls(prec, ucfd):
    """In the fast modes too, NSRANSPrepare / NSRANSLowerSweep /
    NSRANSUpperSweep (in FP32 on the packed per cell-face geometry and
    spectral radii) give the values of the six NS and RANS calls, bit for
    bit, also when a separate NSPrepare comes in between."""
    kw = cases.FLOWSYS["fs5"]
    fs, inp = cases.flowsys_case(**kw)
    outs = []
    for calls in ("both", "separate", "both_after_ns"):
        S, e = make_flowsys(fs, inp, prec=prec, on_device=True)
        S.set_launch_config(threads_per_block=128, sweep_variant=0)
        for _ in range(2):
            S.lusgs_pack(0, kw["turb_factor"], kw["a0"])
            if calls == "separate":
                S.lusgs_ns_prepare(kw["kappa"])
                S.lusgs_rans_prepare(kw["kappa"])
                S.lusgs_ns_lower(kw["kappa"])
                S.lusgs_ns_upper(kw["kappa"])
                S.lusgs_rans_lower(kw["kappa"])
                S.lusgs_rans_upper(kw["kappa"])
            else:
                S.lusgs_nsrans_prepare(kw["kappa"])
                if calls == "both_after_ns":
                    # a separate Prepare afterwards re-gathers one system's
                    # radii: the packed copy must not be used for the next sweeps
                    S.lusgs_pack(0, kw["turb_factor"], kw["a0"])
                    S.lusgs_ns_prepare(kw["kappa"])
                    S.lusgs_rans_prepare(kw["kappa"])
                S.lusgs_nsrans_lower(kw["kappa"])
                S.lusgs_nsrans_upper(kw["kappa"])
            S.lusgs_update(0)
        outs.append(e["upts"].cpu().numpy())
        S.destroy()
    assert np.abs(outs[0] - inp["upts"]).max() > 0
    np.testing.assert_array_equal(outs[0], outs[1])
    np.testing.assert_array_equal(outs[2], outs[1])


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_run_loop_both_systems_equal_separate_sweeps(prec, ucfd):
    """The loop's one-pass sweeps of both systems (one thread per cell:
    launch variants 0-2) give the values of the separate mean-flow and
    turbulence sweeps (two threads per cell, variant 3, one system after the
    other), state and residual history alike, in every arithmetic."""
    kw = cases.FLOWSYS["fs5"]
    fs, inp = cases.flowsys_case(**kw)
    outs = []
    for var in (0, 1, 2, 3):
        S, e = make_flowsys(fs, inp, prec=prec, on_device=True)
        S.set_launch_config(threads_per_block=64, sweep_variant=var)
        S.lusgs_pack(0, kw["turb_factor"], kw["a0"])
        res = np.zeros(3)
        S.lusgs_run(3, kw["kappa"], rans=True, mode=0, resid=res)
        S.lusgs_update(0)
        outs.append((e["upts"].cpu().numpy(), res))
    assert np.all(np.isfinite(outs[0][1])) and outs[0][1][0] > 0
    assert np.abs(outs[0][0] - inp["upts"]).max() > 0
    for up, res in outs[1:]:
        np.testing.assert_array_equal(up, outs[0][0])
        np.testing.assert_array_equal(res, outs[0][1])


def test_flowsys_run_graph_matches_steps(ucfd):
    """UCFDLUSGS_Run (CUDA graph, device-resident) equals the same number of
    explicit Pack-free iterations driven through the API."""
    fs, inp = cases.flowsys_case(**cases.FLOWSYS["fs9"])
    kw = dict(kappa=1.0, a0=0.0, turb_factor=1.0)
    S, e = make_flowsys(fs, inp, prec=2, on_device=True)
    S.lusgs_pack(0, 1.0, 0.0)
    res = np.zeros(5)
    S.lusgs_run(5, 1.0, rans=True, mode=0, resid=res)
    S.lusgs_update(0)
    a = e["upts"].cpu().numpy()
    S2, e2 = make_flowsys(fs, inp, prec=2, on_device=True)
    S2.lusgs_pack(0, 1.0, 0.0)
    res2 = np.zeros(5)
    S2.lusgs_run(5, 1.0, rans=True, mode=1, resid=res2)
    S2.lusgs_update(0)
    np.testing.assert_array_equal(a, e2["upts"].cpu().numpy())
    np.testing.assert_array_equal(res, res2)
    assert np.all(np.isfinite(res)) and res[0] > 0
