"""GPU parity of the block LU-SGS FlowSys path against the oracle, and the
mixed-precision (FP32 sweeps + FP64 refinement) solve to 1e-10."""
import numpy as np
import pytest
import torch

from tests.golden import cases

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def make(b, prec=0, on_device=False, colored=None, nvars=None):
    from ucfd_sparse_gb300.flowsys import FlowSys
    conv = dev if on_device else np.ascontiguousarray
    m = {k: conv(b[k]) for k in ("rowptr", "colidx", "slots", "sides", "face_area", "face_normal", "rcp_vol")}
    nv = b["nvars"] if nvars is None else nvars
    S = FlowSys(b["nlocal"], nv, b["nfvars"], 3, b["nfaces"], 1, m["rowptr"], m["colidx"], m["slots"], m["sides"],
                m["face_area"], m["face_normal"], m["rcp_vol"])
    if colored is not None:
        S.set_coloring(np.ascontiguousarray(colored, dtype=np.int32))
    S.set_precision(prec)
    e = dict(upts=conv(np.array(b["upts"])), rhs=conv(b["rhs"]), dt=conv(b["dt"]), ids=conv(b["cell_ids"]),
             vol=conv(b["vol"]), dsrc=conv(b.get("dsrc", np.zeros_like(b["rhs"]))),
             res=conv(np.zeros_like(b["rhs"])))
    S.set_element(0, b["neles"], 6, e["ids"], e["upts"], e["rhs"], e["dt"], e["dsrc"], e["vol"], e["res"])
    S.set_blusgs(conv(b["jmat"]), conv(b["tjmat"]) if "tjmat" in b else None)
    return S, e


def host(x):
    return x.cpu().numpy() if hasattr(x, "cpu") else x


def run_sweeps(S, nsweeps):
    S.blusgs_pack(0, 0.0)
    S.blusgs_ns_prepare()
    S.blusgs_reset()
    for _ in range(nsweeps):
        S.blusgs_ns_lower()
        S.blusgs_ns_upper()
        S.blusgs_sub_residual(0)
    S.blusgs_update(0)


@pytest.mark.parametrize("name", sorted(cases.BLUSGS))
@pytest.mark.parametrize("on_device", [False, True])
def test_blusgs_natural_order_bitexact(name, on_device, golden, ucfd):
    meta, arr = golden
    kw = cases.BLUSGS[name]
    b = cases.blusgs_case(**kw)
    S, e = make(b, on_device=on_device)
    run_sweeps(S, kw["nsweeps"])
    np.testing.assert_array_equal(host(e["upts"]), arr[f"{name}_upts"])
    np.testing.assert_array_equal(host(e["res"]), arr[f"{name}_resid"])


@pytest.mark.parametrize("name", sorted(cases.BLUSGS))
@pytest.mark.parametrize("prec", [0, 2])
def test_blusgs_pinned_jacobians_read_in_place(name, prec, golden, ucfd):
    """UCFD_HOST_MAP: face Jacobians in pinned host memory are read in place
    by the Prepare kernels; the other host arrays are staged.  FP64 gives the
    golden outputs bit for bit and every mode the staged run's values."""
    from ucfd_sparse_gb300 import lib
    meta, arr = golden
    kw = cases.BLUSGS[name]
    b = cases.blusgs_case(**kw)
    outs = {}
    mode0 = lib.host_array_access()
    assert mode0 == lib.HOST_MAP  # the default
    for mode in (lib.HOST_STAGE, lib.HOST_MAP):
        S, e = make(b, prec=prec)
        jm = torch.from_numpy(np.ascontiguousarray(b["jmat"])).pin_memory()
        S.set_blusgs(jm)
        lib.set_host_array_access(mode)
        try:
            assert lib.host_array_access() == mode
            run_sweeps(S, kw["nsweeps"])
        finally:
            lib.set_host_array_access(mode0)
        outs[mode] = (np.array(e["upts"]), np.array(e["res"]))
        S.destroy()
    for a, r in zip(outs[lib.HOST_MAP], outs[lib.HOST_STAGE]):
        np.testing.assert_array_equal(a, r)
    if prec == 0:
        np.testing.assert_array_equal(outs[lib.HOST_MAP][0], arr[f"{name}_upts"])
        np.testing.assert_array_equal(outs[lib.HOST_MAP][1], arr[f"{name}_resid"])
    with pytest.raises(lib.UCFDError):
        lib.set_host_array_access(2)


def test_blusgs_colored_equals_renumbered(port, ucfd):
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    b = cases.blusgs_case(m=9, seed=5)
    ic, rg, lc = cl.greedy_coloring_csr(b["rowptr"], b["colidx"])
    S, e = make(b, colored=lc)
    assert S.levels() == len(rg)
    run_sweeps(S, 3)
    new = np.empty(b["nlocal"], dtype=np.int64)
    new[ic] = np.arange(b["nlocal"])
    br = mg.renumber_flowsys(b, new)
    up, du, res, _ = port.flowsys_blusgs(br, b["rhs"], b["dt"], b["jmat"], b["vol"], b["upts"], nsweeps=3)
    np.testing.assert_array_equal(e["upts"], up)
    np.testing.assert_array_equal(e["res"], res)


def test_blusgs_fp64_fma_within_tolerance(golden, ucfd):
    meta, arr = golden
    b = cases.blusgs_case(**cases.BLUSGS["blu10"])
    S, e = make(b, prec=1, on_device=True)
    run_sweeps(S, 2)
    ref = arr["blu10_upts"]
    d = host(e["upts"]) - b["upts"]
    r = ref - b["upts"]
    assert np.abs(d - r).max() <= 1e-12 * np.abs(r).max()


SPLIT_ORDERS = {
    "lower_twice": "LLUULU",
    "upper_first": "ULUL",
    "prepare_between": "LUPLUL",
    "reset_between": "LURLU",
}


@pytest.mark.parametrize("order", sorted(SPLIT_ORDERS))
def test_blusgs_fast_sweeps_any_call_order(order, ucfd):
    """The fast build's sweeps reuse the face sums the opposite sweep stored
    only when they belong to the same increments and the same blocks.  Any
    order of lower (L) and upper (U) sweeps, Prepare (P) and Reset (R) gives
    the exact mode's values: the FMA mode within 1e-12 and FP32 within 1e-5
    of the largest change."""
    b = cases.blusgs_case(m=8, seed=7)
    outs = {}
    for prec in (0, 1, 2):
        S, e = make(b, prec=prec, on_device=True)
        S.blusgs_pack(0, 0.0)
        S.blusgs_ns_prepare()
        S.blusgs_reset()
        ops = {"L": S.blusgs_ns_lower, "U": S.blusgs_ns_upper, "P": S.blusgs_ns_prepare, "R": S.blusgs_reset}
        for op in SPLIT_ORDERS[order]:
            ops[op]()
        S.blusgs_update(0)
        outs[prec] = host(e["upts"]) - b["upts"]
        S.destroy()
    r = outs[0]
    scale = np.abs(r).max()
    assert scale > 0
    assert np.abs(outs[1] - r).max() <= 1e-12 * scale
    assert np.abs(outs[2] - r).max() <= 1e-5 * scale


def with_self_faces(b, ncells, seed=0):
    """The same system with a face from each of the first ncells boundary
    cells to the cell itself (a CSR entry naming its own row, with a face of
    its own), as legacy meshes list boundary faces."""
    rng = np.random.default_rng(seed)
    rp, ci, sl, sd = b["rowptr"], b["colidx"], b["slots"], b["sides"]
    n, nF, nv = b["nlocal"], b["nfaces"], b["jmat"].shape[1]
    rows = [i for i in range(n) if rp[i + 1] - rp[i] < 6][:ncells]
    nrp, nci, nsl, nsd = [0], [], [], []
    for i in range(n):
        q0, q1 = rp[i], rp[i + 1]
        nci += list(ci[q0:q1]); nsl += list(sl[q0:q1]); nsd += list(sd[q0:q1])
        if i in rows:
            nci.append(i); nsl.append(nF + rows.index(i)); nsd.append(1)
        nrp.append(len(nci))
    k = len(rows)
    c = dict(b)
    c["rowptr"] = np.array(nrp, dtype=np.int32)
    c["colidx"] = np.array(nci, dtype=np.int32)
    c["slots"] = np.array(nsl, dtype=np.int32)
    c["sides"] = np.array(nsd, dtype=np.int8)
    c["nfaces"] = nF + k
    c["face_area"] = np.concatenate([b["face_area"], rng.uniform(0.5, 1.0, k)])
    c["face_normal"] = np.concatenate([b["face_normal"], np.tile([[1.0], [0.0], [0.0]], (1, k))], axis=1)
    extra = rng.normal(0.0, 0.05, (2, nv, nv, k))
    for r in range(nv):
        extra[0, r, r] += 1.0
        extra[1, r, r] -= 1.0
    c["jmat"] = np.ascontiguousarray(np.concatenate([b["jmat"], extra], axis=3))
    return c


def test_blusgs_faces_to_the_cell_itself(port, ucfd):
    """A mesh with faces from a cell to itself: the exact mode matches the
    oracle bit for bit; the fast build sweeps in full mode (such a face's
    term changes with the cell's own increment) and stays within 1e-12 (FMA)
    of it, in lower-upper pairs and in other call orders."""
    b = with_self_faces(cases.blusgs_case(m=6, seed=2), ncells=12)
    for order in ("LULULU", "LULUUL"):
        outs = {}
        for prec in (0, 1):
            S, e = make(b, prec=prec, on_device=True)
            S.blusgs_pack(0, 0.0)
            S.blusgs_ns_prepare()
            S.blusgs_reset()
            for op in order:
                (S.blusgs_ns_lower if op == "L" else S.blusgs_ns_upper)()
            S.blusgs_update(0)
            outs[prec] = host(e["upts"])
            S.destroy()
        if order == "LULULU":
            ref = port.flowsys_blusgs(b, b["rhs"], b["dt"], b["jmat"], b["vol"], b["upts"], nsweeps=3)[0]
            np.testing.assert_array_equal(outs[0], ref)
        r = outs[0] - b["upts"]
        assert np.abs(r).max() > 0
        assert np.abs(outs[1] - outs[0]).max() <= 1e-12 * np.abs(r).max()


@pytest.mark.parametrize("prec", [0, 2])
def test_blusgs_solve_reaches_1e10(prec, port, ucfd):
    """Plain FP64 sweeps and FP32 sweeps + FP64 refinement both reach a
    1e-10 relative residual; their solutions agree with the oracle run to
    convergence."""
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    b = cases.blusgs_case(m=12, seed=1)
    ic, rg, lc = cl.greedy_coloring_csr(b["rowptr"], b["colidx"])
    S, e = make(b, prec=prec, on_device=True, colored=lc)
    S.blusgs_pack(0, 0.0)
    S.blusgs_ns_prepare()
    S.blusgs_reset()
    n, rel = S.blusgs_solve(1e-10, 400, 8)
    assert rel <= 1e-10, (n, rel)
    assert S.blusgs_residual() <= 1e-10
    S.blusgs_update(0)
    new = np.empty(b["nlocal"], dtype=np.int64)
    new[ic] = np.arange(b["nlocal"])
    br = mg.renumber_flowsys(b, new)
    up = port.flowsys_blusgs(br, b["rhs"], b["dt"], b["jmat"], b["vol"], b["upts"], nsweeps=n + 20)[0]
    dq = up - b["upts"]
    assert np.abs(host(e["upts"]) - up).max() <= 1e-8 * np.abs(dq).max()


def test_blusgs_turbulence_packs_and_sweeps(port, ucfd):
    """k-omega SST pack + RANS prepare/sweeps (blusgs.c:60-120, 260-270,
    388-429) on a 7-variable system against the oracle."""
    from oracle.oracle import P
    from ucfd_sparse_gb300 import meshgen as mg
    b = mg.blusgs_case(5, nvars=7, seed=3)
    b["nfvars"] = 5
    rng = np.random.default_rng(4)
    N, nF = b["nlocal"], b["nfaces"]
    b["upts"][5:] = rng.uniform(0.1, 1.0, (2, N))
    b["dsrc"] = rng.uniform(0.0, 1.0, (7, N))
    t = rng.normal(0.0, 0.05, (2, 2, 2, nF))
    t[0, 0, 0] += 1.0; t[0, 1, 1] += 1.0; t[1, 0, 0] -= 1.0; t[1, 1, 1] -= 1.0
    b["tjmat"] = t
    b["jmat"] = np.ascontiguousarray(b["jmat"][:, :5, :5])
    S, e = make(b)
    S.blusgs_pack(0, 0.0)
    S.blusgs_kwsst_pack(0, 1.5, 0.3)
    S.blusgs_ns_prepare()
    S.blusgs_rans_prepare()
    S.blusgs_reset()
    for _ in range(2):
        S.blusgs_ns_lower(); S.blusgs_ns_upper()
        S.blusgs_rans_lower(); S.blusgs_rans_upper()
    S.blusgs_update(0)
    # oracle
    L = port.L
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    rp, ci, sl = i32(b["rowptr"]), i32(b["colidx"]), i32(b["slots"])
    sd = np.ascontiguousarray(b["sides"], dtype=np.int8)
    fa, rv, ids = f64(b["face_area"]), f64(b["rcp_vol"]), i32(b["cell_ids"])
    rhs, dt, up0, ds = f64(b["rhs"]), f64(b["dt"]), f64(b["upts"]), f64(b["dsrc"])
    jm, tj = f64(b["jmat"]), f64(t)
    rr, dg, tdg = np.zeros(N * 7), np.zeros(N * 25), np.zeros(N * 4)
    du = np.zeros(N * 7)
    upts = up0.copy()
    L.oracle_blusgs_pack(N, N, 7, 5, 0.0, P(ids), P(rhs), P(dt), P(rr), P(dg))
    L.oracle_tblusgs_pack(0, N, N, 7, 5, 0.3, 1.5, P(ids), P(up0), P(ds), P(dt), P(tdg))
    L.oracle_blusgs_prepare(N, 5, nF, P(rp), P(sl), P(sd), P(fa), P(rv), P(dg), P(jm))
    L.oracle_blusgs_prepare(N, 2, nF, P(rp), P(sl), P(sd), P(fa), P(rv), P(tdg), P(tj))
    for _ in range(2):
        for fn in (L.oracle_blusgs_lower, L.oracle_blusgs_upper):
            fn(0, 5, N, 7, nF, P(rp), P(ci), P(sd), P(sl), P(fa), P(rv), P(rr), P(dg), P(jm), P(du))
        for fn in (L.oracle_blusgs_lower, L.oracle_blusgs_upper):
            fn(5, 2, N, 7, nF, P(rp), P(ci), P(sd), P(sl), P(fa), P(rv), P(rr), P(tdg), P(tj), P(du))
    L.oracle_blusgs_update(N, N, 7, P(ids), P(du), P(upts))
    np.testing.assert_array_equal(e["upts"], upts)


def test_transfer_timing_counts_host_copies(ucfd):
    """UCFDSetTransferTiming / UCFDGetTransferStats: a step on host arrays
    counts the staged inputs (at least the face Jacobians) and the state
    copied back; timing off leaves the counters alone."""
    from ucfd_sparse_gb300 import lib
    b = cases.blusgs_case(m=6, seed=2)
    S, e = make(b)
    lib.transfer_timing(True)
    run_sweeps(S, 1)
    st = lib.transfer_stats()
    lib.transfer_timing(False)
    assert st["h2d_bytes"] >= b["jmat"].nbytes and st["h2d_copies"] >= 1 and st["h2d_ms"] > 0
    assert st["d2h_bytes"] >= b["upts"].nbytes and st["d2h_copies"] >= 1
    run_sweeps(S, 1)
    assert lib.transfer_stats() == st
