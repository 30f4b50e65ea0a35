"""Launch autotuner (UCFDFlowSysAutotune): every candidate gives the same
results, tuning leaves the system's state untouched, and the JSON cache
round-trips."""
import numpy as np
import pytest

from tests.golden import cases
from tests.test_gpu_blusgs import host, make, run_sweeps
from tests.test_gpu_lusgs import make_flowsys

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [0, 2])
def test_blusgs_launch_choices_bit_identical(prec, ucfd):
    """Block sizes 64/256 and both sweep variants give bit-identical
    solutions (same operations in the same order per cell)."""
    b = cases.blusgs_case(m=10, seed=2)
    outs = []
    # variants 2 and 3 (bulk copies into shared memory) are FP32-only; the
    # FP64 systems run the register kernel for them
    for tpb, var in ((64, 0), (256, 0), (64, 1), (256, 1), (0, 2), (0, 3), (64, 4), (256, 4)):
        S, e = make(b, prec=prec, on_device=True)
        S.set_launch_config(threads_per_block=tpb, sweep_variant=var)
        run_sweeps(S, 3)
        outs.append(host(e["upts"]))
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])


def test_bulk_sweep_partial_tiles_and_levels(port, ucfd):
    """Natural-order schedule: many levels whose cell ranges start and end
    inside 32-cell tiles; the bulk-copy sweep (FP32) equals the register
    sweep bit for bit and both stay close to the FP64 oracle."""
    b = cases.blusgs_case(m=7, seed=4)
    outs = []
    for var in (0, 2, 3, 4):
        S, e = make(b, prec=2, on_device=True)
        assert S.levels() > 5
        S.set_launch_config(threads_per_block=64, sweep_variant=var)
        run_sweeps(S, 2)
        outs.append(host(e["upts"]))
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])
    up = port.flowsys_blusgs(b, b["rhs"], b["dt"], b["jmat"], b["vol"], b["upts"], nsweeps=2)[0]
    dq = up - b["upts"]
    assert np.abs(outs[0] - up).max() <= 1e-4 * np.abs(dq).max()


def test_dependent_launch_large_and_small_levels(ucfd):
    """Greedy colours of a 40^3 mesh: the big colours (> 16384 cells) take the
    dependent-launch register kernel, the small ones the register-hoisted
    kernel; both equal the plain unrolled kernel bit for bit."""
    from ucfd_sparse_gb300 import coloredlusgs as cl
    b = cases.blusgs_case(m=40, seed=6)
    ic, rg, lc = cl.greedy_coloring_csr(b["rowptr"], b["colidx"])
    sizes = np.diff([0] + rg)
    assert sizes.max() > 16384 and sizes.min() < 16384
    outs = []
    for var in (0, 4):
        S, e = make(b, prec=2, on_device=True, colored=lc)
        S.set_launch_config(threads_per_block=128, sweep_variant=var)
        run_sweeps(S, 3)
        outs.append(host(e["upts"]))
    np.testing.assert_array_equal(outs[1], outs[0])


def test_blusgs_autotune_keeps_golden(golden, ucfd):
    """Autotune runs after Pack + NSPrepare; the sweeps that follow still
    reproduce the golden FP64 result bit for bit."""
    meta, arr = golden
    kw = cases.BLUSGS["blu10"]
    b = cases.blusgs_case(**kw)
    S, e = make(b, on_device=True)
    S.blusgs_pack(0, 0.0)
    S.blusgs_ns_prepare()
    cfg = S.autotune(reps=2)
    assert cfg["threads_per_block"] in (64, 128, 192, 256)
    assert cfg["sweep_variant"] in (0, 1, 4) and cfg["ms"] > 0  # FP64: no bulk-copy variants
    assert S.launch_config()["threads_per_block"] == cfg["threads_per_block"]
    run_sweeps(S, kw["nsweeps"])
    np.testing.assert_array_equal(host(e["upts"]), arr["blu10_upts"])
    np.testing.assert_array_equal(host(e["res"]), arr["blu10_resid"])


@pytest.mark.parametrize("prec", [0, 2])
def test_scalar_sweep_variants_identical(prec, golden, ucfd):
    """The six scalar sweep builds (one thread per cell with 3 register
    budgets, two threads per cell with 2, one thread per active face) give
    the same result; in FP64 it is the golden oracle result bit for bit."""
    from tests.test_gpu_lusgs import flowsys_step
    meta, arr = golden
    name = "fs9"
    kw = cases.FLOWSYS[name]
    fs, inp = cases.flowsys_case(**kw)
    outs = []
    for var in range(6):
        S, e = make_flowsys(fs, inp, prec=prec, on_device=True)
        S.set_launch_config(threads_per_block=128, sweep_variant=var)
        flowsys_step(S, kw, kw["nsteps"])
        outs.append(e["upts"].cpu().numpy())
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])
    if prec == 0:
        np.testing.assert_array_equal(outs[0], arr[f"{name}_upts"])


def test_lusgs_autotune_restores_state(ucfd):
    """Scalar autotune times the Run loop on the packed state and restores
    it: Run(mode=-1) afterwards equals Run on an untuned system."""
    fs, inp = cases.flowsys_case(**cases.FLOWSYS["fs9"])
    S, e = make_flowsys(fs, inp, prec=2, on_device=True)
    S.lusgs_pack(0, 1.0, 0.0)
    cfg = S.autotune(reps=2)
    assert cfg["run_mode"] in (0, 1) and cfg["ms"] > 0
    r1 = np.zeros(4)
    S.lusgs_run(4, 1.0, rans=False, mode=-1, resid=r1)
    S.lusgs_update(0)
    S2, e2 = make_flowsys(fs, inp, prec=2, on_device=True)
    S2.lusgs_pack(0, 1.0, 0.0)
    r2 = np.zeros(4)
    S2.lusgs_run(4, 1.0, rans=False, mode=0, resid=r2)
    S2.lusgs_update(0)
    np.testing.assert_array_equal(e["upts"].cpu().numpy(), e2["upts"].cpu().numpy())
    np.testing.assert_array_equal(r1, r2)


def test_autotune_cache_round_trip(tmp_path, ucfd):
    path = str(tmp_path / "tune.json")
    b = cases.blusgs_case(m=8, seed=3)
    S, e = make(b, prec=2, on_device=True)
    S.blusgs_pack(0, 0.0)
    S.blusgs_ns_prepare()
    first = S.autotune(reps=1, cache=path)
    assert first["source"] == "measured"
    S2, e2 = make(b, prec=2, on_device=True)
    S2.blusgs_pack(0, 0.0)
    S2.blusgs_ns_prepare()
    second = S2.autotune(reps=1, cache=path)
    assert second["source"] == "cache"
    for k in ("threads_per_block", "sweep_variant", "run_mode"):
        assert second[k] == first[k]
