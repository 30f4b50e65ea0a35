"""The allocation-free residual entry point (UCFDBLUSGS_ResidualNoAlloc).

Callers that cannot allocate device memory while they run -- a code whose
device memory is all handed to its own pool at start-up, or whose time-step
loop must not stall on cudaMalloc -- use this variant to monitor the block
LU-SGS residual.  It must agree with UCFDBLUSGS_Residual (same per-cell
arithmetic, different summation order across cells) on consecutive calls,
since every call reuses the same fixed device scratch array.  This file is
collected last so that a failure here stops a ``-x`` run only after every
other test has run.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

REL = 1e-12  # summation-order tolerance on the relative residual


def _system(prec):
    from ucfd_sparse_gb300 import meshgen as mg
    from ucfd_sparse_gb300.flowsys import FlowSys
    b = mg.blusgs_case(10, seed=6)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    m = {k: T(b[k]) for k in ("rowptr", "colidx", "slots", "sides", "face_area", "face_normal", "rcp_vol")}
    S = FlowSys(b["nlocal"], 5, 5, 3, b["nfaces"], 1, m["rowptr"], m["colidx"], m["slots"], m["sides"],
                m["face_area"], m["face_normal"], m["rcp_vol"])
    S.set_precision(prec)
    e = {k: T(b[k]) for k in ("rhs", "dt", "cell_ids", "vol", "jmat")}
    e["upts"] = T(np.array(b["upts"]))
    e["dsrc"] = torch.zeros_like(e["upts"])
    e["res"] = torch.zeros_like(e["upts"])
    S.set_element(0, b["neles"], 6, e["cell_ids"], e["upts"], e["rhs"], e["dt"], e["dsrc"], e["vol"], e["res"])
    S.set_blusgs(e["jmat"])
    S.blusgs_pack(0, 0.0)
    S.blusgs_ns_prepare()
    S.blusgs_reset()
    return S, e


def _noalloc(S, out):
    from ucfd_sparse_gb300 import lib
    lib.call("UCFDBLUSGS_ResidualNoAlloc", S._h, lib.ptr(out) if not isinstance(out, ctypes.c_double)
             else ctypes.addressof(out))


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_noalloc_residual_matches_existing_entry_point(prec, ucfd):
    S, _ = _system(prec)
    for sweeps in (1, 2):
        # two sweeps between checks, then two calls in a row on the same state
        for _ in range(sweeps):
            S.blusgs_ns_lower()
            S.blusgs_ns_upper()
        ref = S.blusgs_residual()
        assert 0.0 < ref < 1.0
        for _ in range(2):
            h = ctypes.c_double(-1.0)
            _noalloc(S, h)
            assert abs(h.value - ref) <= REL * ref
            d = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
            _noalloc(S, d)
            assert abs(float(d.item()) - ref) <= REL * ref


def test_noalloc_residual_requires_prepared_system(ucfd):
    from ucfd_sparse_gb300 import lib
    from ucfd_sparse_gb300 import meshgen as mg
    from ucfd_sparse_gb300.flowsys import FlowSys
    b = mg.blusgs_case(4, seed=1)
    S = FlowSys(b["nlocal"], 5, 5, 3, b["nfaces"], 1, b["rowptr"], b["colidx"], b["slots"], b["sides"],
                b["face_area"], b["face_normal"], b["rcp_vol"])
    S.set_blusgs(b["jmat"])
    h = ctypes.c_double(-1.0)
    with pytest.raises(lib.UCFDError) as ex:
        _noalloc(S, h)
    assert ex.value.status == 8 and "prepared" in str(ex.value)


def test_noalloc_residual_rejects_systems_above_its_limit(ucfd):
    """8,388,610 cells, two more than the fixed scratch array covers: cells
    2k and 2k+1 share face k, so the system is small in memory (about 8 GB on
    the device) yet valid; the allocation-free call refuses it with
    UCFD_ERR_ARGUMENT while UCFDBLUSGS_Residual still computes it."""
    from ucfd_sparse_gb300 import lib
    from ucfd_sparse_gb300.flowsys import FlowSys
    N = 8388610
    nF = N // 2
    dev = torch.device("cuda:0")
    i = torch.arange(N, dtype=torch.int32, device=dev)
    rowptr = torch.arange(N + 1, dtype=torch.int32, device=dev)
    colidx = torch.bitwise_xor(i, 1)
    slots = torch.div(i, 2, rounding_mode="floor")
    sides = torch.where(i % 2 == 0, 1, -1).to(torch.int8)
    area = torch.ones(nF, dtype=torch.float64, device=dev)
    normal = torch.zeros(3, nF, dtype=torch.float64, device=dev)
    normal[0] = 1.0
    rv = torch.ones(N, dtype=torch.float64, device=dev)
    S = FlowSys(N, 5, 5, 3, nF, 1, rowptr, colidx, slots, sides, area, normal, rv)
    jmat = torch.zeros(2, 5, 5, nF, dtype=torch.float64, device=dev)
    for r in range(5):
        jmat[0, r, r] = 1.0
        jmat[1, r, r] = -1.0
    rhs = torch.randn(5, N, dtype=torch.float64, device=dev, generator=torch.Generator(dev).manual_seed(3))
    upts = torch.zeros_like(rhs)
    S.set_element(0, N, 1, i.clone(), upts, rhs, torch.ones(N, dtype=torch.float64, device=dev),
                  torch.zeros_like(rhs), torch.ones(N, dtype=torch.float64, device=dev), torch.zeros_like(rhs))
    S.set_blusgs(jmat)
    S.blusgs_pack(0, 0.0)
    S.blusgs_ns_prepare()
    S.blusgs_reset()
    assert abs(S.blusgs_residual() - 1.0) <= 1e-12  # du = 0: the residual is rhs itself
    h = ctypes.c_double(-1.0)
    with pytest.raises(lib.UCFDError) as ex:
        _noalloc(S, h)
    assert ex.value.status == 2 and "8388608" in str(ex.value)
    assert h.value == -1.0
    S.destroy()
    del jmat
    torch.cuda.empty_cache()
