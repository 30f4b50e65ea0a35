"""Bounded device waits give up and report (no hang, no fault): the grid
barrier of the persistent scalar sweep and the mbarrier wait of the
bulk-copy block sweep, each run on a state that never completes; the
context stays usable afterwards."""
from ctypes import byref, c_int

import numpy as np
import pytest

from tests.golden import cases
from tests.test_gpu_blusgs import host, make, run_sweeps

pytestmark = pytest.mark.gpu


def test_waits_time_out_and_context_survives(golden, ucfd):
    from ucfd_sparse_gb300.lib import call
    a, b = c_int(0), c_int(0)
    call("UCFDSelfTestTimeouts", byref(a), byref(b))
    assert a.value == 1, "grid barrier did not report its timeout"
    assert b.value == 1, "mbarrier wait did not report its timeout"
    # the same process keeps computing correct results
    meta, arr = golden
    kw = cases.BLUSGS["blu10"]
    S, e = make(cases.blusgs_case(**kw), on_device=True)
    run_sweeps(S, kw["nsweeps"])
    np.testing.assert_array_equal(host(e["upts"]), arr["blu10_upts"])
