"""The benchmark's reference arm (CPU): it runs the reference's CPU path
alone -- no library of this repository's product is loaded -- and reports
the GPU arm's metric, unit and workload description."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_loads_no_product_library():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--mesh", "8",
                        "--steps", "3", "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "cell-updates/s" and line["higher_is_better"]
    assert line["config"]["cells"] == 512 and line["config"]["colors"] >= 2
    libs = line["libraries_loaded"]
    assert libs is not None and not any("libucfd_gb300" in p for p in libs), libs
    assert any(p.startswith("oracle/") for p in libs), libs
    assert line["cpu_baseline"]["kind"] in ("reference", "port") and line["cpu_baseline"]["cores"] == 1
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]


def test_cpu_step_composition_and_sweep_bytes():
    """The CPU legs' step is Pack+Prepare+Reset + Update + 40 pairs of
    (lower, upper + SubResidual); the FP32 sweep moves 424 B per interior hex
    cell (6 indices x 4, half the 6 blocks of 100 B, 5 vectors of 20 B)."""
    import numpy as np
    import bench
    assert bench.PAIRS_PER_STEP == 40
    assert bench.compose_cpu_step(2.0, 0.5, 1.0, 1.5) == 2.0 + 0.5 + 40 * 2.5
    rowptr = np.arange(0, 6 * 11, 6)              # 10 cells of 6 faces each
    assert bench.sweep_bytes(rowptr, 4, 5) == 10 * 424
    assert bench.sweep_bytes(rowptr, 8, 5) == 10 * 824


def test_scalar_loop_byte_counts():
    """One sweep of both scalar systems moves 264 B per interior hex cell
    (6 faces x 28 B, 4 + 20 + 72 B per cell); the loop's iteration with the
    one-pass kernels moves fewer bytes than with separate NS and RANS ones."""
    import numpy as np
    import bench
    rowptr = np.arange(0, 6 * 11, 6)              # 10 cells of 6 faces each
    assert bench.nsrans_sweep_bytes(rowptr) == 10 * 264
    assert bench.lusgs_iter_bytes(rowptr, 4, both=True) < bench.lusgs_iter_bytes(rowptr, 4)
