"""CPU-side checks of the C-ABI library: it loads without a GPU, exports
every entry point its headers declare, and its host-only helpers
(connectivity, colourings) match the reference's example utilities."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from tests.golden import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        src = open(os.path.join(inc, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = "\n".join(l for l in src.splitlines() if not l.lstrip().startswith("#"))
        for m in re.finditer(r"UCFD_EXTERN\s+[\w\s\*]+?\b(\w+)\s*\(", src):
            names.add(m.group(1))
    return names


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return {l.split()[-1] for l in out.splitlines() if " T " in l}


def test_library_exports_every_declared_symbol(ucfd):
    from ucfd_sparse_gb300 import lib
    decl = header_symbols()
    assert len(decl) > 80
    exp = exported(lib.LIB_PATH)
    missing = decl - exp
    assert not missing, f"declared but not exported: {sorted(missing)}"
    extra = {s for s in exp if not s.startswith("_")} - decl
    assert not extra, f"exported but not declared in include/: {sorted(extra)}"
    # the ctypes binding covers the whole ABI
    assert decl == set(lib.SIGNATURES)


def test_headers_compile_as_c_and_cpp(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "ucfdlusgs.h"\n#include "coloredlusgs.h"\n#include "lusgs.h"\n'
                   '#include "ucfdsolver.h"\n#include "ucfdmesh.h"\nint main(void){return 0;}\n')
    for cc, std in (("gcc", "-std=c99"), ("g++", "-std=c++17")):
        subprocess.run([cc, std, "-Wall", "-Werror", "-fsyntax-only", "-x", "c" if cc == "gcc" else "c++",
                        "-I", os.path.join(ROOT, "include"), str(src)], check=True)


def test_errors_are_statuses_not_exits(ucfd):
    """Failures return a status with a message (the reference exit()s)."""
    from ucfd_sparse_gb300 import lib
    st = ucfd.UCFDMakeNeiEle(0, 1, 1, None)
    assert st == 2 and "bad arguments" in lib.last_error()
    h = ctypes.c_void_p()
    st = ucfd.UCFDFlowSysCreate(ctypes.byref(h), 0, 5, 5, 3, 1, 1, *([None] * 7))
    assert st == 2 and not h.value


@pytest.mark.parametrize("box", cases.BOXES)
def test_native_connectivity_matches_pbutils(box, golden, ucfd):
    from ucfd_sparse_gb300 import coloredlusgs as cl
    meta, arr = golden
    m, n, l = box
    np.testing.assert_array_equal(cl.make_nei_ele(m, n, l), arr[f"nei_{m}_{n}_{l}"])
    np.testing.assert_array_equal(cl.make_coloring(m, n, l), arr[f"col_{m}_{n}_{l}"])


def test_native_connectivity_32_hash(golden, ucfd):
    import hashlib
    from ucfd_sparse_gb300 import coloredlusgs as cl
    meta, _ = golden
    assert hashlib.sha256(cl.make_nei_ele(32, 32, 32).tobytes()).hexdigest() == meta["nei_32_sha"]
    assert hashlib.sha256(cl.make_coloring(32, 32, 32).tobytes()).hexdigest() == meta["col_32_sha"]


def _check_colouring(nei, icolor, ranges, lcolor):
    N = nei.shape[1]
    assert sorted(icolor.tolist()) == list(range(N))
    start = 0
    for c, end in enumerate(ranges):
        seg = icolor[start:end]
        assert np.all(lcolor[seg] == c + 1)
        assert np.all(np.diff(seg) > 0)
        start = end
    for f in range(nei.shape[0]):
        nb = nei[f]
        ok = (nb < 0) | (nb == np.arange(N))
        assert np.all(ok | (lcolor[np.maximum(nb, 0)] != lcolor)), "neighbours share a colour"


def test_greedy_colouring_native_matches_numpy_and_is_valid(ucfd):
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    c = mg.lusgs_case(9, jitter=0.2, permute=True)
    ic, rg, lc = cl.greedy_coloring(c["nei_ele"])
    ic2, rg2, lc2 = mg.greedy_coloring_np(c["nei_ele"])
    np.testing.assert_array_equal(ic, ic2)
    assert rg == [int(x) for x in rg2]
    _check_colouring(c["nei_ele"], ic, rg, lc)
    # tets (4 faces, boundary -1)
    nei = mg.kuhn_tet_adjacency(4)
    tab = np.where(nei >= 0, nei, np.arange(nei.shape[1])[None, :]).astype(np.int32)
    ic, rg, lc = cl.greedy_coloring(tab)
    _check_colouring(tab, ic, rg, lc)


def test_greedy_colouring_csr(ucfd):
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    b = mg.blusgs_case(6)
    ic, rg, lc = cl.greedy_coloring_csr(b["rowptr"], b["colidx"])
    tab = mg.csr_neighbors_to_table(b["rowptr"], b["colidx"])
    _check_colouring(tab, ic, rg, lc)


def test_bfs_colouring_csr(ucfd):
    """Breadth-first greedy colouring: valid, and two colours on a permuted
    hexahedral mesh (a bipartite graph) where index order needs more."""
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    b = mg.blusgs_case(8)
    ic, rg, lc = cl.greedy_coloring_csr(b["rowptr"], b["colidx"], order="bfs")
    tab = mg.csr_neighbors_to_table(b["rowptr"], b["colidx"])
    _check_colouring(tab, ic, rg, lc)
    assert len(rg) == 2
    assert len(cl.greedy_coloring_csr(b["rowptr"], b["colidx"])[1]) > 2
    # tets: valid, not bipartite
    nei = mg.kuhn_tet_adjacency(4)
    n = nei.shape[1]
    rp = np.arange(0, 4 * n + 1, 4, dtype=np.int32)
    ci = np.where(nei >= 0, nei, np.arange(n)[None, :]).T.reshape(-1).astype(np.int32)
    ic, rg, lc = cl.greedy_coloring_csr(rp, ci, order="bfs")
    tab = np.where(nei >= 0, nei, np.arange(n)[None, :]).astype(np.int32)
    _check_colouring(tab, ic, rg, lc)


def test_meshgen_geometry_is_closed():
    from ucfd_sparse_gb300 import meshgen as mg
    m = mg.HexMesh(6, jitter=0.2, seed=3)
    assert m.vol.sum() == pytest.approx(1.0, rel=1e-12)
    assert np.all(m.vol > 0)
    # closed cells: outward area vectors sum to zero
    s = m.cell_S.sum(axis=0)
    assert np.abs(s).max() < 1e-14
    nei = mg.kuhn_tet_adjacency(3)
    N = nei.shape[1]
    for f in range(4):
        ok = nei[f] >= 0
        back = nei[:, nei[f][ok]]
        assert np.all((back == np.arange(N)[ok][None, :]).any(axis=0)), "tet adjacency not symmetric"


def test_bsr_case_is_diagonally_dominant():
    from ucfd_sparse_gb300 import meshgen as mg
    s = mg.bsr_case(3)
    bn, blk = s["bn"], s["blk"]
    v = s["values"]
    rows = np.repeat(np.arange(bn), np.diff(s["rowptr"]))
    absrow = np.zeros((bn, blk))
    np.add.at(absrow, rows, np.abs(v).sum(axis=2))
    d = np.abs(v[s["diagslots"]][:, np.arange(blk), np.arange(blk)])
    assert np.all(d > absrow - d)


def test_oracle_colouring_equals_native(ucfd, port):
    """The oracle's greedy colouring (used by the CPU legs, which must not
    load the product library) equals UCFDGreedyColoringCSR: on a permuted
    hex mesh, and on a random graph with one-directional edges, self entries
    and negative (boundary) entries."""
    from ucfd_sparse_gb300 import coloredlusgs as cl
    from ucfd_sparse_gb300 import meshgen as mg
    b = mg.blusgs_case(8, seed=2)
    rng = np.random.default_rng(7)
    n = 3000
    deg = rng.integers(0, 7, n)
    rp = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    ci = rng.integers(-1, n, int(rp[-1])).astype(np.int32)
    ci[::17] = np.repeat(np.arange(n), deg)[::17]          # some self entries
    for rowptr, colidx in ((b["rowptr"], b["colidx"]), (rp, ci)):
        ic, rg, lc = cl.greedy_coloring_csr(rowptr, colidx)
        ic2, rg2, lc2 = port.greedy_coloring_csr(rowptr, colidx)
        np.testing.assert_array_equal(ic, ic2)
        np.testing.assert_array_equal(lc, lc2)
        assert rg == rg2


def test_host_array_access_setting(ucfd):
    """UCFDSetHostArrayAccess / UCFDGetHostArrayAccess: process-wide, in-place
    reads of page-locked host Jacobians (UCFD_HOST_MAP) by default; unknown
    modes are rejected with UCFD_ERR_ARGUMENT and leave the setting alone."""
    from ucfd_sparse_gb300 import lib
    assert lib.host_array_access() == lib.HOST_MAP
    try:
        lib.set_host_array_access(lib.HOST_STAGE)
        assert lib.host_array_access() == lib.HOST_STAGE
        assert ucfd.UCFDSetHostArrayAccess(5) == 2 and "UCFD_HOST" in lib.last_error()
        assert lib.host_array_access() == lib.HOST_STAGE
    finally:
        lib.set_host_array_access(lib.HOST_MAP)
    assert lib.host_array_access() == lib.HOST_MAP
