"""Seeded synthetic meshes and systems for the LU-SGS / BLU-SGS / Krylov path.

The reference ships only a regular-box generator (``examples/utils/pbutils.py``:
``make_nei_ele`` 4-36 and ``make_coloring`` 39-56).  This module provides the
same two functions (delegating to the native implementations in the C-ABI
library, which tests pin bit-exactly against pbutils' outputs) plus the
jittered / permuted hexahedral meshes and the Kuhn-split tetrahedral BSR
system used by the parity tests and the benchmark.

All floating-point geometry is written as explicit element-wise arithmetic
(no ``np.sum``/``np.mean`` reductions) so that the generated arrays are
bit-identical on every platform numpy runs on.
"""
from __future__ import annotations

import numpy as np

GAMMA = 1.4

# face order of the reference hex connectivity (pbutils.py:9): -x,+x,-y,+y,-z,+z
HEX_FACE_AXIS = np.array([0, 0, 1, 1, 2, 2])
HEX_FACE_SIGN = np.array([-1.0, 1.0, -1.0, 1.0, -1.0, 1.0])


# --------------------------------------------------------------------------
# regular box connectivity (pbutils.py:4-56), numpy restatement used when the
# native library is not wanted (e.g. while building fixtures)
# --------------------------------------------------------------------------
def box_nei_ele(m: int, n: int, l: int) -> np.ndarray:
    """[6, m*n*l] int32 neighbour table, boundary faces point to the cell itself."""
    N = m * n * l
    idx = np.arange(N, dtype=np.int32).reshape(l, n, m)
    adj = np.empty((6, l, n, m), dtype=np.int32)
    adj[:] = idx[None]
    adj[0][..., 1:] = idx[..., :-1]
    adj[1][..., :-1] = idx[..., 1:]
    adj[2][:, 1:, :] = idx[:, :-1, :]
    adj[3][:, :-1, :] = idx[:, 1:, :]
    adj[4][1:] = idx[:-1]
    adj[5][:-1] = idx[1:]
    return adj.reshape(6, N)


def box_coloring(m: int, n: int, l: int) -> np.ndarray:
    """Checkerboard cell list: cells with (x+y+z) even first, then odd."""
    i = np.arange(m * n * l, dtype=np.int32)
    x, y, z = i % m, (i // m) % n, i // (m * n)
    even = ((x + y + z) & 1) == 0
    return np.concatenate((i[even], i[~even]))


def free_stream(nvars: int, neles: int, rho=GAMMA, u=1.5, v=0.0, w=0.0, p=1.0) -> np.ndarray:
    """Uniform conservative state of the reference examples (omp3d.py:41-66)."""
    et = p / (GAMMA - 1) + 0.5 * rho * u * u
    q = np.zeros((nvars, neles))
    vals = [rho, rho * u, rho * v, rho * w, et]
    for k in range(min(nvars, 5)):
        q[k] = vals[k]
    return q


# --------------------------------------------------------------------------
# jittered hexahedral box
# --------------------------------------------------------------------------
def _cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
                     a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], axis=-1)


def _dot3(a, b):
    return a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1] + a[..., 2] * b[..., 2]


class HexMesh:
    """m^3 hexahedra on the unit cube, interior nodes jittered by U[-j h, j h]^3.

    Cells are numbered x-fastest (``c = x + m*y + m*m*z``, as pbutils).  For
    every cell and each of its six faces (order -x,+x,-y,+y,-z,+z) the mesh
    stores the outward area vector; interior faces are also listed once each
    (``face_a`` -> ``face_b`` along +axis) for the shared-face layout.
    """

    def __init__(self, m: int, jitter: float = 0.0, seed: int = 0):
        self.m = m
        N = m ** 3
        h = 1.0 / m
        rng = np.random.default_rng(seed)
        g = np.arange(m + 1) * h
        P = np.empty((m + 1, m + 1, m + 1, 3))  # [z, y, x, xyz]
        P[..., 0] = g[None, None, :]
        P[..., 1] = g[None, :, None]
        P[..., 2] = g[:, None, None]
        if jitter > 0 and m > 1:
            J = rng.uniform(-jitter * h, jitter * h, size=(m - 1, m - 1, m - 1, 3))
            P[1:-1, 1:-1, 1:-1] = P[1:-1, 1:-1, 1:-1] + J
        self.nodes = P

        # area vectors of all faces, oriented along +axis
        # x-faces at plane i: nodes (k,j,i),(k,j+1,i),(k+1,j+1,i),(k+1,j,i)
        def quad_area(a, b, c, d):
            d1 = c - a
            d2 = d - b
            S = _cross(d1, d2)
            S = 0.5 * S
            ctr = ((a + b) + (c + d)) * 0.25
            return S, ctr

        Sx, Cx = quad_area(P[:-1, :-1, :], P[:-1, 1:, :], P[1:, 1:, :], P[1:, :-1, :])   # [m, m, m+1]
        Sy, Cy = quad_area(P[:-1, :, :-1], P[1:, :, :-1], P[1:, :, 1:], P[:-1, :, 1:])   # [m, m+1, m]
        Sz, Cz = quad_area(P[:, :-1, :-1], P[:, :-1, 1:], P[:, 1:, 1:], P[:, 1:, :-1])   # [m+1, m, m]
        for S, ax in ((Sx, 0), (Sy, 1), (Sz, 2)):
            flip = S[..., ax] < 0
            S[flip] = -S[flip]

        # per-cell outward area vectors and centroids, face order -x,+x,-y,+y,-z,+z
        cS = np.empty((6, m, m, m, 3))
        cC = np.empty((6, m, m, m, 3))
        cS[0], cC[0] = -Sx[:, :, :-1], Cx[:, :, :-1]
        cS[1], cC[1] = Sx[:, :, 1:], Cx[:, :, 1:]
        cS[2], cC[2] = -Sy[:, :-1, :], Cy[:, :-1, :]
        cS[3], cC[3] = Sy[:, 1:, :], Cy[:, 1:, :]
        cS[4], cC[4] = -Sz[:-1], Cz[:-1]
        cS[5], cC[5] = Sz[1:], Cz[1:]
        vol = _dot3(cC[0], cS[0])
        for f in range(1, 6):
            vol = vol + _dot3(cC[f], cS[f])
        vol = vol / 3.0
        self.cell_S = cS.reshape(6, N, 3)
        self.vol = vol.reshape(N)
        area = np.sqrt(_dot3(self.cell_S, self.cell_S))      # [6, N]
        self.cell_area = area
        self.cell_normal = self.cell_S / area[..., None]      # [6, N, 3]
        self.nei = box_nei_ele(m, m, m)

        # interior shared faces: (a -> b along +axis), area vector along +axis
        c = np.arange(N, dtype=np.int64).reshape(m, m, m)
        fa, fb, fS = [], [], []
        fa.append(c[:, :, :-1].ravel()); fb.append(c[:, :, 1:].ravel()); fS.append(Sx[:, :, 1:-1].reshape(-1, 3))
        fa.append(c[:, :-1, :].ravel()); fb.append(c[:, 1:, :].ravel()); fS.append(Sy[:, 1:-1, :].reshape(-1, 3))
        fa.append(c[:-1].ravel()); fb.append(c[1:].ravel()); fS.append(Sz[1:-1].reshape(-1, 3))
        self.face_a = np.concatenate(fa)
        self.face_b = np.concatenate(fb)
        S = np.concatenate(fS)
        self.face_area = np.sqrt(_dot3(S, S))
        self.face_normal = S / self.face_area[:, None]        # [nF, 3]

    @property
    def ncells(self):
        return self.m ** 3

    @property
    def nfaces(self):
        return self.face_a.shape[0]

    # ---- colored array ("legacy") layout -------------------------------
    def legacy_geometry(self, perm: np.ndarray | None = None):
        """fnorm_vol [6,N], vec_fnorm [6,3,N], nei_ele [6,N] (int32).

        With ``perm`` (new index = perm[old]) the cells are renumbered, so
        neighbour gathers become irregular.
        """
        N = self.ncells
        fnorm_vol = self.cell_area / self.vol[None, :]
        vec = np.ascontiguousarray(self.cell_normal.transpose(0, 2, 1))  # [6,3,N]
        nei = self.nei.astype(np.int32)
        if perm is None:
            return np.ascontiguousarray(fnorm_vol), vec, nei
        inv = np.empty(N, dtype=np.int64)
        inv[perm] = np.arange(N)
        return (np.ascontiguousarray(fnorm_vol[:, inv]), np.ascontiguousarray(vec[:, :, inv]),
                np.ascontiguousarray(perm[nei[:, inv]].astype(np.int32)))

    # ---- FlowSys (CSR over shared faces) layout ------------------------
    def flowsys(self, perm: np.ndarray | None = None, face_perm: np.ndarray | None = None):
        """Rank-level CSR of the reference FlowSys (src/lusgs/flowsys.h:34-59).

        Rank ``r = perm[cell]``; each rank lists its interior faces in the
        order -x,+x,-y,+y,-z,+z.  ``sides`` is +1 where the rank is the face's
        first cell (the stored normal points out of it) and -1 otherwise.
        """
        N, nF = self.ncells, self.nfaces
        perm = np.arange(N) if perm is None else np.asarray(perm)
        fslot = np.arange(nF) if face_perm is None else np.asarray(face_perm)
        # per cell-face: slot of the shared face (or -1 at the boundary)
        m = self.m
        slot_of = -np.ones((6, N), dtype=np.int64)
        nx = m * m * (m - 1)
        c = np.arange(N).reshape(m, m, m)
        xs = np.arange(nx).reshape(m, m, m - 1)
        slot_of[1, c[:, :, :-1].ravel()] = xs.ravel()
        slot_of[0, c[:, :, 1:].ravel()] = xs.ravel()
        ys = nx + np.arange(nx).reshape(m, m - 1, m)
        slot_of[3, c[:, :-1, :].ravel()] = ys.ravel()
        slot_of[2, c[:, 1:, :].ravel()] = ys.ravel()
        zs = 2 * nx + np.arange(nx).reshape(m - 1, m, m)
        slot_of[5, c[:-1].ravel()] = zs.ravel()
        slot_of[4, c[1:].ravel()] = zs.ravel()
        inv = np.empty(N, dtype=np.int64)
        inv[perm] = np.arange(N)
        deg = (slot_of >= 0).sum(axis=0)[inv]                  # per rank
        rowptr = np.zeros(N + 1, dtype=np.int32)
        rowptr[1:] = np.cumsum(deg)
        nnz = int(rowptr[-1])
        colidx = np.empty(nnz, dtype=np.int32)
        slots = np.empty(nnz, dtype=np.int32)
        sides = np.empty(nnz, dtype=np.int8)
        # fill rank by rank in face order
        pos = rowptr[:-1].astype(np.int64).copy()
        cells_of_rank = inv
        for f in range(6):
            s = slot_of[f, cells_of_rank]
            ok = s >= 0
            r = np.nonzero(ok)[0]
            sl = s[ok]
            nb_cell = self.nei[f, cells_of_rank[r]]
            colidx[pos[r]] = perm[nb_cell]
            slots[pos[r]] = fslot[sl]
            sides[pos[r]] = 1 if f % 2 == 1 else -1
            pos[r] += 1
        face_area = np.empty(nF)
        face_area[fslot] = self.face_area
        face_normal = np.empty((3, nF))
        face_normal[:, fslot] = self.face_normal.T
        rcp_vol = np.empty(N)
        rcp_vol[perm] = 1.0 / self.vol
        return dict(nlocal=N, nfaces=nF, rowptr=rowptr, colidx=colidx, slots=slots,
                    sides=sides, face_area=face_area, face_normal=face_normal,
                    rcp_vol=rcp_vol, perm=perm)


def random_perm(n: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).permutation(n).astype(np.int64)


# --------------------------------------------------------------------------
# scalar colored LU-SGS workload (configs: 32^3 box; jittered/permuted boxes)
# --------------------------------------------------------------------------
def lusgs_case(m: int, nvars: int = 5, jitter: float = 0.0, permute: bool = False, seed: int = 0):
    """Arrays of one colored LU-SGS step in the reference array layout.

    fspr ~ U[0.5, 2] per cell-face, dt ~ U[1e-3, 1e-2], rhs ~ N(0, 1) per
    (variable, cell), upts = the reference examples' free stream.
    """
    mesh = HexMesh(m, jitter=jitter, seed=seed)
    N = mesh.ncells
    perm = random_perm(N, seed + 1) if permute else None
    fnorm_vol, vec_fnorm, nei = mesh.legacy_geometry(perm)
    rng = np.random.default_rng(seed + 2)
    fspr = rng.uniform(0.5, 2.0, size=(6, N))
    dt = rng.uniform(1e-3, 1e-2, size=N)
    rhs = rng.standard_normal((nvars, N))
    upts = free_stream(nvars, N)
    if nvars > 5:
        upts[5:] = rng.uniform(0.1, 1.0, size=(nvars - 5, N))
    return dict(m=m, neles=N, nface=6, nvars=nvars, nei_ele=nei, fnorm_vol=fnorm_vol,
                vec_fnorm=vec_fnorm, fspr=fspr, dt=dt, rhs=rhs, upts=upts, perm=perm)


def colors_from_icolor(icolor: np.ndarray, ranges: list[int]) -> np.ndarray:
    """lcolor (1-based colour of each cell) from an icolor list and its range ends."""
    lcolor = np.empty(icolor.shape[0], dtype=np.int32)
    start = 0
    for c, end in enumerate(ranges):
        lcolor[icolor[start:end]] = c + 1
        start = end
    return lcolor


def greedy_coloring_np(nei: np.ndarray, order: np.ndarray | None = None):
    """Greedy first-fit colouring of a [nface, N] neighbour table (pure numpy
    loop; small meshes only).  Returns (icolor, ranges, lcolor)."""
    nface, N = nei.shape
    order = np.arange(N) if order is None else order
    col = np.zeros(N, dtype=np.int32)
    for i in order:
        used = set(int(col[j]) for j in nei[:, i] if j != i and col[j] > 0)
        c = 1
        while c in used:
            c += 1
        col[i] = c
    nc = int(col.max())
    icolor = np.concatenate([np.nonzero(col == c)[0] for c in range(1, nc + 1)]).astype(np.int32)
    ranges = list(np.cumsum([int((col == c).sum()) for c in range(1, nc + 1)]))
    return icolor, ranges, col


# --------------------------------------------------------------------------
# BLU-SGS workload (FlowSys layout with 5x5 face Jacobians)
# --------------------------------------------------------------------------
def blusgs_case(m: int, nvars: int = 5, jitter: float = 0.2, permute: bool = True, seed: int = 0):
    """FlowSys arrays, jmat [2][nv][nv][nfaces] and per-element inputs.

    jmat half 0 (the A+ split) = sigma I + E0, half 1 (A-) = -sigma I + E1,
    sigma = fspr of the face ~ U[0.5, 2], E ~ N(0, 0.05^2) per entry.
    Elements are the cells in x-fastest order; ``cell_ids`` maps them to ranks.
    """
    mesh = HexMesh(m, jitter=jitter, seed=seed)
    N = mesh.ncells
    perm = random_perm(N, seed + 1) if permute else np.arange(N)
    fs = mesh.flowsys(perm)
    nF = fs['nfaces']
    rng = np.random.default_rng(seed + 3)
    sigma = rng.uniform(0.5, 2.0, size=nF)
    E = rng.normal(0.0, 0.05, size=(2, nvars, nvars, nF))
    jmat = E
    for r in range(nvars):
        jmat[0, r, r] += sigma
        jmat[1, r, r] -= sigma
    dt = rng.uniform(1e-3, 1e-2, size=N)
    rhs = rng.standard_normal((nvars, N))
    upts = free_stream(nvars, N)
    vol = mesh.vol.copy()
    fs.update(dict(nvars=nvars, nfvars=min(nvars, 5), ndims=3, jmat=np.ascontiguousarray(jmat), fspr_face=sigma,
                   neles=N,
                   cell_ids=perm.astype(np.int32), dt=dt, rhs=rhs, upts=upts, vol=vol,
                   mesh=mesh))
    return fs


def lusgs_flowsys_case(m: int, nvars: int = 6, jitter: float = 0.2, permute: bool = True, seed: int = 0,
                       rhs_scale: float = 1.0):
    """Scalar LU-SGS FlowSys workload: jittered, permuted hex mesh with
    per-face spectral radii fspr, tfspr ~ U[0.5, 2], dt ~ U[1e-3, 1e-2],
    rhs ~ N(0, 1) * rhs_scale and the free stream (turbulence variables
    ~ U[0.1, 1]).  A pseudo-time loop that re-applies the same rhs drifts
    the state by ~rhs/diag per iteration; rhs_scale = 1e-3 keeps it physical
    for thousands of iterations."""
    mesh = HexMesh(m, jitter=jitter, seed=seed)
    N = mesh.ncells
    perm = random_perm(N, seed + 1) if permute else np.arange(N)
    fs = mesh.flowsys(perm)
    rng = np.random.default_rng(seed + 5)
    nF = fs["nfaces"]
    upts = free_stream(nvars, N)
    if nvars > 5:
        upts[5:] = rng.uniform(0.1, 1.0, size=(nvars - 5, N))
    fs.update(dict(nvars=nvars, nfvars=min(nvars, 5), ndims=3, neles=N, cell_ids=perm.astype(np.int32),
                   fspr=rng.uniform(0.5, 2.0, nF), tfspr=rng.uniform(0.5, 2.0, nF),
                   dt=rng.uniform(1e-3, 1e-2, N), rhs=rng.standard_normal((nvars, N)) * rhs_scale, upts=upts,
                   vol=mesh.vol.copy()))
    return fs


def renumber_flowsys(fs: dict, new_of_rank: np.ndarray) -> dict:
    """The same FlowSys mesh with ranks renumbered (new rank = new_of_rank[old]).

    Rows keep their per-row face order, so a natural-order sweep of the
    result visits every cell with the arithmetic of the original row.
    """
    N = fs['nlocal']
    old_of_new = np.empty(N, dtype=np.int64)
    old_of_new[new_of_rank] = np.arange(N)
    rp = fs['rowptr']
    deg = (rp[1:] - rp[:-1])[old_of_new]
    rowptr = np.zeros(N + 1, dtype=np.int32)
    rowptr[1:] = np.cumsum(deg)
    src = _row_gather(rp, old_of_new)
    out = dict(fs)
    out.update(rowptr=rowptr, colidx=new_of_rank[fs['colidx'][src]].astype(np.int32),
               slots=fs['slots'][src].copy(), sides=fs['sides'][src].copy(),
               rcp_vol=fs['rcp_vol'][old_of_new].copy())
    if 'cell_ids' in fs:
        out['cell_ids'] = new_of_rank[fs['cell_ids']].astype(np.int32)
    return out


def _row_gather(rp, rows):
    deg = (rp[1:] - rp[:-1])[rows].astype(np.int64)
    start = rp[:-1][rows].astype(np.int64)
    off = np.repeat(start - np.concatenate([[0], np.cumsum(deg)[:-1]]), deg)
    return np.arange(int(deg.sum())) + off


def csr_neighbors_to_table(rowptr, colidx, width=None):
    """Pad a CSR neighbour list to a [width, N] table (self for missing entries)."""
    N = rowptr.shape[0] - 1
    deg = rowptr[1:] - rowptr[:-1]
    width = int(deg.max()) if width is None else width
    tab = np.tile(np.arange(N, dtype=np.int32), (width, 1))
    for p in range(width):
        has = deg > p
        tab[p, has] = colidx[rowptr[:-1][has] + p]
    return tab


# --------------------------------------------------------------------------
# Kuhn-split tetrahedral BSR system (GMRES workload)
# --------------------------------------------------------------------------
def kuhn_tet_adjacency(m: int):
    """Face-neighbour table [4, 6 m^3] of the 6-tetrahedra Kuhn split of an
    m^3 box.  Every hex (x-fastest numbering) is split along its
    (0,0,0)-(1,1,1) diagonal into the 6 tets of the axis permutations, which
    makes the split conforming.  Tet ``6*hex + t``; missing neighbours
    (boundary faces) are -1."""
    import itertools
    nn = m + 1
    h = np.arange(m ** 3, dtype=np.int64)
    hx, hy, hz = h % m, (h // m) % m, h // (m * m)
    perms = list(itertools.permutations(range(3)))
    nodes = np.empty((m ** 3, len(perms), 4), dtype=np.int64)
    for t, p in enumerate(perms):
        off = np.zeros(3, dtype=np.int64)
        for k in range(4):
            if k > 0:
                off[p[k - 1]] += 1
            nodes[:, t, k] = (hx + off[0]) + nn * ((hy + off[1]) + nn * (hz + off[2]))
    nodes = nodes.reshape(-1, 4)
    ncell = nodes.shape[0]
    # each tet face as its sorted node triple, cell-major (tet, face k);
    # faces shared by two tets are equal triples, adjacent once sorted
    tris = np.empty((ncell, 4, 3), dtype=np.int64)
    for k in range(4):
        tris[:, k] = np.sort(np.delete(nodes, k, axis=1), axis=1)
    tris = tris.reshape(-1, 3)
    order = np.lexsort((tris[:, 2], tris[:, 1], tris[:, 0]))
    st = tris[order]
    same = np.all(st[1:] == st[:-1], axis=1)
    i0 = order[:-1][same]
    i1 = order[1:][same]
    nei = -np.ones(ncell * 4, dtype=np.int64)
    nei[i0] = i1 // 4
    nei[i1] = i0 // 4
    return nei.reshape(ncell, 4).T.astype(np.int32).copy()


def bsr_case(m: int, blk: int = 5, seed: int = 0, scale: float = 1.0):
    """Diagonally dominant BSR system on the Kuhn-tet dual graph.

    Off-diagonal blocks ~ N(0,1)*scale; the diagonal block has N(0,1)*scale
    off-diagonal entries and diagonal entries = sum of |entries| of the rest
    of its scalar row + U[0.1, 1].  Columns are sorted within each row.
    Returns dict(bn, blk, rowptr, colidx, values [nnzb, blk, blk], diagslots,
    rhs, nei).
    """
    nei = kuhn_tet_adjacency(m)
    return bsr_from_table(nei, blk, seed, scale)


def bsr_from_table(nei: np.ndarray, blk: int, seed: int = 0, scale: float = 1.0):
    nf, bn = nei.shape
    rng = np.random.default_rng(seed)
    cols = np.concatenate([nei, np.arange(bn, dtype=np.int32)[None]], axis=0)   # [nf+1, bn]
    valid = cols >= 0
    cols = np.where(valid, cols, np.int32(2 ** 31 - 1))
    srt = np.sort(cols, axis=0)
    deg = valid.sum(axis=0)
    rowptr = np.zeros(bn + 1, dtype=np.int32)
    rowptr[1:] = np.cumsum(deg)
    mask = srt.T < 2 ** 31 - 1
    colidx = srt.T[mask].astype(np.int32)
    rows = np.repeat(np.arange(bn), deg)
    nnzb = colidx.shape[0]
    values = rng.standard_normal((nnzb, blk, blk)) * scale
    isdiag = colidx == rows
    diagslots = np.nonzero(isdiag)[0].astype(np.int32)
    absrow = np.abs(values)
    # per scalar row: sum of |a| over all entries of the block row except the diagonal entry
    rs = np.zeros((bn, blk))
    rowabs = absrow[:, :, 0]
    for c in range(1, blk):
        rowabs = rowabs + absrow[:, :, c]
    np.add.at(rs, rows, rowabs)
    dvals = values[diagslots]
    for r in range(blk):
        rs[:, r] -= np.abs(dvals[:, r, r])
        dvals[:, r, r] = rs[:, r] + rng.uniform(0.1, 1.0, size=bn)
    values[diagslots] = dvals
    rhs = rng.standard_normal(bn * blk)
    return dict(bn=bn, blk=blk, rowptr=rowptr, colidx=colidx, values=np.ascontiguousarray(values),
                diagslots=diagslots, rhs=rhs, nei=nei)


def renumber_bsr(sys: dict, new_of_old: np.ndarray) -> dict:
    """Symmetric block renumbering of a BSR system, columns re-sorted per row."""
    bn, blk = sys['bn'], sys['blk']
    old_of_new = np.empty(bn, dtype=np.int64)
    old_of_new[new_of_old] = np.arange(bn)
    rp = sys['rowptr']
    deg = (rp[1:] - rp[:-1])[old_of_new]
    rowptr = np.zeros(bn + 1, dtype=np.int32)
    rowptr[1:] = np.cumsum(deg)
    src = _row_gather(rp, old_of_new)
    newcol = new_of_old[sys['colidx'][src]]
    rows = np.repeat(np.arange(bn), deg)
    order = np.lexsort((newcol, rows))
    src = src[order]
    colidx = newcol[order].astype(np.int32)
    values = sys['values'][src]
    diagslots = np.nonzero(colidx == rows)[0].astype(np.int32)
    rhs = sys['rhs'].reshape(bn, blk)[old_of_new].reshape(-1)
    out = dict(sys)
    out.update(rowptr=rowptr, colidx=colidx, values=np.ascontiguousarray(values),
               diagslots=diagslots, rhs=np.ascontiguousarray(rhs))
    return out
