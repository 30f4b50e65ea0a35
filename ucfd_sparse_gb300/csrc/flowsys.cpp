// flowsys.cpp -- the FlowSys LU-SGS / BLU-SGS API (ucfdlusgs.h) on the GPU.
//
// Object model follows src/lusgs/flowsys.{h,c}: the handle keeps the
// caller's mesh/element pointers; work arrays are library-owned (here in
// device memory).  The rank cells are renumbered internally into a
// level-major order (graph.h) so that each level is a contiguous range of
// independent cells; all per-cell and per-cell-face arrays are stored with
// the internal cell index fastest (coalesced, one thread per cell).
#include <algorithm>
#include <cmath>
#include <memory>

#include "../../include/ucfdlusgs.h"
#include "graph.h"
#include "launch.h"
#include "ucfd_internal.h"

using namespace ucfd;

namespace {

struct Elem {
    int neles = 0, nface = 0;
    int *cell_ids = nullptr;
    double *uptsb = nullptr, *rhs = nullptr, *dt = nullptr, *dsrc = nullptr, *vol = nullptr,
           *resid_out = nullptr;
    DevBuf<int> s_ids;
    DevBuf<double> s_upts, s_rhs, s_dt, s_dsrc, s_vol, s_res;
};

enum { MODE_NONE = 0, MODE_LUSGS = 1, MODE_BLUSGS = 2 };

// Arrays of one precision (double for the FP64 modes, float for FP32).
template <typename S>
struct Work {
    DevBuf<S> fa, rv, nrm;                 // geometry (ELL)
    DevBuf<S> u, du, diag, base, lamN, lamT, rhs0;  // scalar LU-SGS
    DevBuf<S> rhs, bdu, dup, J, LU, tJ, tLU;        // block LU-SGS
    DevBuf<S> r, delta;                    // refinement
    DevBuf<S> fl_geo[2];                   // face lists (lower, upper): normal + fa * rv per entry
    DevBuf<S> ulo;                         // FP32 mode: low part of the float-float state u + ulo (UCFDLUSGS_Run)
    DevBuf<S> crhs;                        // fast modes: D^-1 rhs, the block sweeps' right-hand side
    DevBuf<S> spart;                       // fast modes: each block sweep's own-side sums (SweepSplit)
    DevBuf<float4> geo4;                   // FP32 run loop with both systems: (normal, fa * rv) per cell-face
    DevBuf<float2> lam2;                   // and (lam, tlam) per cell-face
};

// Which increments the fast block sweeps' stored sums (Work::spart) belong
// to: the sweeps into du in direction dir (0 lower, 1 upper) with the
// blocks of Prepare number ver.  The next sweep in the other direction
// into the same du reads them instead of forming that side again.
struct SplitState {
    const void *du = nullptr;
    int dir = -1;
    unsigned ver = 0;
};

}  // namespace

struct _FlowSys {
    int nlocal = 0, nvars = 0, nfvars = 0, ntvars = 0, ndims = 0, nfaces = 0, nelem = 0;
    int *rowptr = nullptr, *colidx = nullptr, *slots = nullptr;
    int8_t *sides = nullptr;
    double *face_area = nullptr, *face_normal = nullptr, *rcp_vol = nullptr;
    int mode = MODE_NONE;
    double *fspr = nullptr, *tfspr = nullptr, *jmat = nullptr, *tjmat = nullptr;
    std::vector<Elem> eles;

    int prec = UCFD_PREC_FP64;
    int block = 0;     // sweep threads per block (0: launcher default)
    int variant = 0;   // block sweep: 0 unrolled faces, 1 face loop
    int run_mode = 0;  // UCFDLUSGS_Run with mode -1
    double tuned_ms = 0;
    cudaStream_t own = nullptr, user = nullptr;
    bool async = false;

    std::vector<int> color;
    bool colored = false;

    // topology
    bool topo = false;
    long long N = 0;
    int P = 0;
    Schedule sch;
    DevBuf<int> d_iperm, d_nei, d_slot;
    DevBuf<int8_t> d_side;
    DevBuf<double> fa64, rv64;

    Work<double> w64;
    Work<float> w32;
    DevBuf<double> D, dd, LU64, tD, tLU64, J64, rhs64, x64;  // FP64 block arrays
    DevBuf<double> jt;  // Prepare scratch: face Jacobians, one record per face
    DevBuf<int> d_sweep_err;  // set by a bulk-copy block sweep whose copy wait gave up
    bool du64_valid = false;
    bool c_valid[2] = {false, false};  // crhs of the NS / turbulence rows matches rhs and the factors
    bool x_zero = false;  // the correction du is all zeros (Reset, no sweep since)
    SplitState split[2];           // NS / turbulence rows of the fast block sweeps
    unsigned jver[2] = {1, 1};     // Prepare count of the NS / turbulence blocks
    bool has_self = false;         // some CSR row lists itself
    bool lam2_ok = false;          // Work::lam2 packs the current NS and RANS spectral radii (FP32)
    DevBuf<double> part, red, resid;
    PinnedBuf<double> h_red;

    // CUDA graph of one scalar pseudo-time iteration
    cudaGraphExec_t run_exec = nullptr;
    int run_rans = -1;
    double run_kappa = 0;
    bool run_state = false;  // set by UCFDLUSGS_Run, cleared by Pack
    // scalar sweep variant 5: per sweep direction (lower, upper) the active
    // faces cell by cell -- offsets [N + 1], neighbour and ELL slot per entry
    DevBuf<int> fl_off[2], fl_nb[2], fl_q[2];
    // persistent sweeps: level offsets on the device, barrier {count, gen}, timeout flag
    DevBuf<int> d_lev_off, d_err;
    DevBuf<unsigned> d_bar;

    cudaStream_t stream() const { return user ? user : own; }
};

namespace {

void finish(FlowSys s, bool force_sync = false) {
    UCFD_CHECK_LAUNCH();
    if (!s->async || force_sync) UCFD_CUDA(cudaStreamSynchronize(s->stream()));
}

// Build the level schedule and the ELL mesh arrays (once).
void build_topology(FlowSys s) {
    if (s->topo) return;
    ensure_device();
    const int n = s->nlocal;
    std::vector<int> rp, ci, sl;
    std::vector<int8_t> sd;
    to_host(s->rowptr, (size_t)n + 1, rp);
    UCFD_REQUIRE(rp[0] == 0, "rowptr[0] must be 0");
    for (int i = 0; i < n; ++i) UCFD_REQUIRE(rp[i + 1] >= rp[i], "rowptr must be non-decreasing");
    const size_t nnz = (size_t)rp[n];
    to_host(s->colidx, nnz, ci);
    to_host(s->slots, nnz, sl);
    to_host(s->sides, nnz, sd);
    for (size_t p = 0; p < nnz; ++p) {
        UCFD_REQUIRE(ci[p] >= 0 && ci[p] < n, "colidx[%zu] = %d out of range", p, ci[p]);
        UCFD_REQUIRE(sl[p] >= 0 && sl[p] < s->nfaces, "slots[%zu] = %d out of range", p, sl[p]);
        UCFD_REQUIRE(sd[p] == 1 || sd[p] == -1, "sides[%zu] = %d must be +1 or -1", p, (int)sd[p]);
    }
    std::vector<double> fa, fn, rv;
    to_host(s->face_area, (size_t)s->nfaces, fa);
    to_host(s->face_normal, (size_t)s->nfaces * s->ndims, fn);
    to_host(s->rcp_vol, (size_t)n, rv);

    s->sch = s->colored ? schedule_colored(n, rp.data(), ci.data(), s->color.data())
                        : schedule_natural(n, rp.data(), ci.data());
    s->has_self = false;
    for (int i = 0; i < n && !s->has_self; ++i)
        for (int q = rp[i]; q < rp[i + 1]; ++q) s->has_self = s->has_self || ci[q] == i;
    // spatial locality inside each level (the cells of a level are
    // independent, so the order does not change any result)
    const std::vector<int> bfs = bfs_rank(n, rp.data(), ci.data());
    if (s->mode == MODE_BLUSGS) {
        // block LU-SGS: inside each level the cells with the same set of
        // faces towards earlier levels first come together (then breadth-
        // first), so the fast sweeps that skip the other side's faces skip
        // whole sectors of the block arrays
        std::vector<int> lev(n), mask(n, 0);
        for (int l = 0; l < s->sch.nlev; ++l)
            for (int k = s->sch.lev_off[l]; k < s->sch.lev_off[l + 1]; ++k) lev[s->sch.perm[k]] = l;
        for (int i = 0; i < n; ++i)
            for (int q = rp[i]; q < rp[i + 1] && q - rp[i] < 30; ++q)
                if (lev[ci[q]] < lev[i]) mask[i] |= 1 << (q - rp[i]);
        sort_levels_by(s->sch, mask, bfs);
    } else {
        sort_levels_by(s->sch, bfs);
    }
    const Schedule &sch = s->sch;
    int P = 0;
    for (int i = 0; i < n; ++i) P = std::max(P, rp[i + 1] - rp[i]);
    P = std::max(P, 1);
    const long long N = n;
    s->N = N;
    s->P = P;
    std::vector<int> nei((size_t)P * N, -1), slot((size_t)P * N, -1);
    std::vector<int8_t> side((size_t)P * N, 0);
    std::vector<double> efa((size_t)P * N, 0.0), erv(N), enrm((size_t)P * s->ndims * N, 0.0);
    for (long long k = 0; k < N; ++k) {
        const int r = sch.perm[k];
        erv[k] = rv[r];
        for (int p = 0; p < rp[r + 1] - rp[r]; ++p) {
            const int q = rp[r] + p;
            nei[p * N + k] = sch.iperm[ci[q]];
            slot[p * N + k] = sl[q];
            side[p * N + k] = sd[q];
            efa[p * N + k] = fa[sl[q]];
            for (int d = 0; d < s->ndims; ++d)
                enrm[(p * s->ndims + d) * N + k] = sd[q] * fn[sl[q] + (size_t)d * s->nfaces];
        }
    }
    cudaStream_t st = s->stream();
    s->d_iperm.upload(sch.iperm.data(), N, st);
    s->d_nei.upload(nei.data(), nei.size(), st);
    s->d_slot.upload(slot.data(), slot.size(), st);
    s->d_side.upload(side.data(), side.size(), st);
    s->fa64.upload(efa.data(), efa.size(), st);
    s->rv64.upload(erv.data(), erv.size(), st);
    s->w64.nrm.upload(enrm.data(), enrm.size(), st);
    if (s->prec == UCFD_PREC_FP32) {
        std::vector<float> f(efa.begin(), efa.end());
        s->w32.fa.upload(f.data(), f.size(), st);
        std::vector<float> g(erv.begin(), erv.end());
        s->w32.rv.upload(g.data(), g.size(), st);
        std::vector<float> h(enrm.begin(), enrm.end());
        s->w32.nrm.upload(h.data(), h.size(), st);
    }
    UCFD_CUDA(cudaStreamSynchronize(st));
    s->topo = true;
}

Elem &elem(FlowSys s, int eidx) {
    UCFD_REQUIRE(eidx >= 0 && eidx < s->nelem, "element index %d out of range [0, %d)", eidx, s->nelem);
    Elem &e = s->eles[eidx];
    UCFD_REQUIRE(e.neles > 0 && e.cell_ids, "element %d was not set (UCFDFlowSysSetElement)", eidx);
    return e;
}

const int *ids_view(FlowSys s, Elem &e) { return device_view<int>(e.cell_ids, e.neles, e.s_ids, s->stream()); }

template <typename S>
Work<S> &work(FlowSys s);
template <>
Work<double> &work<double>(FlowSys s) { return s->w64; }
template <>
Work<float> &work<float>(FlowSys s) { return s->w32; }

template <typename S>
const S *geo_fa(FlowSys s) {
    if constexpr (std::is_same<S, double>::value) return s->fa64.p;
    else return s->w32.fa.p;
}
template <typename S>
const S *geo_rv(FlowSys s) {
    if constexpr (std::is_same<S, double>::value) return s->rv64.p;
    else return s->w32.rv.p;
}

#define KCALL(EX, fn, ...)                         \
    do {                                           \
        if constexpr (EX) kexact::fn(__VA_ARGS__); \
        else kfast::fn(__VA_ARGS__);               \
    } while (0)

// Calls body.template operator()<S, EX>() with the precision of the handle.
template <typename F>
void dispatch(FlowSys s, F &&body) {
    switch (s->prec) {
        case UCFD_PREC_FP64: body.template operator()<double, true>(); break;
        case UCFD_PREC_FP64_FMA: body.template operator()<double, false>(); break;
        case UCFD_PREC_FP32: body.template operator()<float, false>(); break;
        default: fail(UCFD_ERR_STATE, "bad precision %d", s->prec);
    }
}

void need_mode(FlowSys s, int m) {
    UCFD_REQUIRE(s, "null FlowSys handle");
    if (s->mode != m)
        fail(UCFD_ERR_STATE, "FlowSys is not set up for %s (call UCFDFlowSysSet%s first)",
             m == MODE_LUSGS ? "LU-SGS" : "BLU-SGS", m == MODE_LUSGS ? "LUSGS" : "BLUSGS");
}

// ---- scalar LU-SGS --------------------------------------------------------
// Polls of the persistent kernel's grid barrier before it gives up (each
// poll sleeps ~64 ns): about a second, far beyond any legitimate wait.
constexpr long long kBarrierMaxSpin = 1ll << 24;
// Polls of a bulk copy's mbarrier before a block sweep gives up (each
// poll may suspend for a while): far beyond a copy's microseconds.
constexpr long long kBulkMaxSpin = 1ll << 20;

// Scalar sweep variant 5 (one thread per active face): the face lists of
// both sweep directions, built on the host from the level schedule at first
// use (never inside a stream capture: run_graph_build calls this first),
// and their geometry in the working precision.
template <typename S>
void ensure_face_lists(FlowSys s) {
    Work<S> &w = work<S>(s);
    if (w.fl_geo[0].p && w.fl_geo[1].p) return;
    cudaStream_t st = s->stream();
    const long long N = s->N;
    const int P = s->P;
    UCFD_REQUIRE((long long)P * N < (1ll << 31), "face-list sweep: %lld cell-faces exceed int32", (long long)P * N);
    if (!s->fl_nb[0].p || !s->fl_nb[1].p) {
        std::vector<int> nei((size_t)P * N);
        UCFD_CUDA(cudaMemcpyAsync(nei.data(), s->d_nei.p, nei.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
        UCFD_CUDA(cudaStreamSynchronize(st));
        std::vector<int> lev((size_t)N);
        for (int l = 0; l < s->sch.nlev; ++l)
            for (int k = s->sch.lev_off[l]; k < s->sch.lev_off[l + 1]; ++k) lev[k] = l;
        for (int dir = 0; dir < 2; ++dir) {
            std::vector<int> off((size_t)N + 1), nb, q;
            nb.reserve((size_t)P * N / 2 + 1);
            q.reserve((size_t)P * N / 2 + 1);
            for (long long k = 0; k < N; ++k) {
                off[k] = (int)nb.size();
                for (int p = 0; p < P; ++p) {
                    const int g = nei[(size_t)p * N + k];
                    if (g < 0) continue;
                    // active: the neighbour's level comes earlier in this sweep
                    if (dir == 0 ? lev[g] < lev[k] : lev[g] > lev[k]) {
                        nb.push_back(g);
                        q.push_back((int)(p * N + k));
                    }
                }
            }
            off[N] = (int)nb.size();
            s->fl_off[dir].upload(off.data(), off.size(), st);
            s->fl_nb[dir].upload(nb.data(), nb.size(), st);
            s->fl_q[dir].upload(q.data(), q.size(), st);
        }
    }
    for (int dir = 0; dir < 2; ++dir) {
        const long long E = (long long)s->fl_nb[dir].n;
        w.fl_geo[dir].ensure((size_t)4 * (E > 0 ? E : 1));
        kfast::face_list_geo<S>(E, N, s->ndims, s->fl_q[dir].p, w.nrm.p, geo_fa<S>(s), geo_rv<S>(s),
                                w.fl_geo[dir].p, st);
    }
    UCFD_CHECK_LAUNCH();
    UCFD_CUDA(cudaStreamSynchronize(st));
}

// sys: 0 the mean-flow system, 1 the turbulence system, 2 both in one pass
// (one thread per cell; the run loop's choice, see run_sweeps_both).
// packed: the run loop's sweep of both systems in FP32 reads the packed
// per cell-face geometry and spectral radii that run_gather_lambda formed.
template <typename S, bool EX>
void lusgs_sweep(FlowSys s, int sys, bool upper, double kappa, bool persistent = false, bool packed = false) {
    const bool rans = sys == 1;
    Work<S> &w = work<S>(s);
    const long long N = s->N;
    ScalarSweepArgs<S> a{};
    a.cells = nullptr;
    a.lcolor = nullptr;
    a.nface = s->P;
    a.ld = N;
    a.nei = s->d_nei.p;
    a.fa = geo_fa<S>(s);
    a.rv = geo_rv<S>(s);
    a.nrm = w.nrm.p;
    a.lam = rans ? w.lamT.p : w.lamN.p;
    a.tlam = sys == 2 ? w.lamT.p : nullptr;
    if (sys == 2 && packed && s->lam2_ok && w.geo4.p && w.lam2.p) {
        a.geo4 = w.geo4.p;
        a.lam2 = w.lam2.p;
    }
    a.u = w.u.p;
    a.nbsrc = w.du.p;
    a.own_in = w.du.p;
    a.own_out = w.du.p;
    a.diag = w.diag.p;
    a.diag_vs = N;
    a.kappa = (S)kappa;
    a.gamma = (S)constants().gamma;
    a.pmin = (S)constants().pmin;
    a.upper = upper ? 1 : 0;
    // scalar sweeps: variant 1 / 2 = the builds for 3 / 4 resident blocks of
    // 256 per SM; 3 / 4 = two threads per cell, default / 64-register build
    a.regcap = (s->variant == 1) ? 3 : (s->variant == 2 || s->variant == 4) ? 4 : 0;
    a.pair = (s->variant == 3 || s->variant == 4) && sys != 2 ? 1 : 0;
    // 5: one thread per active face, from the face lists
    a.facelist = (s->variant == 5 && !persistent && sys != 2) ? 1 : 0;
    if (a.facelist) {
        ensure_face_lists<S>(s);
        const int dir = upper ? 1 : 0;
        a.fl_off = s->fl_off[dir].p;
        a.fl_nb = s->fl_nb[dir].p;
        a.fl_q = s->fl_q[dir].p;
        a.fl_geo = w.fl_geo[dir].p;
    }
    const int L = s->sch.nlev;
    if (persistent) {
        // one cooperative launch per sweep, bounded grid barrier between levels
        a.t0 = a.t1 = a.lo = a.hi = 0;
        KCALL(EX, scalar_sweep_persistent<S>, a, s->nvars, s->nfvars, s->ndims, sys, s->d_lev_off.p, L,
              s->d_bar.p, s->d_err.p, kBarrierMaxSpin, s->stream());
        return;
    }
    for (int q = 0; q < L; ++q) {
        const int l = upper ? L - 1 - q : q;
        a.t0 = s->sch.lev_off[l];
        a.t1 = s->sch.lev_off[l + 1];
        a.lo = a.t0;
        a.hi = a.t1;
        KCALL(EX, scalar_sweep<S>, a, s->nvars, s->nfvars, s->ndims, sys, s->block, s->stream());
    }
}

template <typename S, bool EX>
void lusgs_prepare(FlowSys s, bool rans, double kappa, const S *base) {
    Work<S> &w = work<S>(s);
    KCALL(EX, fs_lusgs_prepare<S>, s->N, s->P, rans ? s->nfvars : 0, rans ? s->nvars : s->nfvars, (S)kappa,
          s->d_nei.p, geo_fa<S>(s), geo_rv<S>(s), rans ? w.lamT.p : w.lamN.p, base, w.diag.p, s->stream());
}

template <typename S>
void lusgs_alloc(FlowSys s) {
    Work<S> &w = work<S>(s);
    const long long n = (long long)s->nvars * s->N;
    w.u.ensure(n);
    w.du.ensure(n);
    w.diag.ensure(n);
    w.base.ensure(n);
    w.rhs0.ensure(n);
}

// ---- block LU-SGS -----------------------------------------------------------
template <typename S>
void blusgs_alloc(FlowSys s) {
    Work<S> &w = work<S>(s);
    const long long N = s->N, nv = s->nvars;
    w.rhs.ensure(nv * N);
    w.bdu.ensure(nv * N);
    w.dup.ensure(nv * N);
    // block arrays in the cell-tiled layout (whole tiles of 32 cells)
    const long long b2 = (long long)s->nfvars * s->nfvars;
    s->D.ensure(tiled_size(N, b2));
    s->dd.ensure(N);
    s->LU64.ensure(tiled_size(N, b2));
    w.J.ensure(tiled_size(N, (long long)s->P * b2));
    if (std::is_same<S, float>::value) {
        w.LU.ensure(tiled_size(N, b2));
        s->rhs64.ensure(nv * N);
        s->x64.ensure(nv * N);
    }
    if (s->ntvars > 0) {
        const long long t2 = (long long)s->ntvars * s->ntvars;
        s->tD.ensure(tiled_size(N, t2));
        s->tLU64.ensure(tiled_size(N, t2));
        w.tJ.ensure(tiled_size(N, (long long)s->P * t2));
        if (std::is_same<S, float>::value) w.tLU.ensure(tiled_size(N, t2));
    }
    if (!s->d_sweep_err.p) s->d_sweep_err.zero(1, s->stream());
}

// Bulk-copy sweeps report a copy wait that gave up through d_sweep_err;
// read (and clear) it at the points where the host synchronises anyway.
void check_sweep_err(FlowSys s) {
    if (!s->d_sweep_err.p) return;
    int err = 0;
    UCFD_CUDA(cudaMemcpyAsync(&err, s->d_sweep_err.p, sizeof(int), cudaMemcpyDeviceToHost, s->stream()));
    UCFD_CUDA(cudaStreamSynchronize(s->stream()));
    if (err) {
        s->d_sweep_err.zero(1, s->stream());
        fail(UCFD_ERR_TIMEOUT, "block sweep: a bulk copy into shared memory did not complete in time");
    }
}

template <typename S>
S *blu_rhs(FlowSys s) { return work<S>(s).rhs.p; }

template <typename S>
const S *blu_LU(FlowSys s, bool turb) {
    if constexpr (std::is_same<S, double>::value) return turb ? s->tLU64.p : s->LU64.p;
    else return turb ? s->w32.tLU.p : s->w32.LU.p;
}

// Right-hand side of the fast modes' block sweeps (their blocks are
// M = D^-1 J fv, so a sweep starts from D^-1 rhs): computed from the packed
// rhs when Pack or Prepare changed it; the exact mode sweeps rhs itself.
template <typename S, bool EX>
const S *sweep_rhs(FlowSys s, bool turb) {
    Work<S> &w = work<S>(s);
    if constexpr (EX) return w.rhs.p;
    const int B = turb ? s->ntvars : s->nfvars;
    const int var0 = turb ? s->nfvars : 0;
    if (!s->c_valid[turb ? 1 : 0]) {
        w.crhs.ensure((size_t)s->nvars * s->N);
        kfast::fs_blusgs_rhs_solve<S>(B, s->N, var0, blu_LU<S>(s, turb), w.rhs.p, w.crhs.p, s->stream());
        s->c_valid[turb ? 1 : 0] = true;
    }
    return w.crhs.p;
}

template <typename S, bool EX>
void blusgs_sweep_into(FlowSys s, bool turb, bool upper, const S *rhs, S *du) {
    Work<S> &w = work<S>(s);
    const int B = turb ? s->ntvars : s->nfvars;
    const int var0 = turb ? s->nfvars : 0;
    const int L = s->sch.nlev;
    SweepSplit<S> sp;
    if constexpr (!EX) {
        // the fast build's split sums: partial when the stored sums are the
        // previous opposite sweep's into the same du with the same blocks
        SplitState &ss = s->split[turb ? 1 : 0];
        sp.part = w.spart.ensure((size_t)s->nvars * s->N);
        sp.upper = upper ? 1 : 0;
        // (a face to the cell itself changes with the cell's own increment:
        // such meshes always sweep in full mode)
        sp.full = (!s->has_self && ss.du == du && ss.dir == (upper ? 0 : 1) && ss.ver == s->jver[turb ? 1 : 0])
                      ? 0 : 1;
    }
    for (int q = 0; q < L; ++q) {
        const int l = upper ? L - 1 - q : q;
        KCALL(EX, fs_blusgs_sweep<S>, B, s->sch.lev_off[l], s->sch.lev_off[l + 1], s->N, s->P, var0,
              s->d_nei.p, geo_fa<S>(s), geo_rv<S>(s), turb ? w.tJ.p : w.J.p, blu_LU<S>(s, turb), rhs, du,
              s->block, s->variant, s->d_sweep_err.p, kBulkMaxSpin, sp, s->stream());
    }
    if constexpr (!EX) s->split[turb ? 1 : 0] = SplitState{du, upper ? 1 : 0, s->jver[turb ? 1 : 0]};
}

// du of the fast block sweeps was set to zero: both sides' sums are zero,
// so the next lower sweep can start from stored (zero) sums.
template <typename S>
void split_zero(FlowSys s, bool turb, const S *du, cudaStream_t st) {
    Work<S> &w = work<S>(s);
    const int B = turb ? s->ntvars : s->nfvars;
    const int var0 = turb ? s->nfvars : 0;
    w.spart.ensure((size_t)s->nvars * s->N);
    UCFD_CUDA(cudaMemsetAsync(w.spart.p + (size_t)var0 * s->N, 0, (size_t)B * s->N * sizeof(S), st));
    s->split[turb ? 1 : 0] = SplitState{du, 1, s->jver[turb ? 1 : 0]};
}

void split_forget(FlowSys s) { s->split[0] = s->split[1] = SplitState{}; }

// FP64 residual of the NS block system for x; returns ||r|| and ||rhs||.
template <typename Sx, typename R, bool EX>
void blusgs_residual(FlowSys s, const Sx *x, R *r_out, double *rnorm, double *bnorm) {
    const int nbmax = (int)((s->N + 255) / 256) + 1;
    s->part.ensure((size_t)2 * nbmax);
    s->red.ensure(2);
    const double *J64 = s->prec == UCFD_PREC_FP32 ? s->J64.p : s->w64.J.p;
    const double *rhs64 = s->prec == UCFD_PREC_FP32 ? s->rhs64.p : s->w64.rhs.p;
    // the FMA mode's blocks are M = D^-1 J fv (nullptr face areas)
    const double *fa = s->prec == UCFD_PREC_FP64_FMA ? nullptr : s->fa64.p;
    int nb = 0;
    if constexpr (EX)
        kexact::fs_blusgs_residual<Sx, R>(s->nfvars, s->N, s->P, 0, s->nvars, s->d_nei.p, fa, s->rv64.p,
                                          J64, s->D.p, rhs64, x, r_out, s->part.p, nbmax, &nb, s->stream());
    else
        kfast::fs_blusgs_residual<Sx, R>(s->nfvars, s->N, s->P, 0, s->nvars, s->d_nei.p, fa, s->rv64.p,
                                         J64, s->D.p, rhs64, x, r_out, s->part.p, nbmax, &nb, s->stream());
    kfast::pair_reduce(nb, s->part.p, s->red.p, s->stream());
    double *h = s->h_red.ensure(2);
    UCFD_CUDA(cudaMemcpyAsync(h, s->red.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s->stream()));
    UCFD_CUDA(cudaStreamSynchronize(s->stream()));
    check_sweep_err(s);
    *rnorm = std::sqrt(h[0]);
    *bnorm = std::sqrt(h[1]);
}

}  // namespace

namespace {
// Whether a run loop with the turbulence system sweeps both systems in one
// pass per level: with one thread per cell (launch variants 0-2 and the
// persistent kernel).  The two systems' sweeps read only the state and
// their own increments, so sweeping them together gives the values of
// NS Prepare, lower, upper, then RANS Prepare, lower, upper, while every
// neighbour index, face normal, area and mean-flow state is loaded once
// instead of twice.
bool run_sweeps_both(FlowSys s, bool persistent) {
    return s->ntvars > 0 && (persistent || s->variant <= 2);
}

// One pseudo-time iteration on device-resident state (see UCFDLUSGS_Run).
template <typename S, bool EX>
void lusgs_iteration(FlowSys s, bool rans, double kappa, double *resid_slot, bool persistent) {
    Work<S> &w = work<S>(s);
    cudaStream_t st = s->stream();
    const size_t n = (size_t)s->nvars * s->N;
    UCFD_CUDA(cudaMemcpyAsync(w.du.p, w.rhs0.p, n * sizeof(S), cudaMemcpyDeviceToDevice, st));
    if (rans && run_sweeps_both(s, persistent)) {
        KCALL(EX, fs_lusgs_prepare_both<S>, s->N, s->P, s->nfvars, s->nvars, (S)kappa, s->d_nei.p, geo_fa<S>(s),
              geo_rv<S>(s), w.lamN.p, w.lamT.p, w.base.p, w.diag.p, st);
        lusgs_sweep<S, EX>(s, 2, false, kappa, persistent, true);
        lusgs_sweep<S, EX>(s, 2, true, kappa, persistent, true);
    } else {
        lusgs_prepare<S, EX>(s, false, kappa, w.base.p);
        lusgs_sweep<S, EX>(s, 0, false, kappa, persistent);
        lusgs_sweep<S, EX>(s, 0, true, kappa, persistent);
        if (rans) {
            lusgs_prepare<S, EX>(s, true, kappa, w.base.p);
            lusgs_sweep<S, EX>(s, 1, false, kappa, persistent);
            lusgs_sweep<S, EX>(s, 1, true, kappa, persistent);
        }
    }
    // u += du over the swept variables, ||du|| in FP64; FP32 mode adds into
    // the FP64 master state and rounds the working copy from it
    const int v1 = rans ? s->nvars : s->nfvars;
    if constexpr (std::is_same<S, float>::value)
        kfast::axpy_master((long long)v1 * s->N, w.du.p, w.u.p, w.ulo.p, s->part.p, resid_slot, st);
    else
        kfast::axpy_norm<S>((long long)v1 * s->N, w.du.p, w.u.p, s->part.p, resid_slot, st);
}

void run_graph_drop(FlowSys s) {
    if (s->run_exec) cudaGraphExecDestroy(s->run_exec);
    s->run_exec = nullptr;
}

// The packed per cell-face geometry and both spectral radii of the FP32
// sweeps of both systems, from lamN and lamT as just gathered.
template <typename S>
void pack_both(FlowSys s, cudaStream_t st) {
    if constexpr (std::is_same<S, float>::value) {
        Work<S> &w = work<S>(s);
        const long long nl = (long long)s->P * s->N;
        if (!w.geo4.p) {
            w.geo4.ensure((size_t)nl);
            kfast::pack_geo4(s->N, s->P, s->ndims, w.nrm.p, geo_fa<S>(s), geo_rv<S>(s), w.geo4.p, st);
        }
        w.lam2.ensure((size_t)nl);
        kfast::pack_lam2(nl, w.lamN.p, w.lamT.p, w.lam2.p, st);
        s->lam2_ok = true;
    }
}

// Spectral radii of the loop, gathered from the face arrays (fspr / tfspr)
// into the ELL layout, and the scratch of the loop's norms.
template <typename S>
void run_gather_lambda(FlowSys s, bool rans, int niter) {
    static thread_local DevBuf<double> stage;
    cudaStream_t st = s->stream();
    Work<S> &w = work<S>(s);
    s->part.ensure(4096);
    s->red.ensure(4);
    s->resid.ensure((size_t)std::max(niter, 1));
    w.lamN.ensure((size_t)s->P * s->N);
    kfast::gather_idx<S>((long long)s->P * s->N, s->d_slot.p, device_view<double>(s->fspr, s->nfaces, stage, st),
                         w.lamN.p, st);
    s->lam2_ok = false;
    if (rans) {
        w.lamT.ensure((size_t)s->P * s->N);
        kfast::gather_idx<S>((long long)s->P * s->N, s->d_slot.p, device_view<double>(s->tfspr, s->nfaces, stage, st),
                             w.lamT.p, st);
        // FP32 loop sweeping both systems: the geometry (fixed with the mesh)
        // and both spectral radii packed per cell-face, so a face costs two
        // vector loads instead of six
        pack_both<S>(s, st);
    }
}


// One iteration captured once per (rans, kappa, launch shape) and replayed.
template <typename S, bool EX>
void run_graph_build(FlowSys s, bool rans, double kappa) {
    if (s->run_exec && s->run_rans == (int)rans && s->run_kappa == kappa) return;
    run_graph_drop(s);
    cudaStream_t st = s->stream();
    if (s->variant == 5) ensure_face_lists<S>(s);  // host work: before the capture
    UCFD_CUDA(cudaStreamSynchronize(st));
    cudaGraph_t g;
    UCFD_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
        lusgs_iteration<S, EX>(s, rans, kappa, s->red.p, false);
    } catch (...) {
        cudaStreamEndCapture(st, &g);
        throw;
    }
    UCFD_CUDA(cudaStreamEndCapture(st, &g));
    UCFD_CUDA(cudaGraphInstantiate(&s->run_exec, g, 0));
    cudaGraphDestroy(g);
    s->run_rans = rans;
    s->run_kappa = kappa;
}

// Persistent sweeps: barrier state and timeout flag start cleared ...
void run_persistent_begin(FlowSys s) {
    cudaStream_t st = s->stream();
    if (!s->d_lev_off.p) s->d_lev_off.upload(s->sch.lev_off.data(), s->sch.lev_off.size(), st);
    s->d_bar.zero(2, st);
    s->d_err.zero(1, st);
}

// ... and a barrier wait that gave up is reported after the launches.
void run_persistent_check(FlowSys s) {
    int err = 0;
    UCFD_CUDA(cudaMemcpyAsync(&err, s->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, s->stream()));
    UCFD_CUDA(cudaStreamSynchronize(s->stream()));
    if (err) fail(UCFD_ERR_TIMEOUT, "persistent sweep: a grid barrier wait timed out");
}

// Mean device time (ms) of fn over reps calls after one untimed call.
struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    EventPair() {
        UCFD_CUDA(cudaEventCreate(&a));
        UCFD_CUDA(cudaEventCreate(&b));
    }
    ~EventPair() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

template <typename F>
double time_ms(cudaStream_t st, int reps, F &&fn) {
    fn();
    EventPair ev;
    UCFD_CUDA(cudaEventRecord(ev.a, st));
    for (int r = 0; r < reps; ++r) fn();
    UCFD_CUDA(cudaEventRecord(ev.b, st));
    UCFD_CUDA(cudaEventSynchronize(ev.b));
    UCFD_CHECK_LAUNCH();
    float ms = 0.f;
    UCFD_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
    return (double)ms / reps;
}

constexpr int kTuneBlocks[] = {64, 128, 192, 256};

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

ucfd_status_t UCFDFlowSysCreate(FlowSys *sys, UCFDInt nlocal, UCFDInt nvars, UCFDInt nfvars, UCFDInt ndims,
                                UCFDInt nfaces, UCFDInt nelem, UCFDInt *rowptr, UCFDInt *colidx, UCFDInt *slots,
                                UCFDInt8 *sides, UCFDReal *face_area, UCFDReal *face_normal, UCFDReal *rcp_vol) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(sys, "null FlowSys pointer");
    *sys = nullptr;
    UCFD_REQUIRE(nlocal > 0 && nvars > 0 && nfvars > 0 && nfvars <= nvars && nvars <= 16,
                 "bad sizes nlocal=%d nvars=%d nfvars=%d", nlocal, nvars, nfvars);
    UCFD_REQUIRE(ndims == 2 || ndims == 3, "ndims must be 2 or 3 (got %d)", ndims);
    UCFD_REQUIRE(nfaces > 0 && nelem > 0, "bad sizes nfaces=%d nelem=%d", nfaces, nelem);
    UCFD_REQUIRE(rowptr && colidx && slots && sides && face_area && face_normal && rcp_vol,
                 "null mesh array");
    ensure_device();
    std::unique_ptr<_FlowSys> s(new _FlowSys());
    s->nlocal = nlocal;
    s->nvars = nvars;
    s->nfvars = nfvars;
    s->ntvars = nvars - nfvars;
    s->ndims = ndims;
    s->nfaces = nfaces;
    s->nelem = nelem;
    s->rowptr = rowptr;
    s->colidx = colidx;
    s->slots = slots;
    s->sides = sides;
    s->face_area = face_area;
    s->face_normal = face_normal;
    s->rcp_vol = rcp_vol;
    s->eles.resize(nelem);
    UCFD_CUDA(cudaStreamCreateWithFlags(&s->own, cudaStreamNonBlocking));
    *sys = s.release();
    UCFD_API_END
}

ucfd_status_t UCFDFlowSysSetElement(FlowSys *sys, UCFDInt eidx, UCFDInt neles, UCFDInt nface, UCFDInt *cell_ids,
                                    UCFDReal *uptsb, UCFDReal *rhs, UCFDReal *dt, UCFDReal *dsrc, UCFDReal *vol,
                                    UCFDReal *resid_out) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(sys && *sys, "null FlowSys handle");
    FlowSys s = *sys;
    UCFD_REQUIRE(eidx >= 0 && eidx < s->nelem, "element index %d out of range", eidx);
    UCFD_REQUIRE(neles > 0 && cell_ids, "element %d: neles must be positive and cell_ids non-null", eidx);
    Elem &e = s->eles[eidx];
    e.neles = neles;
    e.nface = nface;
    e.cell_ids = cell_ids;
    e.uptsb = uptsb;
    e.rhs = rhs;
    e.dt = dt;
    e.dsrc = dsrc;
    e.vol = vol;
    e.resid_out = resid_out;
    UCFD_API_END
}

ucfd_status_t UCFDFlowSysDestroy(FlowSys *sys) {
    UCFD_API_BEGIN
    if (!sys || !*sys) return UCFD_SUCCESS;
    FlowSys s = *sys;
    if (s->own) cudaStreamSynchronize(s->own);
    if (s->run_exec) cudaGraphExecDestroy(s->run_exec);
    if (s->own) cudaStreamDestroy(s->own);
    delete s;
    *sys = nullptr;
    UCFD_API_END
}

ucfd_status_t UCFDFlowSysSetColoring(FlowSys s, const UCFDInt *color) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(s, "null FlowSys handle");
    UCFD_REQUIRE(!s->topo, "the colouring must be set before the first Prepare or sweep");
    if (!color) {
        s->colored = false;
        s->color.clear();
    } else {
        to_host(color, (size_t)s->nlocal, s->color);
        s->colored = true;
    }
    UCFD_API_END
}

ucfd_status_t UCFDFlowSysColorGreedy(FlowSys s, UCFDInt *ncolors) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(s, "null FlowSys handle");
    UCFD_REQUIRE(!s->topo, "the colouring must be set before the first Prepare or sweep");
    std::vector<int> rp, ci;
    to_host(s->rowptr, (size_t)s->nlocal + 1, rp);
    to_host(s->colidx, (size_t)rp[s->nlocal], ci);
    int nc = 0;
    s->color = greedy_color_csr(s->nlocal, rp.data(), ci.data(), &nc);
    s->colored = true;
    if (ncolors) *ncolors = nc;
    UCFD_API_END
}

ucfd_status_t UCFDFlowSysGetLevels(FlowSys s, UCFDInt *nlevels) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(s && nlevels, "null argument");
    build_topology(s);
    *nlevels = s->sch.nlev;
    UCFD_API_END
}

ucfd_status_t UCFDFlowSysSetPrecision(FlowSys s, int precision) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(s, "null FlowSys handle");
    UCFD_REQUIRE(precision == UCFD_PREC_FP64 || precision == UCFD_PREC_FP64_FMA || precision == UCFD_PREC_FP32,
                 "unknown precision %d", precision);
    UCFD_REQUIRE(!s->topo, "precision must be set before the first Prepare or sweep");
    s->prec = precision;
    UCFD_API_END
}

ucfd_status_t UCFDFlowSysSetLaunch(FlowSys s, int threads_per_block) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(s, "null FlowSys handle");
    UCFD_REQUIRE(threads_per_block == 0 || (threads_per_block % 32 == 0 && threads_per_block <= 256),
                 "threads_per_block must be 0 or a multiple of 32 up to 256");
    s->block = threads_per_block;
    run_graph_drop(s);
    UCFD_API_END
}

ucfd_status_t UCFDFlowSysGetLaunchConfig(FlowSys s, UCFDLaunchConfig *cfg) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(s && cfg, "null argument");
    cfg->threads_per_block = s->block;
    cfg->sweep_variant = s->variant;
    cfg->run_mode = s->run_mode;
    cfg->ms = s->tuned_ms;
    UCFD_API_END
}

ucfd_status_t UCFDFlowSysSetLaunchConfig(FlowSys s, const UCFDLaunchConfig *cfg) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(s && cfg, "null argument");
    const int b = cfg->threads_per_block;
    UCFD_REQUIRE(b == 0 || (b % 32 == 0 && b >= 32 && b <= 256),
                 "threads_per_block must be 0 or a multiple of 32 up to 256 (got %d)", b);
    UCFD_REQUIRE(cfg->sweep_variant >= 0 && cfg->sweep_variant <= 5, "sweep_variant must be 0..5");
    UCFD_REQUIRE(cfg->run_mode == 0 || cfg->run_mode == 1, "run_mode must be 0 or 1");
    if (b != s->block || cfg->sweep_variant != s->variant) run_graph_drop(s);
    s->block = b;
    s->variant = cfg->sweep_variant;
    s->run_mode = cfg->run_mode;
    s->tuned_ms = 0;
    UCFD_API_END
}

ucfd_status_t UCFDFlowSysAutotune(FlowSys s, int reps, UCFDLaunchConfig *best) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(s, "null FlowSys handle");
    UCFD_REQUIRE(reps >= 1 && reps <= 1000, "reps must be in [1, 1000]");
    UCFD_REQUIRE(s->mode == MODE_LUSGS || s->mode == MODE_BLUSGS, "Autotune needs SetLUSGS or SetBLUSGS first");
    build_topology(s);
    cudaStream_t st = s->stream();
    UCFD_CUDA(cudaStreamSynchronize(st));
    double best_ms = -1;
    int best_block = s->block, best_var = s->variant, best_mode = s->run_mode;
    // a failed candidate leaves the launch configuration as it was
    struct Keep {
        FlowSys s;
        int b, v;
        bool done = false;
        ~Keep() {
            if (!done) {
                s->block = b;
                s->variant = v;
                run_graph_drop(s);
            }
        }
    } keep{s, s->block, s->variant};
    auto consider = [&](double ms, int b, int v, int m) {
        if (best_ms < 0 || ms < best_ms) {
            best_ms = ms;
            best_block = b;
            best_var = v;
            best_mode = m;
        }
    };
    const size_t n = (size_t)s->nvars * s->N;
    if (s->mode == MODE_BLUSGS) {
        dispatch(s, [&]<typename S, bool EX>() {
            Work<S> &w = work<S>(s);
            UCFD_REQUIRE(w.rhs.p && w.J.p && blu_LU<S>(s, false), "Autotune before Pack and NSPrepare");
            DevBuf<S> scratch;
            scratch.zero(n, st);
            auto pair_ms = [&] {
                return time_ms(st, reps, [&] {
                    blusgs_sweep_into<S, EX>(s, false, false, w.rhs.p, scratch.p);
                    blusgs_sweep_into<S, EX>(s, false, true, w.rhs.p, scratch.p);
                });
            };
            // the unrolled kernels exist for ELL widths 6 and 4 only
            const bool unrolled = s->P == 6 || s->P == 4;
            for (int v : {0, 1, 4}) {
                if (v != 0 && !unrolled) continue;
                for (int b : kTuneBlocks) {
                    s->block = b;
                    s->variant = v;
                    consider(pair_ms(), b, v, s->run_mode);
                }
            }
            // bulk-copy kernels (FP32, 5x5 blocks): fixed launch shape
            if (std::is_same<S, float>::value && unrolled && s->nfvars == 5) {
                for (int v = 2; v <= 3; ++v) {
                    s->block = 0;
                    s->variant = v;
                    consider(pair_ms(), 0, v, s->run_mode);
                }
                check_sweep_err(s);
            }
        });
    } else {
        UCFD_REQUIRE(s->fspr, "fspr is not set");
        dispatch(s, [&]<typename S, bool EX>() {
            Work<S> &w = work<S>(s);
            UCFD_REQUIRE(w.u.p, "Autotune before Pack");
            // the loop of the handle's systems: with the turbulence system
            // when its spectral radius is set
            const bool rans = s->ntvars > 0 && s->tfspr;
            // the loop writes u, du, diag and the spectral radii: keep them
            DevBuf<S> su, sdu, sdiag, slam, slamT;
            DevBuf<S> sulo;
            const size_t nl = (size_t)s->P * s->N;
            const bool had_lam = w.lamN.p != nullptr;
            const bool had_lamT = w.lamT.p != nullptr;
            su.ensure(n);
            sdu.ensure(n);
            sdiag.ensure(n);
            if (w.ulo.p) {
                sulo.ensure(n);
                UCFD_CUDA(cudaMemcpyAsync(sulo.p, w.ulo.p, n * sizeof(S), cudaMemcpyDeviceToDevice, st));
            }
            UCFD_CUDA(cudaMemcpyAsync(su.p, w.u.p, n * sizeof(S), cudaMemcpyDeviceToDevice, st));
            UCFD_CUDA(cudaMemcpyAsync(sdu.p, w.du.p, n * sizeof(S), cudaMemcpyDeviceToDevice, st));
            UCFD_CUDA(cudaMemcpyAsync(sdiag.p, w.diag.p, n * sizeof(S), cudaMemcpyDeviceToDevice, st));
            if (had_lam) {
                slam.ensure(nl);
                UCFD_CUDA(cudaMemcpyAsync(slam.p, w.lamN.p, nl * sizeof(S), cudaMemcpyDeviceToDevice, st));
            }
            if (rans && had_lamT) {
                slamT.ensure(nl);
                UCFD_CUDA(cudaMemcpyAsync(slamT.p, w.lamT.p, nl * sizeof(S), cudaMemcpyDeviceToDevice, st));
            }
            run_gather_lambda<S>(s, rans, 1);
            // variant 0: unconstrained registers; 1 / 2: at most 80 / 64 registers;
            // 3 / 4: two threads per cell; 5: one thread per active face (the
            // persistent kernel stays one per cell)
            for (int v = 0; v <= 5; ++v) {
                s->variant = v;
                for (int b : kTuneBlocks) {
                    s->block = b;
                    run_graph_drop(s);
                    run_graph_build<S, EX>(s, rans, 1.0);
                    const double ms = time_ms(st, reps, [&] { UCFD_CUDA(cudaGraphLaunch(s->run_exec, st)); });
                    consider(ms, b, v, 0);
                }
                run_graph_drop(s);
                if (v > 2) continue;
                // the persistent kernel has its own fixed launch shape
                run_persistent_begin(s);
                const double pms =
                    time_ms(st, reps, [&] { lusgs_iteration<S, EX>(s, rans, 1.0, s->red.p, true); });
                run_persistent_check(s);
                consider(pms, 256, v, 1);
            }
            UCFD_CUDA(cudaMemcpyAsync(w.u.p, su.p, n * sizeof(S), cudaMemcpyDeviceToDevice, st));
            if (w.ulo.p) UCFD_CUDA(cudaMemcpyAsync(w.ulo.p, sulo.p, n * sizeof(S), cudaMemcpyDeviceToDevice, st));
            UCFD_CUDA(cudaMemcpyAsync(w.du.p, sdu.p, n * sizeof(S), cudaMemcpyDeviceToDevice, st));
            UCFD_CUDA(cudaMemcpyAsync(w.diag.p, sdiag.p, n * sizeof(S), cudaMemcpyDeviceToDevice, st));
            if (had_lam) UCFD_CUDA(cudaMemcpyAsync(w.lamN.p, slam.p, nl * sizeof(S), cudaMemcpyDeviceToDevice, st));
            if (rans && had_lamT)
                UCFD_CUDA(cudaMemcpyAsync(w.lamT.p, slamT.p, nl * sizeof(S), cudaMemcpyDeviceToDevice, st));
            UCFD_CUDA(cudaStreamSynchronize(st));
            if (!had_lam) w.lamN.release();
            if (rans && !had_lamT) w.lamT.release();
        });
    }
    keep.done = true;
    split_forget(s);  // the candidates swept into scratch buffers
    s->block = best_block;
    s->variant = best_var;
    s->run_mode = best_mode;
    s->tuned_ms = best_ms;
    run_graph_drop(s);
    if (best) {
        best->threads_per_block = best_block;
        best->sweep_variant = best_var;
        best->run_mode = best_mode;
        best->ms = best_ms;
    }
    UCFD_API_END
}

ucfd_status_t UCFDFlowSysSetStream(FlowSys s, void *cuda_stream, int async) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(s, "null FlowSys handle");
    UCFD_CUDA(cudaStreamSynchronize(s->stream()));
    s->user = (cudaStream_t)cuda_stream;
    s->async = cuda_stream && async;
    UCFD_API_END
}

// ---- scalar LU-SGS (lusgs.c) ------------------------------------------------
ucfd_status_t UCFDFlowSysSetLUSGS(FlowSys *sys, UCFDReal *fspr, UCFDReal *tfspr) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(sys && *sys, "null FlowSys handle");
    UCFD_REQUIRE(fspr, "fspr must not be null");
    FlowSys s = *sys;
    UCFD_REQUIRE(s->mode == MODE_NONE || s->mode == MODE_LUSGS, "FlowSys already set up for BLU-SGS");
    s->mode = MODE_LUSGS;
    s->fspr = fspr;
    s->tfspr = tfspr;
    UCFD_API_END
}

ucfd_status_t UCFDLUSGS_Pack(FlowSys s, UCFDInt eidx, UCFDReal turb_factor, UCFDReal a0) {
    UCFD_API_BEGIN
    need_mode(s, MODE_LUSGS);
    build_topology(s);
    Elem &e = elem(s, eidx);
    UCFD_REQUIRE(e.uptsb && e.rhs && e.dt && e.dsrc, "element %d: uptsb, rhs, dt and dsrc are needed by Pack", eidx);
    cudaStream_t st = s->stream();
    const size_t nv = (size_t)s->nvars * e.neles;
    const int *ids = ids_view(s, e);
    const double *up = device_view<double>(e.uptsb, nv, e.s_upts, st);
    const double *rh = device_view<double>(e.rhs, nv, e.s_rhs, st);
    const double *dt = device_view<double>(e.dt, e.neles, e.s_dt, st);
    const double *ds = device_view<double>(e.dsrc, nv, e.s_dsrc, st);
    dispatch(s, [&]<typename S, bool EX>() {
        lusgs_alloc<S>(s);
        Work<S> &w = work<S>(s);
        KCALL(EX, fs_lusgs_pack<S>, e.neles, s->nvars, s->nfvars, s->N, turb_factor, a0, ids, s->d_iperm.p, up, rh,
              dt, ds, w.u.p, w.du.p, w.diag.p, st);
        if constexpr (std::is_same<S, float>::value) {
            w.ulo.ensure((size_t)s->nvars * s->N);
            kfast::state_lo_pack(e.neles, s->nvars, s->N, ids, s->d_iperm.p, up, w.ulo.p, st);
        }
        const size_t n = (size_t)s->nvars * s->N;
        UCFD_CUDA(cudaMemcpyAsync(w.base.p, w.diag.p, n * sizeof(S), cudaMemcpyDeviceToDevice, st));
        UCFD_CUDA(cudaMemcpyAsync(w.rhs0.p, w.du.p, n * sizeof(S), cudaMemcpyDeviceToDevice, st));
    });
    s->run_state = false;
    finish(s, !is_device_ptr(e.uptsb));
    UCFD_API_END
}

ucfd_status_t UCFDLUSGS_Update(FlowSys s, UCFDInt eidx) {
    UCFD_API_BEGIN
    need_mode(s, MODE_LUSGS);
    build_topology(s);
    Elem &e = elem(s, eidx);
    UCFD_REQUIRE(e.uptsb, "element %d: uptsb is null", eidx);
    cudaStream_t st = s->stream();
    const size_t nv = (size_t)s->nvars * e.neles;
    const int *ids = ids_view(s, e);
    const bool dev = is_device_ptr(e.uptsb);
    double *up = dev ? e.uptsb : const_cast<double *>(device_view<double>(e.uptsb, nv, e.s_upts, st));
    dispatch(s, [&]<typename S, bool EX>() {
        Work<S> &w = work<S>(s);
        UCFD_REQUIRE(w.du.p, "Update before Pack");
        // after UCFDLUSGS_Run the device-resident state itself is written back
        // (FP32 mode: its float-float pair, summed in FP64)
        if constexpr (std::is_same<S, float>::value) {
            if (s->run_state) {
                kfast::state_ff_update(e.neles, s->nvars, s->N, ids, s->d_iperm.p, w.u.p, w.ulo.p, up, st);
                return;
            }
        }
        KCALL(EX, fs_lusgs_update<S>, e.neles, s->nvars, s->N, ids, s->d_iperm.p, s->run_state ? w.u.p : w.du.p, up,
              s->run_state ? 1 : 0, st);
    });
    if (!dev) copy_d2h(e.uptsb, up, nv * sizeof(double), st);
    finish(s, !dev);
    UCFD_API_END
}

// sys: 0 mean-flow system (NS*), 1 turbulence system (RANS*), 2 both
// (NSRANS*: one kernel over the faces, the values of NS* then RANS*).
static ucfd_status_t lusgs_prepare_api(FlowSys s, int sys, UCFDReal kappa) {
    UCFD_API_BEGIN
    need_mode(s, MODE_LUSGS);
    build_topology(s);
    UCFD_REQUIRE(sys == 1 || s->fspr, "fspr is not set");
    UCFD_REQUIRE(sys == 0 || s->tfspr, "tfspr is not set");
    if (sys != 0) UCFD_REQUIRE(s->ntvars > 0, "RANS prepare needs turbulence variables (nvars > nfvars)");
    cudaStream_t st = s->stream();
    static thread_local DevBuf<double> stageN, stageT;
    const double *lfN = sys != 1 ? device_view<double>(s->fspr, (size_t)s->nfaces, stageN, st) : nullptr;
    const double *lfT = sys != 0 ? device_view<double>(s->tfspr, (size_t)s->nfaces, stageT, st) : nullptr;
    dispatch(s, [&]<typename S, bool EX>() {
        Work<S> &w = work<S>(s);
        UCFD_REQUIRE(w.diag.p, "Prepare before Pack");
        const long long nl = (long long)s->P * s->N;
        if (lfN) {
            w.lamN.ensure((size_t)nl);
            kfast::gather_idx<S>(nl, s->d_slot.p, lfN, w.lamN.p, st);
        }
        if (lfT) {
            w.lamT.ensure((size_t)nl);
            kfast::gather_idx<S>(nl, s->d_slot.p, lfT, w.lamT.p, st);
        }
        s->lam2_ok = false;
        if (sys == 2) {
            KCALL(EX, fs_lusgs_prepare_both<S>, s->N, s->P, s->nfvars, s->nvars, (S)kappa, s->d_nei.p, geo_fa<S>(s),
                  geo_rv<S>(s), w.lamN.p, w.lamT.p, (const S *)nullptr, w.diag.p, st);
            pack_both<S>(s, st);
        } else {
            lusgs_prepare<S, EX>(s, sys == 1, kappa, nullptr);
        }
    });
    finish(s, (lfN && !is_device_ptr(s->fspr)) || (lfT && !is_device_ptr(s->tfspr)));
    UCFD_API_END
}

static ucfd_status_t lusgs_sweep_api(FlowSys s, int sys, bool upper, UCFDReal kappa) {
    UCFD_API_BEGIN
    need_mode(s, MODE_LUSGS);
    build_topology(s);
    if (sys != 0) UCFD_REQUIRE(s->ntvars > 0, "RANS sweep needs turbulence variables (nvars > nfvars)");
    dispatch(s, [&]<typename S, bool EX>() {
        Work<S> &w = work<S>(s);
        UCFD_REQUIRE(w.du.p, "sweep before Pack");
        UCFD_REQUIRE(sys == 1 || w.lamN.p, "sweep before NSPrepare");
        UCFD_REQUIRE(sys == 0 || w.lamT.p, "sweep before RANSPrepare");
        if (sys == 2 && s->variant > 2) {
            // the one-pass kernel is one thread per cell; the other launch
            // variants sweep the two systems one after the other
            lusgs_sweep<S, EX>(s, 0, upper, kappa);
            lusgs_sweep<S, EX>(s, 1, upper, kappa);
        } else {
            lusgs_sweep<S, EX>(s, sys, upper, kappa, false, sys == 2);
        }
    });
    finish(s);
    UCFD_API_END
}

ucfd_status_t UCFDLUSGS_NSPrepare(FlowSys s, UCFDReal kappa) { return lusgs_prepare_api(s, 0, kappa); }
ucfd_status_t UCFDLUSGS_RANSPrepare(FlowSys s, UCFDReal kappa) { return lusgs_prepare_api(s, 1, kappa); }
ucfd_status_t UCFDLUSGS_NSLowerSweep(FlowSys s, UCFDReal kappa) { return lusgs_sweep_api(s, 0, false, kappa); }
ucfd_status_t UCFDLUSGS_NSUpperSweep(FlowSys s, UCFDReal kappa) { return lusgs_sweep_api(s, 0, true, kappa); }
ucfd_status_t UCFDLUSGS_RANSLowerSweep(FlowSys s, UCFDReal kappa) { return lusgs_sweep_api(s, 1, false, kappa); }
ucfd_status_t UCFDLUSGS_RANSUpperSweep(FlowSys s, UCFDReal kappa) { return lusgs_sweep_api(s, 1, true, kappa); }
ucfd_status_t UCFDLUSGS_NSRANSPrepare(FlowSys s, UCFDReal kappa) { return lusgs_prepare_api(s, 2, kappa); }
ucfd_status_t UCFDLUSGS_NSRANSLowerSweep(FlowSys s, UCFDReal kappa) { return lusgs_sweep_api(s, 2, false, kappa); }
ucfd_status_t UCFDLUSGS_NSRANSUpperSweep(FlowSys s, UCFDReal kappa) { return lusgs_sweep_api(s, 2, true, kappa); }

ucfd_status_t UCFDLUSGS_Run(FlowSys s, UCFDInt niter, UCFDReal kappa, int rans, int mode, UCFDReal *resid) {
    UCFD_API_BEGIN
    need_mode(s, MODE_LUSGS);
    build_topology(s);
    UCFD_REQUIRE(niter >= 0, "niter must be >= 0");
    UCFD_REQUIRE(mode == -1 || mode == 0 || mode == 1,
                 "mode must be 0 (graph), 1 (persistent) or -1 (launch configuration)");
    if (mode == -1) mode = s->run_mode;
    if (rans) UCFD_REQUIRE(s->ntvars > 0 && s->tfspr, "RANS loop needs turbulence variables and tfspr");
    cudaStream_t st = s->stream();
    dispatch(s, [&]<typename S, bool EX>() {
        Work<S> &w = work<S>(s);
        UCFD_REQUIRE(w.u.p, "Run before Pack");
        run_gather_lambda<S>(s, rans, niter);
        if (mode == 0) {
            run_graph_build<S, EX>(s, rans, kappa);
            for (int it = 0; it < niter; ++it) {
                UCFD_CUDA(cudaGraphLaunch(s->run_exec, st));
                UCFD_CUDA(cudaMemcpyAsync(s->resid.p + it, s->red.p, sizeof(double), cudaMemcpyDeviceToDevice, st));
            }
        } else {
            run_persistent_begin(s);
            for (int it = 0; it < niter; ++it) lusgs_iteration<S, EX>(s, rans, kappa, s->resid.p + it, true);
        }
    });
    if (resid && niter > 0)
        UCFD_CUDA(cudaMemcpyAsync(resid, s->resid.p, niter * sizeof(double), cudaMemcpyDefault, st));
    if (mode == 1) run_persistent_check(s);
    s->run_state = true;
    finish(s, resid != nullptr);
    UCFD_API_END
}

// ---- block LU-SGS (blusgs.c) -------------------------------------------------
ucfd_status_t UCFDFlowSysSetBLUSGS(FlowSys *sys, UCFDReal *jmat, UCFDReal *tjmat) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(sys && *sys, "null FlowSys handle");
    UCFD_REQUIRE(jmat, "jmat must not be null");
    FlowSys s = *sys;
    UCFD_REQUIRE(s->mode == MODE_NONE || s->mode == MODE_BLUSGS, "FlowSys already set up for LU-SGS");
    s->mode = MODE_BLUSGS;
    s->jmat = jmat;
    s->tjmat = tjmat;
    UCFD_API_END
}

ucfd_status_t UCFDBLUSGS_Pack(FlowSys s, UCFDInt eidx, UCFDReal a0) {
    UCFD_API_BEGIN
    need_mode(s, MODE_BLUSGS);
    build_topology(s);
    Elem &e = elem(s, eidx);
    UCFD_REQUIRE(e.rhs && e.dt, "element %d: rhs and dt are needed by Pack", eidx);
    cudaStream_t st = s->stream();
    const size_t nv = (size_t)s->nvars * e.neles;
    const int *ids = ids_view(s, e);
    const double *rh = device_view<double>(e.rhs, nv, e.s_rhs, st);
    const double *dt = device_view<double>(e.dt, e.neles, e.s_dt, st);
    dispatch(s, [&]<typename S, bool EX>() {
        blusgs_alloc<S>(s);
        double *r64 = std::is_same<S, float>::value ? s->rhs64.p : nullptr;
        KCALL(EX, fs_blusgs_pack<S>, e.neles, s->nvars, s->nfvars, s->N, a0, ids, s->d_iperm.p, rh, dt,
              blu_rhs<S>(s), r64, s->dd.p, st);
    });
    s->c_valid[0] = s->c_valid[1] = false;
    finish(s, !is_device_ptr(e.rhs));
    UCFD_API_END
}

static ucfd_status_t tpack_api(FlowSys s, int model, UCFDInt eidx, UCFDReal factor, UCFDReal a0) {
    UCFD_API_BEGIN
    need_mode(s, MODE_BLUSGS);
    build_topology(s);
    UCFD_REQUIRE(s->ntvars > 0, "turbulence pack needs nvars > nfvars");
    UCFD_REQUIRE(model != 0 || s->ntvars == 2, "k-omega SST pack needs 2 turbulence variables");
    UCFD_REQUIRE(model != 1 || s->ntvars == 1, "Spalart-Allmaras pack needs 1 turbulence variable");
    Elem &e = elem(s, eidx);
    UCFD_REQUIRE(e.uptsb && e.dsrc && e.dt, "element %d: uptsb, dsrc and dt are needed", eidx);
    cudaStream_t st = s->stream();
    const size_t nv = (size_t)s->nvars * e.neles;
    const int *ids = ids_view(s, e);
    const double *up = device_view<double>(e.uptsb, nv, e.s_upts, st);
    const double *ds = device_view<double>(e.dsrc, nv, e.s_dsrc, st);
    const double *dt = device_view<double>(e.dt, e.neles, e.s_dt, st);
    dispatch(s, [&]<typename S, bool EX>() { blusgs_alloc<S>(s); });
    kfast::fs_tblusgs_pack(model, e.neles, s->nvars, s->ntvars, s->N, a0, factor, constants().betast, ids,
                           s->d_iperm.p, up, ds, dt, s->tD.p, st);
    s->c_valid[1] = false;
    finish(s, !is_device_ptr(e.uptsb));
    UCFD_API_END
}

ucfd_status_t UCFDBLUSGS_KWSST_Pack(FlowSys s, UCFDInt eidx, UCFDReal turb_factor, UCFDReal a0) {
    return tpack_api(s, 0, eidx, turb_factor, a0);
}
ucfd_status_t UCFDBLUSGS_SA_Pack(FlowSys s, UCFDInt eidx, UCFDReal turb_factor, UCFDReal a0) {
    return tpack_api(s, 1, eidx, turb_factor, a0);
}

static ucfd_status_t blusgs_prepare_api(FlowSys s, bool turb) {
    UCFD_API_BEGIN
    need_mode(s, MODE_BLUSGS);
    build_topology(s);
    const double *jm = turb ? s->tjmat : s->jmat;
    UCFD_REQUIRE(jm, "%s is not set", turb ? "tjmat" : "jmat");
    if (turb) UCFD_REQUIRE(s->ntvars > 0, "RANS prepare needs turbulence variables");
    cudaStream_t st = s->stream();
    const int B = turb ? s->ntvars : s->nfvars;
    static thread_local DevBuf<double> stage;
    // page-locked host Jacobians are read in place by the transpose kernel
    // under UCFD_HOST_MAP; otherwise staged
    const double *jd = (const double *)host_mapped(jm);
    if (!jd) jd = device_view<double>(jm, (size_t)2 * B * B * s->nfaces, stage, st);
    dispatch(s, [&]<typename S, bool EX>() {
        Work<S> &w = work<S>(s);
        UCFD_REQUIRE(w.rhs.p, "Prepare before Pack");
        double *D = turb ? s->tD.p : s->D.p;
        const double *dd = turb ? nullptr : s->dd.p;
        double *LU64 = turb ? s->tLU64.p : s->LU64.p;
        S *LU_s = nullptr;
        double *J64 = nullptr;
        if constexpr (std::is_same<S, float>::value) {
            // FP32 sweeps read the rounded factors only
            LU_s = turb ? w.tLU.p : w.LU.p;
            LU64 = nullptr;
            if (!turb) J64 = s->J64.ensure(tiled_size(s->N, (long long)s->P * B * B));
        }
        double *jt = s->jt.ensure((size_t)2 * B * B * s->nfaces);
        KCALL(EX, fs_blusgs_prepare<S>, B, s->N, s->P, (long long)s->nfaces, s->d_nei.p, s->d_slot.p, s->d_side.p,
              s->fa64.p, s->rv64.p, jd, dd, D, LU64, LU_s, turb ? w.tJ.p : w.J.p, J64, jt, st);
    });
    s->c_valid[turb ? 1 : 0] = false;
    ++s->jver[turb ? 1 : 0];  // new blocks: stored sweep sums are stale
    finish(s, !is_device_ptr(jm));
    UCFD_API_END
}

ucfd_status_t UCFDBLUSGS_NSPrepare(FlowSys s) { return blusgs_prepare_api(s, false); }
ucfd_status_t UCFDBLUSGS_RANSPrepare(FlowSys s) { return blusgs_prepare_api(s, true); }

static ucfd_status_t blusgs_sweep_api(FlowSys s, bool turb, bool upper) {
    UCFD_API_BEGIN
    need_mode(s, MODE_BLUSGS);
    build_topology(s);
    if (turb) UCFD_REQUIRE(s->ntvars > 0, "RANS sweep needs turbulence variables");
    dispatch(s, [&]<typename S, bool EX>() {
        Work<S> &w = work<S>(s);
        UCFD_REQUIRE(w.rhs.p, "sweep before Pack");
        UCFD_REQUIRE(blu_LU<S>(s, turb), "sweep before Prepare");
        blusgs_sweep_into<S, EX>(s, turb, upper, sweep_rhs<S, EX>(s, turb), w.bdu.p);
    });
    s->du64_valid = false;
    s->x_zero = false;
    finish(s);
    if (!s->async) check_sweep_err(s);
    UCFD_API_END
}

ucfd_status_t UCFDBLUSGS_NSLowerSweep(FlowSys s) { return blusgs_sweep_api(s, false, false); }
ucfd_status_t UCFDBLUSGS_NSUpperSweep(FlowSys s) { return blusgs_sweep_api(s, false, true); }
ucfd_status_t UCFDBLUSGS_RANSLowerSweep(FlowSys s) { return blusgs_sweep_api(s, true, false); }
ucfd_status_t UCFDBLUSGS_RANSUpperSweep(FlowSys s) { return blusgs_sweep_api(s, true, true); }

ucfd_status_t UCFDBLUSGS_Reset(FlowSys s) {
    UCFD_API_BEGIN
    need_mode(s, MODE_BLUSGS);
    build_topology(s);
    cudaStream_t st = s->stream();
    const size_t n = (size_t)s->nvars * s->N;
    dispatch(s, [&]<typename S, bool EX>() {
        blusgs_alloc<S>(s);
        Work<S> &w = work<S>(s);
        w.bdu.zero(n, st);
        w.dup.zero(n, st);
        if (std::is_same<S, float>::value) s->x64.zero(n, st);
        if constexpr (!EX) {
            split_zero<S>(s, false, w.bdu.p, st);
            if (s->ntvars > 0) split_zero<S>(s, true, w.bdu.p, st);
        }
    });
    s->du64_valid = false;
    s->x_zero = true;
    finish(s);
    UCFD_API_END
}

ucfd_status_t UCFDBLUSGS_SubResidual(FlowSys s, UCFDInt eidx) {
    UCFD_API_BEGIN
    need_mode(s, MODE_BLUSGS);
    build_topology(s);
    Elem &e = elem(s, eidx);
    UCFD_REQUIRE(e.vol && e.resid_out, "element %d: vol and resid_out are needed", eidx);
    cudaStream_t st = s->stream();
    const size_t nv = (size_t)s->nvars * e.neles;
    const int *ids = ids_view(s, e);
    const double *vol = device_view<double>(e.vol, e.neles, e.s_vol, st);
    const bool dev = is_device_ptr(e.resid_out);
    double *res = dev ? e.resid_out : e.s_res.ensure(nv);
    dispatch(s, [&]<typename S, bool EX>() {
        Work<S> &w = work<S>(s);
        UCFD_REQUIRE(w.bdu.p, "SubResidual before Pack");
        KCALL(EX, fs_blusgs_subres<S>, e.neles, s->nvars, s->N, ids, s->d_iperm.p, vol, w.bdu.p, w.dup.p, res, st);
    });
    if (!dev) copy_d2h(e.resid_out, res, nv * sizeof(double), st);
    finish(s, !dev);
    UCFD_API_END
}

ucfd_status_t UCFDBLUSGS_Update(FlowSys s, UCFDInt eidx) {
    UCFD_API_BEGIN
    need_mode(s, MODE_BLUSGS);
    build_topology(s);
    Elem &e = elem(s, eidx);
    UCFD_REQUIRE(e.uptsb, "element %d: uptsb is null", eidx);
    cudaStream_t st = s->stream();
    const size_t nv = (size_t)s->nvars * e.neles;
    const int *ids = ids_view(s, e);
    const bool dev = is_device_ptr(e.uptsb);
    double *up = dev ? e.uptsb : const_cast<double *>(device_view<double>(e.uptsb, nv, e.s_upts, st));
    if (s->prec == UCFD_PREC_FP32 && s->du64_valid) {
        kfast::fs_blusgs_update<double>(e.neles, s->nvars, s->N, ids, s->d_iperm.p, s->x64.p, up, st);
    } else {
        dispatch(s, [&]<typename S, bool EX>() {
            Work<S> &w = work<S>(s);
            UCFD_REQUIRE(w.bdu.p, "Update before Pack");
            KCALL(EX, fs_blusgs_update<S>, e.neles, s->nvars, s->N, ids, s->d_iperm.p, w.bdu.p, up, st);
        });
    }
    if (!dev) copy_d2h(e.uptsb, up, nv * sizeof(double), st);
    finish(s, !dev);
    UCFD_API_END
}

ucfd_status_t UCFDBLUSGS_Residual(FlowSys s, UCFDReal *relres) {
    UCFD_API_BEGIN
    need_mode(s, MODE_BLUSGS);
    build_topology(s);
    UCFD_REQUIRE(relres, "null relres");
    double rn = 0, bn = 0;
    if (s->prec == UCFD_PREC_FP32) {
        UCFD_REQUIRE(s->J64.p, "Residual before NSPrepare");
        if (s->du64_valid)
            blusgs_residual<double, double, false>(s, s->x_zero ? nullptr : s->x64.p, (double *)nullptr, &rn, &bn);
        else
            blusgs_residual<float, float, false>(s, s->x_zero ? nullptr : s->w32.bdu.p, (float *)nullptr, &rn, &bn);
    } else {
        UCFD_REQUIRE(s->w64.J.p, "Residual before NSPrepare");
        blusgs_residual<double, double, false>(s, s->x_zero ? nullptr : s->w64.bdu.p, (double *)nullptr, &rn, &bn);
    }
    *relres = bn > 0 ? rn / bn : rn;
    UCFD_API_END
}

ucfd_status_t UCFDBLUSGS_Solve(FlowSys s, UCFDReal rtol, UCFDInt max_sweeps, UCFDInt inner_sweeps, UCFDInt *nsweeps,
                               UCFDReal *relres) {
    UCFD_API_BEGIN
    need_mode(s, MODE_BLUSGS);
    build_topology(s);
    UCFD_REQUIRE(max_sweeps > 0 && inner_sweeps > 0, "max_sweeps and inner_sweeps must be positive");
    cudaStream_t st = s->stream();
    int pairs = 0;
    double rn = 0, bn = 0, rel = 0;
    if (s->prec == UCFD_PREC_FP32) {
        Work<float> &w = s->w32;
        UCFD_REQUIRE(s->J64.p && w.LU.p, "Solve before NSPrepare");
        const size_t n = (size_t)s->nvars * s->N;
        w.r.ensure(n);
        w.delta.ensure(n);
        if (!s->du64_valid) kfast::convert<float, double>((long long)n, w.bdu.p, s->x64.p, st);
        blusgs_residual<double, float, false>(s, s->x_zero ? nullptr : s->x64.p, w.r.p, &rn, &bn);
        rel = bn > 0 ? rn / bn : rn;
        while (rel > rtol && pairs < max_sweeps) {
            // the sweeps' right-hand side D^-1 r (their blocks are D^-1 J fv)
            kfast::fs_blusgs_rhs_solve<float>(s->nfvars, s->N, 0, w.LU.p, w.r.p, w.r.p, st);
            w.delta.zero(n, st);
            split_zero<float>(s, false, w.delta.p, st);
            const int m = std::min(inner_sweeps, max_sweeps - pairs);
            for (int q = 0; q < m; ++q) {
                blusgs_sweep_into<float, false>(s, false, false, w.r.p, w.delta.p);
                blusgs_sweep_into<float, false>(s, false, true, w.r.p, w.delta.p);
            }
            pairs += m;
            kfast::axpy_into<float>((long long)n, w.delta.p, s->x64.p, st);
            blusgs_residual<double, float, false>(s, s->x64.p, w.r.p, &rn, &bn);
            rel = bn > 0 ? rn / bn : rn;
            UCFD_CHECK_LAUNCH();
        }
        kfast::convert<double, float>((long long)n, s->x64.p, w.bdu.p, st);
        s->du64_valid = true;
        split_forget(s);  // du now holds the refined solution
    } else {
        Work<double> &w = s->w64;
        UCFD_REQUIRE(w.J.p, "Solve before NSPrepare");
        const bool ex = s->prec == UCFD_PREC_FP64;
        blusgs_residual<double, double, false>(s, s->x_zero ? nullptr : w.bdu.p, (double *)nullptr, &rn, &bn);
        rel = bn > 0 ? rn / bn : rn;
        while (rel > rtol && pairs < max_sweeps) {
            const int m = std::min(inner_sweeps, max_sweeps - pairs);
            for (int q = 0; q < m; ++q) {
                if (ex) {
                    blusgs_sweep_into<double, true>(s, false, false, w.rhs.p, w.bdu.p);
                    blusgs_sweep_into<double, true>(s, false, true, w.rhs.p, w.bdu.p);
                } else {
                    const double *c = sweep_rhs<double, false>(s, false);
                    blusgs_sweep_into<double, false>(s, false, false, c, w.bdu.p);
                    blusgs_sweep_into<double, false>(s, false, true, c, w.bdu.p);
                }
            }
            pairs += m;
            blusgs_residual<double, double, false>(s, w.bdu.p, (double *)nullptr, &rn, &bn);
            rel = bn > 0 ? rn / bn : rn;
            UCFD_CHECK_LAUNCH();
        }
    }
    if (pairs > 0) s->x_zero = false;
    if (nsweeps) *nsweeps = pairs;
    if (relres) *relres = rel;
    finish(s, true);
    UCFD_API_END
}

}  // extern "C"

// ---------------------------------------------------------------------------
// read-only view for allocation-free entry points (flowsys_view.h)
// ---------------------------------------------------------------------------
#include "flowsys_view.h"

bool ucfd::flowsys_block_view(FlowSys s, BlockSystemView &v) {
    if (!s || s->mode != MODE_BLUSGS || !s->topo || !s->D.p) return false;
    BlockSystemView t;
    t.N = s->N;
    t.P = s->P;
    t.B = s->nfvars;
    t.nei = s->d_nei.p;
    t.fa = s->prec == UCFD_PREC_FP64_FMA ? nullptr : s->fa64.p;  // FMA mode: J64 holds D^-1 J fa rv
    t.rv = s->rv64.p;
    t.D = s->D.p;
    if (s->prec == UCFD_PREC_FP32) {
        if (!s->J64.p || !s->rhs64.p) return false;
        t.J64 = s->J64.p;
        t.rhs64 = s->rhs64.p;
        if (s->du64_valid) t.x64 = s->x64.p;
        else t.x32 = s->w32.bdu.p;
    } else {
        if (!s->w64.J.p || !s->w64.rhs.p) return false;
        t.J64 = s->w64.J.p;
        t.rhs64 = s->w64.rhs.p;
        t.x64 = s->w64.bdu.p;
    }
    t.stream = (void *)s->stream();
    v = t;
    return true;
}
