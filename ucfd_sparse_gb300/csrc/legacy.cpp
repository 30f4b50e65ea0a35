// legacy.cpp -- the array-based (colored) LU-SGS entry points of
// coloredlusgs.h.  Stateless calls on the caller's layout: one thread per
// cell of the colour range (parallel_*) or of each level of the
// natural-order schedule (serial_*).  Host arrays are staged to the GPU for
// the call and the written array is copied back before returning.
#include <mutex>
#include <unordered_map>

#include "../../include/coloredlusgs.h"
#include "graph.h"
#include "launch.h"
#include "ucfd_internal.h"

using namespace ucfd;

namespace {

struct LegacyCtx {
    std::mutex mu;
    int nvars = 5, nfvars = 5, ndims = 3;
    int prec = UCFD_PREC_FP64;
    cudaStream_t stream = nullptr;
    ucfd_status_t last = UCFD_SUCCESS;
    DevBuf<int> s_nei, s_icolor, s_lcolor;
    DevBuf<double> s_fnv, s_vec, s_upts, s_rhs, s_dub, s_diag, s_fspr, s_dt;
    // natural-order schedule cache of the serial sweeps
    const void *sched_key = nullptr;
    int sched_n = -1, sched_nf = -1;
    uint64_t sched_hash = 0;
    int nlev = 0;
    std::vector<int> lev_off;
    DevBuf<int> d_perm, d_level;
};

LegacyCtx &ctx() {
    static LegacyCtx c;
    return c;
}

cudaStream_t stream_of(LegacyCtx &c) {
    if (!c.stream) {
        ensure_device();
        UCFD_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    }
    return c.stream;
}

template <typename T>
struct Arr {
    T *user;      // caller pointer
    T *dev;       // device pointer used by kernels
    size_t count;
    bool host;
};

template <typename T>
Arr<T> stage(T *p, size_t count, DevBuf<T> &buf, cudaStream_t s) {
    UCFD_REQUIRE(p || count == 0, "null array argument");
    Arr<T> a{p, p, count, false};
    if (!is_device_ptr(p)) {
        a.host = true;
        buf.upload(p, count, s);
        a.dev = buf.p;
    }
    return a;
}

template <typename T>
void writeback(const Arr<T> &a, cudaStream_t s) {
    if (a.host && a.count)
        copy_d2h(a.user, a.dev, a.count * sizeof(T), s);
}

void done(cudaStream_t s) {
    UCFD_CHECK_LAUNCH();
    UCFD_CUDA(cudaStreamSynchronize(s));
}

uint64_t fnv_hash(const int *p, size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; ++i) {
        h ^= (uint32_t)p[i];
        h *= 1099511628211ull;
    }
    return h;
}

// Levels of the natural-order sweep over the nei_ele table (cached by
// pointer, sizes and a hash of the contents).
void serial_schedule(LegacyCtx &c, int neles, int nface, const int *nei, cudaStream_t s) {
    std::vector<int> h;
    to_host(nei, (size_t)neles * nface, h);
    const uint64_t hs = fnv_hash(h.data(), h.size());
    if (c.sched_key == nei && c.sched_n == neles && c.sched_nf == nface && c.sched_hash == hs) return;
    std::vector<int> rp(neles + 1), ci((size_t)neles * nface);
    for (int i = 0; i <= neles; ++i) rp[i] = i * nface;
    for (int i = 0; i < neles; ++i)
        for (int f = 0; f < nface; ++f) {
            const int nb = h[(size_t)f * neles + i];
            UCFD_REQUIRE(nb >= 0 && nb < neles, "nei_ele[%d][%d] = %d out of range", f, i, nb);
            ci[(size_t)i * nface + f] = nb;
        }
    Schedule sch = schedule_natural(neles, rp.data(), ci.data());
    std::vector<int> level(neles);
    for (int l = 0; l < sch.nlev; ++l)
        for (int k = sch.lev_off[l]; k < sch.lev_off[l + 1]; ++k) level[sch.perm[k]] = l;
    c.d_perm.upload(sch.perm.data(), neles, s);
    c.d_level.upload(level.data(), neles, s);
    c.lev_off = sch.lev_off;
    c.nlev = sch.nlev;
    c.sched_key = nei;
    c.sched_n = neles;
    c.sched_nf = nface;
    c.sched_hash = hs;
}

// One sweep launch over cells[t0, t1) with the colour test on lcolor.
void launch_sweep(LegacyCtx &c, bool upper, bool rans, int t0, int t1, int neles, int nface, const int *nei,
                  const int *cells, const int *lcolor, const double *fnv, const double *vec, const double *upts,
                  const double *nbsrc, const double *own_in, double *own_out, const double *diag,
                  const double *fspr, cudaStream_t s) {
    ScalarSweepArgs<double> a{};
    a.t0 = t0;
    a.t1 = t1;
    a.cells = cells;
    a.lcolor = lcolor;
    a.lo = a.hi = 0;
    a.nface = nface;
    a.ld = neles;
    a.nei = nei;
    a.fa = fnv;
    a.rv = nullptr;
    a.nrm = vec;
    a.lam = fspr;
    a.u = upts;
    a.nbsrc = nbsrc;
    a.own_in = own_in;
    a.own_out = own_out;
    a.diag = diag;
    a.diag_vs = 0;
    a.kappa = 1.0;
    a.gamma = constants().gamma;
    a.pmin = constants().pmin;
    a.upper = upper ? 1 : 0;
    if (c.prec == UCFD_PREC_FP64)
        kexact::scalar_sweep<double>(a, c.nvars, c.nfvars, c.ndims, rans ? 1 : 0, 0, s);
    else
        kfast::scalar_sweep<double>(a, c.nvars, c.nfvars, c.ndims, rans ? 1 : 0, 0, s);
}

// Shared body of every sweep entry point.  serial: natural order over all
// cells; otherwise icolor[n0:ne) with lcolor.  inplace: the C-example form
// (dub read and written by both sweeps).
void sweep(bool serial, bool upper, bool rans, bool inplace, int n0, int ne, int neles, int nface, int *nei,
           int *icolor, int *lcolor, double *fnv, double *vec, double *upts, double *rhs, double *dub,
           double *diag, double *fspr) {
    LegacyCtx &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    UCFD_REQUIRE(neles > 0 && nface > 0, "neles and nface must be positive");
    if (rans) UCFD_REQUIRE(c.nvars > c.nfvars, "RANS sweeps need nvars > nfvars (UCFDLegacySetDims)");
    if (!serial) {
        UCFD_REQUIRE(0 <= n0 && n0 <= ne && ne <= neles, "colour range [%d, %d) outside [0, %d]", n0, ne, neles);
        UCFD_REQUIRE(icolor && lcolor, "icolor and lcolor are required");
    }
    cudaStream_t s = stream_of(c);
    const size_t N = neles, nv = (size_t)c.nvars * N;
    auto a_nei = stage<int>(nei, nface * N, c.s_nei, s);
    auto a_fnv = stage<double>(fnv, nface * N, c.s_fnv, s);
    auto a_vec = stage<double>(vec, (size_t)nface * c.ndims * N, c.s_vec, s);
    auto a_upts = stage<double>(upts, nv, c.s_upts, s);
    auto a_dub = stage<double>(dub, nv, c.s_dub, s);
    auto a_diag = stage<double>(diag, N, c.s_diag, s);
    auto a_fspr = stage<double>(fspr, nface * N, c.s_fspr, s);
    Arr<double> a_rhs = a_dub;
    if (!inplace) a_rhs = stage<double>(rhs, nv, c.s_rhs, s);
    // lower: neighbours and result in dub, own input rhs; upper: neighbours
    // and result in rhs, own input dub (README.md:41-50)
    double *nbsrc = upper ? a_rhs.dev : a_dub.dev;
    double *own_in = upper ? a_dub.dev : a_rhs.dev;
    double *own_out = upper ? a_rhs.dev : a_dub.dev;
    if (inplace) nbsrc = own_in = own_out = a_dub.dev;
    if (serial) {
        serial_schedule(c, neles, nface, nei, s);
        for (int q = 0; q < c.nlev; ++q) {
            const int l = upper ? c.nlev - 1 - q : q;
            launch_sweep(c, upper, rans, c.lev_off[l], c.lev_off[l + 1], neles, nface, a_nei.dev, c.d_perm.p,
                         c.d_level.p, a_fnv.dev, a_vec.dev, a_upts.dev, nbsrc, own_in, own_out, a_diag.dev,
                         a_fspr.dev, s);
        }
    } else {
        auto a_ic = stage<int>(icolor, N, c.s_icolor, s);
        auto a_lc = stage<int>(lcolor, N, c.s_lcolor, s);
        launch_sweep(c, upper, rans, n0, ne, neles, nface, a_nei.dev, a_ic.dev, a_lc.dev, a_fnv.dev, a_vec.dev,
                     a_upts.dev, nbsrc, own_in, own_out, a_diag.dev, a_fspr.dev, s);
    }
    writeback(upper && !inplace ? a_rhs : a_dub, s);
    done(s);
}

void pre(int neles, int nface, double factor, double *fnv, double *dt, double *diag, double *fspr) {
    LegacyCtx &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    UCFD_REQUIRE(neles > 0 && nface > 0, "neles and nface must be positive");
    cudaStream_t s = stream_of(c);
    const size_t N = neles;
    auto a_fnv = stage<double>(fnv, nface * N, c.s_fnv, s);
    auto a_dt = stage<double>(dt, N, c.s_dt, s);
    auto a_fspr = stage<double>(fspr, nface * N, c.s_fspr, s);
    auto a_diag = stage<double>(diag, N, c.s_diag, s);
    if (c.prec == UCFD_PREC_FP64)
        kexact::legacy_pre<double>(neles, nface, factor, a_fnv.dev, a_dt.dev, a_diag.dev, a_fspr.dev, s);
    else
        kfast::legacy_pre<double>(neles, nface, factor, a_fnv.dev, a_dt.dev, a_diag.dev, a_fspr.dev, s);
    writeback(a_diag, s);
    done(s);
}

void update(bool rans, int neles, double *upts, double *rhs) {
    LegacyCtx &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    UCFD_REQUIRE(neles > 0, "neles must be positive");
    cudaStream_t s = stream_of(c);
    const size_t nv = (size_t)c.nvars * neles;
    auto a_up = stage<double>(upts, nv, c.s_upts, s);
    auto a_rhs = stage<double>(rhs, nv, c.s_rhs, s);
    const int k0 = rans ? c.nfvars : 0, k1 = rans ? c.nvars : c.nfvars;
    kexact::legacy_update<double>(neles, k0, k1, a_up.dev, a_rhs.dev, s);
    writeback(a_up, s);
    done(s);
}

template <typename F>
void guarded(F &&f) {
    ucfd_status_t st = UCFD_SUCCESS;
    try {
        clear_error();
        f();
    } catch (const Error &e) {
        st = e.st;
    } catch (const std::bad_alloc &) {
        set_error("host allocation failed");
        st = UCFD_ERR_NOMEM;
    } catch (...) {
        set_error("unexpected exception");
        st = UCFD_FAILED;
    }
    ctx().last = st;
    if (st != UCFD_SUCCESS) fprintf(stderr, "[ucfd_gb300] %s\n", UCFDGetLastError());
}

}  // namespace

extern "C" {

ucfd_status_t UCFDLegacySetDims(int nvars, int nfvars, int ndims) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(ndims == 2 || ndims == 3, "ndims must be 2 or 3");
    UCFD_REQUIRE(nfvars == ndims + 2, "nfvars must be ndims + 2");
    UCFD_REQUIRE(nvars >= nfvars && nvars <= nfvars + 2, "nvars must be nfvars .. nfvars + 2");
    LegacyCtx &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    c.nvars = nvars;
    c.nfvars = nfvars;
    c.ndims = ndims;
    UCFD_API_END
}

ucfd_status_t UCFDLegacySetPrecision(int precision) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(precision == UCFD_PREC_FP64 || precision == UCFD_PREC_FP64_FMA,
                 "the array API works on double arrays: UCFD_PREC_FP64 or UCFD_PREC_FP64_FMA");
    LegacyCtx &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    c.prec = precision;
    UCFD_API_END
}

ucfd_status_t UCFDLegacyLastStatus(void) { return ctx().last; }

void serial_pre_lusgs(int neles, int nface, double factor, double *fnorm_vol, double *dt, double *diag,
                      double *fspr) {
    guarded([&] { pre(neles, nface, factor, fnorm_vol, dt, diag, fspr); });
}
void parallel_pre_lusgs(int neles, int nface, double factor, double *fnorm_vol, double *dt, double *diag,
                        double *fspr) {
    guarded([&] { pre(neles, nface, factor, fnorm_vol, dt, diag, fspr); });
}

#define SERIAL_ARGS int neles, int nface, int *nei_ele, double *fnorm_vol, double *vec_fnorm, double *upts, \
                    double *rhs, double *dub, double *diag, double *fspr
#define PAR_ARGS int n0, int ne, int neles, int nface, int *nei_ele, int *icolor, int *lcolor, double *fnorm_vol, \
                 double *vec_fnorm, double *upts, double *rhs, double *dub, double *diag, double *fspr

void ns_serial_lower_sweep(SERIAL_ARGS) {
    guarded([&] { sweep(true, false, false, false, 0, neles, neles, nface, nei_ele, nullptr, nullptr, fnorm_vol,
                        vec_fnorm, upts, rhs, dub, diag, fspr); });
}
void ns_serial_upper_sweep(SERIAL_ARGS) {
    guarded([&] { sweep(true, true, false, false, 0, neles, neles, nface, nei_ele, nullptr, nullptr, fnorm_vol,
                        vec_fnorm, upts, rhs, dub, diag, fspr); });
}
void rans_serial_lower_sweep(SERIAL_ARGS) {
    guarded([&] { sweep(true, false, true, false, 0, neles, neles, nface, nei_ele, nullptr, nullptr, fnorm_vol,
                        vec_fnorm, upts, rhs, dub, diag, fspr); });
}
void rans_serial_upper_sweep(SERIAL_ARGS) {
    guarded([&] { sweep(true, true, true, false, 0, neles, neles, nface, nei_ele, nullptr, nullptr, fnorm_vol,
                        vec_fnorm, upts, rhs, dub, diag, fspr); });
}
void ns_parallel_lower_sweep(PAR_ARGS) {
    guarded([&] { sweep(false, false, false, false, n0, ne, neles, nface, nei_ele, icolor, lcolor, fnorm_vol,
                        vec_fnorm, upts, rhs, dub, diag, fspr); });
}
void ns_parallel_upper_sweep(PAR_ARGS) {
    guarded([&] { sweep(false, true, false, false, n0, ne, neles, nface, nei_ele, icolor, lcolor, fnorm_vol,
                        vec_fnorm, upts, rhs, dub, diag, fspr); });
}
void rans_parallel_lower_sweep(PAR_ARGS) {
    guarded([&] { sweep(false, false, true, false, n0, ne, neles, nface, nei_ele, icolor, lcolor, fnorm_vol,
                        vec_fnorm, upts, rhs, dub, diag, fspr); });
}
void rans_parallel_upper_sweep(PAR_ARGS) {
    guarded([&] { sweep(false, true, true, false, n0, ne, neles, nface, nei_ele, icolor, lcolor, fnorm_vol,
                        vec_fnorm, upts, rhs, dub, diag, fspr); });
}

void lusgs_serial_ns_update(int neles, double *upts, double *rhs) { guarded([&] { update(false, neles, upts, rhs); }); }
void lusgs_parallel_ns_update(int neles, double *upts, double *rhs) { guarded([&] { update(false, neles, upts, rhs); }); }
void lusgs_serial_rans_update(int neles, double *upts, double *rhs) { guarded([&] { update(true, neles, upts, rhs); }); }
void lusgs_parallel_rans_update(int neles, double *upts, double *rhs) { guarded([&] { update(true, neles, upts, rhs); }); }

// C-example spellings: dub in place, no rhs.
void serial_ns_lower_sweep(int neles, int nface, int *nei_ele, double *fnorm_vol, double *vec_fnorm, double *upts,
                           double *dub, double *diag, double *fspr) {
    guarded([&] { sweep(true, false, false, true, 0, neles, neles, nface, nei_ele, nullptr, nullptr, fnorm_vol,
                        vec_fnorm, upts, nullptr, dub, diag, fspr); });
}
void serial_ns_upper_sweep(int neles, int nface, int *nei_ele, double *fnorm_vol, double *vec_fnorm, double *upts,
                           double *dub, double *diag, double *fspr) {
    guarded([&] { sweep(true, true, false, true, 0, neles, neles, nface, nei_ele, nullptr, nullptr, fnorm_vol,
                        vec_fnorm, upts, nullptr, dub, diag, fspr); });
}
void serial_ns_lusgs_update(int neles, double *upts, double *dub) { guarded([&] { update(false, neles, upts, dub); }); }
void parallel_ns_lower_sweep(int n0, int ne, int neles, int nface, int *nei_ele, int *icolor, int *lcolor,
                             double *fnorm_vol, double *vec_fnorm, double *upts, double *dub, double *diag,
                             double *fspr) {
    guarded([&] { sweep(false, false, false, true, n0, ne, neles, nface, nei_ele, icolor, lcolor, fnorm_vol,
                        vec_fnorm, upts, nullptr, dub, diag, fspr); });
}
void parallel_ns_upper_sweep(int n0, int ne, int neles, int nface, int *nei_ele, int *icolor, int *lcolor,
                             double *fnorm_vol, double *vec_fnorm, double *upts, double *dub, double *diag,
                             double *fspr) {
    guarded([&] { sweep(false, true, false, true, n0, ne, neles, nface, nei_ele, icolor, lcolor, fnorm_vol,
                        vec_fnorm, upts, nullptr, dub, diag, fspr); });
}

}  // extern "C"
