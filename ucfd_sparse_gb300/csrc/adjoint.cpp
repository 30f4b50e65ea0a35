// adjoint.cpp -- one colored LU-SGS step on device arrays and its
// reverse-mode derivative (ucfdadjoint.h).
#include <vector>

#include "../../include/ucfdadjoint.h"
#include "launch.h"
#include "ucfd_internal.h"

using namespace ucfd;

namespace {

void require_dev(const void *p, const char *name) {
    UCFD_REQUIRE(p, "%s is null", name);
    UCFD_REQUIRE(is_device_ptr(p), "%s must be device memory", name);
}

template <typename T, bool EX>
void step(int neles, int nface, int nvars, int nfvars, int ndims, const int *nei, const int *icolor, int ncolors,
          const int *ranges, const int *lcolor, double factor, const T *fnv, const T *vec, const T *fspr, const T *dt,
          const T *upts, const T *rhs, T *diag, T *dub, T *dq, cudaStream_t s) {
    if constexpr (EX) kexact::legacy_pre<T>(neles, nface, (T)factor, fnv, dt, diag, fspr, s);
    else kfast::legacy_pre<T>(neles, nface, (T)factor, fnv, dt, diag, fspr, s);
    ScalarSweepArgs<T> a{};
    a.cells = icolor;
    a.lcolor = lcolor;
    a.nface = nface;
    a.ld = neles;
    a.nei = nei;
    a.fa = fnv;
    a.rv = nullptr;
    a.nrm = vec;
    a.lam = fspr;
    a.u = upts;
    a.diag = diag;
    a.diag_vs = 0;
    a.kappa = T(1);
    a.gamma = (T)constants().gamma;
    a.pmin = (T)constants().pmin;
    for (int pass = 0; pass < 2; ++pass) {
        const bool upper = pass == 1;
        a.upper = upper ? 1 : 0;
        a.nbsrc = upper ? dq : dub;
        a.own_in = upper ? dub : rhs;
        a.own_out = upper ? dq : dub;
        for (int q = 0; q < ncolors; ++q) {
            const int c = upper ? ncolors - 1 - q : q;
            a.t0 = c == 0 ? 0 : ranges[c - 1];
            a.t1 = ranges[c];
            if constexpr (EX) kexact::scalar_sweep<T>(a, nvars, nfvars, ndims, 0, 0, s);
            else kfast::scalar_sweep<T>(a, nvars, nfvars, ndims, 0, 0, s);
        }
    }
}

template <typename T>
void adjoint(int neles, int nface, int nvars, int nfvars, int ndims, const int *nei, const int *rface,
             const int *icolor, int ncolors, const int *ranges, const int *lcolor, double factor, const T *fnv,
             const T *vec, const T *fspr, const T *dt, const T *upts, const T *diag, const T *dub, const T *dq,
             const T *gdq, T *grhs, T *gdt, T *gfspr, T *work, cudaStream_t s) {
    const long long N = neles;
    T *qbar = work, *wbuf = work + (long long)nfvars * N, *dbar = work + 2ll * nfvars * N;
    UCFD_CUDA(cudaMemsetAsync(grhs, 0, sizeof(T) * nvars * N, s));
    AdjArgs a{0, 0, neles, nface, icolor, lcolor, nei, rface};
    const T g = (T)constants().gamma, pm = (T)constants().pmin;
    for (int c = 0; c < ncolors; ++c) {
        a.t0 = c == 0 ? 0 : ranges[c - 1];
        a.t1 = ranges[c];
        kfast::adj_upper<T>(a, nfvars, ndims, g, pm, fnv, vec, fspr, upts, diag, dub, dq, gdq, qbar, dbar, gfspr, s);
    }
    for (int c = ncolors - 1; c >= 0; --c) {
        a.t0 = c == 0 ? 0 : ranges[c - 1];
        a.t1 = ranges[c];
        kfast::adj_lower<T>(a, nfvars, ndims, g, pm, (T)factor, fnv, vec, fspr, dt, upts, diag, dub, qbar, wbuf, dbar,
                            grhs, gdt, gfspr, s);
    }
}

void check_common(int precision, int neles, int nface, int nvars, int nfvars, int ndims, int ncolors,
                  const int *ranges) {
    UCFD_REQUIRE(precision == UCFD_PREC_FP64 || precision == UCFD_PREC_FP64_FMA || precision == UCFD_PREC_FP32,
                 "unknown precision %d", precision);
    UCFD_REQUIRE(neles > 0 && nface > 0 && ncolors > 0 && ranges, "bad sizes");
    UCFD_REQUIRE(nfvars == ndims + 2 && nvars >= nfvars, "nfvars must be ndims + 2 and nvars >= nfvars");
    int prev = 0;
    for (int c = 0; c < ncolors; ++c) {
        UCFD_REQUIRE(ranges[c] >= prev, "colour ranges must be non-decreasing");
        prev = ranges[c];
    }
    UCFD_REQUIRE(prev == neles, "the last colour range must end at neles");
}

}  // namespace

extern "C" {

ucfd_status_t UCFDReverseFaces(int neles, int nface, const int *nei_ele, int *rface) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(neles > 0 && nface > 0 && nei_ele && rface, "UCFDReverseFaces: bad arguments");
    const long long N = neles;
    for (int i = 0; i < neles; ++i)
        for (int f = 0; f < nface; ++f) {
            const int j = nei_ele[f * N + i];
            UCFD_REQUIRE(j >= 0 && j < neles, "nei_ele[%d][%d] = %d out of range", f, i, j);
            int r = f;
            if (j != i) {
                r = -1;
                for (int g = 0; g < nface; ++g)
                    if (nei_ele[g * N + j] == i) {
                        r = g;
                        break;
                    }
                UCFD_REQUIRE(r >= 0, "cell %d lists %d as a neighbour but not the reverse", i, j);
            }
            rface[f * N + i] = r;
        }
    UCFD_API_END
}

ucfd_status_t UCFDColoredStep(int precision, int neles, int nface, int nvars, int nfvars, int ndims,
                              const int *nei_ele, const int *icolor, int ncolors, const int *ranges,
                              const int *lcolor, double factor, const void *fnorm_vol, const void *vec_fnorm,
                              const void *fspr, const void *dt, const void *upts, const void *rhs, void *diag,
                              void *dub, void *dq, void *stream) {
    UCFD_API_BEGIN
    check_common(precision, neles, nface, nvars, nfvars, ndims, ncolors, ranges);
    for (auto [p, n] : {std::pair<const void *, const char *>{nei_ele, "nei_ele"}, {icolor, "icolor"},
                        {lcolor, "lcolor"}, {fnorm_vol, "fnorm_vol"}, {vec_fnorm, "vec_fnorm"}, {fspr, "fspr"},
                        {dt, "dt"}, {upts, "upts"}, {rhs, "rhs"}, {diag, "diag"}, {dub, "dub"}, {dq, "dq"}})
        require_dev(p, n);
    cudaStream_t s = (cudaStream_t)stream;
    if (precision == UCFD_PREC_FP32)
        step<float, false>(neles, nface, nvars, nfvars, ndims, nei_ele, icolor, ncolors, ranges, lcolor, factor,
                           (const float *)fnorm_vol, (const float *)vec_fnorm, (const float *)fspr, (const float *)dt,
                           (const float *)upts, (const float *)rhs, (float *)diag, (float *)dub, (float *)dq, s);
    else if (precision == UCFD_PREC_FP64)
        step<double, true>(neles, nface, nvars, nfvars, ndims, nei_ele, icolor, ncolors, ranges, lcolor, factor,
                           (const double *)fnorm_vol, (const double *)vec_fnorm, (const double *)fspr,
                           (const double *)dt, (const double *)upts, (const double *)rhs, (double *)diag,
                           (double *)dub, (double *)dq, s);
    else
        step<double, false>(neles, nface, nvars, nfvars, ndims, nei_ele, icolor, ncolors, ranges, lcolor, factor,
                            (const double *)fnorm_vol, (const double *)vec_fnorm, (const double *)fspr,
                            (const double *)dt, (const double *)upts, (const double *)rhs, (double *)diag,
                            (double *)dub, (double *)dq, s);
    UCFD_CHECK_LAUNCH();
    if (!stream) UCFD_CUDA(cudaStreamSynchronize(s));
    UCFD_API_END
}

ucfd_status_t UCFDColoredStepAdjoint(int precision, int neles, int nface, int nvars, int nfvars, int ndims,
                                     const int *nei_ele, const int *rface, const int *icolor, int ncolors,
                                     const int *ranges, const int *lcolor, double factor, const void *fnorm_vol,
                                     const void *vec_fnorm, const void *fspr, const void *dt, const void *upts,
                                     const void *diag, const void *dub, const void *dq, const void *gdq, void *grhs,
                                     void *gdt, void *gfspr, void *work, void *stream) {
    UCFD_API_BEGIN
    check_common(precision, neles, nface, nvars, nfvars, ndims, ncolors, ranges);
    for (auto [p, n] : {std::pair<const void *, const char *>{nei_ele, "nei_ele"}, {rface, "rface"},
                        {icolor, "icolor"}, {lcolor, "lcolor"}, {fnorm_vol, "fnorm_vol"}, {vec_fnorm, "vec_fnorm"},
                        {fspr, "fspr"}, {dt, "dt"}, {upts, "upts"}, {diag, "diag"}, {dub, "dub"}, {dq, "dq"},
                        {gdq, "gdq"}, {grhs, "grhs"}, {gdt, "gdt"}, {gfspr, "gfspr"}, {work, "work"}})
        require_dev(p, n);
    cudaStream_t s = (cudaStream_t)stream;
    if (precision == UCFD_PREC_FP32)
        adjoint<float>(neles, nface, nvars, nfvars, ndims, nei_ele, rface, icolor, ncolors, ranges, lcolor, factor,
                       (const float *)fnorm_vol, (const float *)vec_fnorm, (const float *)fspr, (const float *)dt,
                       (const float *)upts, (const float *)diag, (const float *)dub, (const float *)dq,
                       (const float *)gdq, (float *)grhs, (float *)gdt, (float *)gfspr, (float *)work, s);
    else
        adjoint<double>(neles, nface, nvars, nfvars, ndims, nei_ele, rface, icolor, ncolors, ranges, lcolor, factor,
                        (const double *)fnorm_vol, (const double *)vec_fnorm, (const double *)fspr,
                        (const double *)dt, (const double *)upts, (const double *)diag, (const double *)dub,
                        (const double *)dq, (const double *)gdq, (double *)grhs, (double *)gdt, (double *)gfspr,
                        (double *)work, s);
    UCFD_CHECK_LAUNCH();
    if (!stream) UCFD_CUDA(cudaStreamSynchronize(s));
    UCFD_API_END
}

}  // extern "C"
