// launch.h -- host-callable launchers of the device kernels.
//
// The same declarations exist in two namespaces, one per build of the
// kernel source:
//   kexact  built with -fmad=false (no FMA contraction), FP64 instantiations:
//           bit-for-bit the reference arithmetic (UCFD_PREC_FP64);
//   kfast   built with FMA contraction, FP64 and FP32 instantiations
//           (UCFD_PREC_FP64_FMA, UCFD_PREC_FP32) and the GMRES reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kargs.h"

#define UCFD_DECLARE_LAUNCHERS                                                                     \
    /* ---- scalar LU-SGS ---- */                                                                  \
    template <typename T>                                                                          \
    void scalar_sweep(const ::ucfd::ScalarSweepArgs<T> &a, int nv, int nfv, int ndims, int rans,   \
                      int block, cudaStream_t s);                                                  \
    template <typename T>                                                                          \
    void scalar_sweep_persistent(const ::ucfd::ScalarSweepArgs<T> &a, int nv, int nfv, int ndims,  \
                                 int rans, const int *lev_off, int nlev, unsigned *bar, int *err,  \
                                 long long max_spin, cudaStream_t s);                              \
    template <typename T>                                                                          \
    void face_list_geo(long long E, long long ld, int ndims, const int *q, const T *nrm,           \
                       const T *fa, const T *rv, T *geo, cudaStream_t s);                          \
    void pack_geo4(long long N, int P, int ndims, const float *nrm, const float *fa,               \
                   const float *rv, void *geo4, cudaStream_t s);                                   \
    void pack_lam2(long long n, const float *lam, const float *tlam, void *lam2, cudaStream_t s);  \
    template <typename T>                                                                          \
    void legacy_pre(int neles, int nface, T factor, const T *fnorm_vol, const T *dt, T *diag,      \
                    const T *fspr, cudaStream_t s);                                                \
    template <typename T>                                                                          \
    void legacy_update(int neles, int k0, int k1, T *upts, const T *rhs, cudaStream_t s);          \
    template <typename T>                                                                          \
    void fs_lusgs_pack(int neles, int nvars, int nfvars, long long N, double turb_factor,          \
                       double a0, const int *cell_ids, const int *iperm, const double *upts,       \
                       const double *rhs, const double *dt, const double *dsrc, T *u, T *du,       \
                       T *diag, cudaStream_t s);                                                   \
    template <typename T>                                                                          \
    void fs_lusgs_update(int neles, int nvars, long long N, const int *cell_ids, const int *iperm, \
                         const T *du, double *upts, int assign, cudaStream_t s);                   \
    template <typename T>                                                                          \
    void fs_lusgs_prepare(long long N, int maxdeg, int nv0, int nv1, T kappa, const int *nei,      \
                          const T *fa, const T *rv, const T *lam, const T *base, T *diag,          \
                          cudaStream_t s);                                                         \
    template <typename T>                                                                          \
    void fs_lusgs_prepare_both(long long N, int maxdeg, int nfv, int nv, T kappa, const int *nei,  \
                               const T *fa, const T *rv, const T *lam, const T *tlam,              \
                               const T *base, T *diag, cudaStream_t s);                            \
    template <typename Td>                                                                         \
    void gather_idx(long long n, const int *idx, const double *src, Td *dst, cudaStream_t s);      \
    void pair_reduce(int nblocks, const double *part, double *out, cudaStream_t s);                \
    /* ---- block LU-SGS ---- */                                                                   \
    template <typename S>                                                                          \
    void fs_blusgs_pack(int neles, int nvars, int B, long long N, double a0, const int *cell_ids,   \
                        const int *iperm, const double *rhs, const double *dt, S *rhs_s,           \
                        double *rhs64, double *D, cudaStream_t s);                                 \
    void fs_tblusgs_pack(int model, int neles, int nvars, int nt, long long N, double a0,          \
                         double factor, double betast, const int *cell_ids, const int *iperm,      \
                         const double *uptsb, const double *dsrc, const double *dt, double *D,     \
                         cudaStream_t s);                                                          \
    template <typename S>                                                                          \
    void fs_blusgs_prepare(int B, long long N, int P, long long nF, const int *nei,               \
                           const int *slot, const int8_t *side, const double *fa,                  \
                           const double *rv, const double *jmat, const double *dd, double *D,      \
                           double *LU64, S *LU_s, S *J_s, double *J64, double *jt,                 \
                           cudaStream_t s);                                                        \
    template <typename S>                                                                          \
    void fs_blusgs_sweep(int B, int t0, int t1, long long N, int P, int var0, const int *nei,      \
                         const S *fa, const S *rv, const S *J, const S *LU, const S *rhs, S *du,   \
                         int block, int variant, int *err, long long max_spin,                     \
                         const ::ucfd::SweepSplit<S> &sp, cudaStream_t s);                         \
    template <typename S>                                                                          \
    void fs_blusgs_rhs_solve(int B, long long N, int var0, const S *LU, const S *b, S *c,          \
                             cudaStream_t s);                                                      \
    template <typename Sx, typename R>                                                             \
    void fs_blusgs_residual(int B, long long N, int P, int var0, int nvars, const int *nei,        \
                            const double *fa, const double *rv, const double *J64,                 \
                            const double *D, const double *rhs64, const Sx *x, R *r_out,           \
                            double *part, int nblocks_max, int *nblocks_used, cudaStream_t s);     \
    template <typename S>                                                                          \
    void fs_blusgs_subres(int neles, int nvars, long long N, const int *cell_ids,                  \
                          const int *iperm, const double *vol, const S *du, S *dup, double *res,   \
                          cudaStream_t s);                                                         \
    template <typename S>                                                                          \
    void fs_blusgs_update(int neles, int nvars, long long N, const int *cell_ids,                  \
                          const int *iperm, const S *du, double *upts, cudaStream_t s);            \
    /* ---- Krylov ---- */                                                                         \
    template <typename Tv, typename Ta>                                                            \
    void bsr_spmv(int B, int bn, int P, const int *col, const Tv *val, double alpha,               \
                  const double *x, double beta, double *y, int block, cudaStream_t s);             \
    template <typename Tl>                                                                         \
    void pc_prepare(int B, int bn, const int *perm, const long long *dslot, const double *values,  \
                    double *LU64, Tl *LU_l, int factor, cudaStream_t s);                           \
    template <typename T>                                                                          \
    void pc_lower(int B, int t0, int t1, int bn, int PL, const int *Lcol, const T *Lval,           \
                  const T *LU, T *b, int block, int mode, cudaStream_t s);                         \
    template <typename T>                                                                          \
    void pc_upper(int B, int t0, int t1, int bn, int PU, const int *Ucol, const T *Uval,           \
                  const T *LU, T *b, int block, int mode, cudaStream_t s);                         \
    void ilu_factor(int B, int scalar, int t0, int t1, const int *rows, const int *rowptr,         \
                    const int *colidx, const int *diagslots, double *vals, cudaStream_t s);        \
    template <typename T>                                                                          \
    void ell_gather(int B, int bn, int P, const int *src, const double *vals, T *out,              \
                    cudaStream_t s);                                                               \
    void fingerprint(long long n, const int *a, unsigned long long *out, cudaStream_t s);          \
    template <typename Ts, typename Td>                                                            \
    void gather_rows(int bn, int B, const int *perm, const Ts *src, Td *dst, cudaStream_t s);      \
    template <typename Ts, typename Td>                                                            \
    void scatter_rows(int bn, int B, const int *perm, const Ts *src, Td *dst, cudaStream_t s);     \
    template <typename Ts, typename Td>                                                            \
    void convert(long long n, const Ts *src, Td *dst, cudaStream_t s);                             \
    template <typename Ts>                                                                         \
    void axpy_into(long long n, const Ts *x, double *y, cudaStream_t s);                           \
    template <typename S>                                                                          \
    void axpy_norm(long long n, const S *x, S *y, double *part, double *out, cudaStream_t s);      \
    void axpy_master(long long n, const float *x, float *hi, float *lo, double *part, double *out,   \
                     cudaStream_t s);                                                              \
    void state_lo_pack(int neles, int nvars, long long N, const int *cell_ids, const int *iperm,   \
                       const double *upts, float *lo, cudaStream_t s);                             \
    void state_ff_update(int neles, int nvars, long long N, const int *cell_ids, const int *iperm, \
                         const float *hi, const float *lo, double *upts, cudaStream_t s);          \
    /* ---- adjoint of the colored LU-SGS step ---- */                                            \
    template <typename T>                                                                          \
    void adj_upper(const ::ucfd::AdjArgs &a, int nfv, int ndims, T gamma, T pmin, const T *fnv,    \
                   const T *vec, const T *fspr, const T *upts, const T *diag, const T *dub,        \
                   const T *dq, const T *gdq, T *qbar, T *dbar, T *gfspr, cudaStream_t s);         \
    template <typename T>                                                                          \
    void adj_lower(const ::ucfd::AdjArgs &a, int nfv, int ndims, T gamma, T pmin, T factor,        \
                   const T *fnv, const T *vec, const T *fspr, const T *dt, const T *upts,          \
                   const T *diag, const T *dub, const T *qbar, T *wbuf, const T *dbar, T *grhs,    \
                   T *gdt, T *gfspr, cudaStream_t s);                                              \
    /* ---- GMRES pieces ---- */                                                                   \
    int gm_blocks(long long n);                                                                    \
    void gm_dots(long long n, int K, const double *V, long long ldv, const double *w,              \
                 double *part, cudaStream_t s);                                                    \
    void gm_update(long long n, int K, const double *V, long long ldv, const double *h, double *w, \
                   int mode, double *part, cudaStream_t s);                                        \
    void gm_reduce(int nblocks, int K, const double *part, double *out, int accumulate,            \
                   cudaStream_t s);                                                                \
    void gm_sumsq(long long n, const double *x, double *part, cudaStream_t s);                     \
    void gm_cycle_begin(int nblocks, const double *part, void *st, double *y, double *out_norm,    \
                        cudaStream_t s);                                                           \
    void gm_scale(long long n, const void *st, const double *src, double *dst, cudaStream_t s);    \
    void gm_givens(int j, int ld, int nblocks, const double *part_norm, double *H,                 \
                   const double *h2, double *cs, double *sn, double *y, double haptol,             \
                   double rel_floor, void *st, cudaStream_t s);                                    \
    void gm_backsub(int ld, const double *H, double *y, const void *st, cudaStream_t s);           \
    void gm_solution(long long n, const double *V, long long ldv, const double *y,                 \
                     const void *st, double *x, cudaStream_t s);                                   \
    size_t gm_state_bytes();                                                                       \
    /* ---- BiCGSTAB pieces ---- */                                                                \
    size_t bc_state_bytes();                                                                       \
    void bc_dot(long long n, const double *x, const double *y, double *part, const void *st,       \
                cudaStream_t s);                                                                   \
    void bc_start(int nb, const double *part, void *st, int maxiter, cudaStream_t s);              \
    void bc_direction(long long n, const void *st, const double *r, const double *v, double *p,   \
                      double *pt, cudaStream_t s);                                                 \
    void bc_alpha(int nb, const double *part, void *st, cudaStream_t s);                           \
    void bc_s(long long n, const void *st, const double *r, const double *v, double *sv,          \
              double *shat, cudaStream_t s);                                                       \
    void bc_fused5(long long n, const double *rt, const double *sv, const double *t, double *part, \
                   const void *st, cudaStream_t s);                                                \
    void bc_omega(int nb, const double *part, void *st, double tol, double *hist, cudaStream_t s);  \
    void bc_update(long long n, const void *st, const double *pt, const double *shat,             \
                   const double *sv, const double *t, double *x, double *r, cudaStream_t s);       \
    void bc_advance(void *st, int maxiter, cudaStream_t s);                                        \
    void norm2_to(long long n, const double *x, double *part, double *out, cudaStream_t s);

namespace kexact {
UCFD_DECLARE_LAUNCHERS
}
namespace kfast {
UCFD_DECLARE_LAUNCHERS
}
