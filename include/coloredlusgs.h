/*
 * coloredlusgs.h -- array-based (colored) LU-SGS entry points of
 * libucfd_gb300.so.
 *
 * These are the functions the reference examples bind:
 *   Python ctypes (canonical argument lists): examples/omp3d.py:22-35
 *   (parallel_*) and examples/mpi3d.py:21-34 (serial_*);
 *   C declarations used by examples/omp3d.c:180-189 and mpi3d.c:166-174
 *   (the "dub only" aliases at the end of this header).
 * The reference snapshot has no source for them (the examples include
 * coloredlusgs.h / lusgs.h, which are absent); their meaning comes from
 * README.md:15-50, doc/1_introduction.md:16-26 and doc/3.1_lusgs.md:79-127
 * and equals the FlowSys routines (src/lusgs/lusgs.c) on the colour-
 * renumbered mesh with kappa = 1 and rcp_vol = 1.
 *
 * Layouts (row-major, cell index fastest):
 *   fnorm_vol, fspr, nei_ele [nface][neles]  (boundary faces point to self)
 *   vec_fnorm [nface][ndims][neles] outward unit normals
 *   upts, rhs, dub [nvars][neles];  dt, diag [neles]
 *   icolor [neles] cells listed colour by colour; lcolor [neles] colour of
 *   each cell (any integers; "lower" = smaller colour)
 * Per the README, the lower sweep writes dQ* into dub, the upper sweep
 * writes dQ into rhs, and the update adds rhs into upts.  A parallel sweep
 * call processes icolor[n0:ne) (one colour); serial sweeps process all
 * cells in natural order.  ns_* sweeps update variables [0, nfvars) with
 * the Euler flux, rans_* sweeps variables [nfvars, nvars) with the
 * turbulence convective flux.  nvars / nfvars / ndims are compile-time
 * macros in the reference (Makefile.inc:21-24); here they are set with
 * UCFDLegacySetDims (default 5 / 5 / 3, the Euler 3-D case).
 * Pointers may be host or device memory; every call completes before it
 * returns.
 */
#pragma once

#include "ucfd_gb300.h"

#if defined(__cplusplus)
extern "C" {
#endif

/* Variable counts of the array API (reference: NVARS/NFVARS/NDIMS macros). */
UCFD_EXTERN ucfd_status_t UCFDLegacySetDims(int nvars, int nfvars, int ndims);
/* Arithmetic of the array API sweeps: UCFD_PREC_FP64 (default, bit-exact)
 * or UCFD_PREC_FP64_FMA (the arrays are double, so no FP32 here). */
UCFD_EXTERN ucfd_status_t UCFDLegacySetPrecision(int precision);

/* diag[i] = 1/(dt[i]*factor) + sum_f 0.5*fspr[f,i]*fnorm_vol[f,i] */
UCFD_EXTERN void serial_pre_lusgs(int neles, int nface, double factor, double *fnorm_vol,
                                  double *dt, double *diag, double *fspr);
UCFD_EXTERN void parallel_pre_lusgs(int neles, int nface, double factor, double *fnorm_vol,
                                    double *dt, double *diag, double *fspr);

/* natural-order sweeps (mpi3d.py:23-24, 29-34) */
UCFD_EXTERN void ns_serial_lower_sweep(int neles, int nface, int *nei_ele, double *fnorm_vol,
                                       double *vec_fnorm, double *upts, double *rhs, double *dub,
                                       double *diag, double *fspr);
UCFD_EXTERN void ns_serial_upper_sweep(int neles, int nface, int *nei_ele, double *fnorm_vol,
                                       double *vec_fnorm, double *upts, double *rhs, double *dub,
                                       double *diag, double *fspr);
UCFD_EXTERN void rans_serial_lower_sweep(int neles, int nface, int *nei_ele, double *fnorm_vol,
                                         double *vec_fnorm, double *upts, double *rhs,
                                         double *dub, double *diag, double *fspr);
UCFD_EXTERN void rans_serial_upper_sweep(int neles, int nface, int *nei_ele, double *fnorm_vol,
                                         double *vec_fnorm, double *upts, double *rhs,
                                         double *dub, double *diag, double *fspr);

/* one-colour sweeps over icolor[n0:ne) (omp3d.py:24-25, 30-35, 78-93) */
UCFD_EXTERN void ns_parallel_lower_sweep(int n0, int ne, int neles, int nface, int *nei_ele,
                                         int *icolor, int *lcolor, double *fnorm_vol,
                                         double *vec_fnorm, double *upts, double *rhs,
                                         double *dub, double *diag, double *fspr);
UCFD_EXTERN void ns_parallel_upper_sweep(int n0, int ne, int neles, int nface, int *nei_ele,
                                         int *icolor, int *lcolor, double *fnorm_vol,
                                         double *vec_fnorm, double *upts, double *rhs,
                                         double *dub, double *diag, double *fspr);
UCFD_EXTERN void rans_parallel_lower_sweep(int n0, int ne, int neles, int nface, int *nei_ele,
                                           int *icolor, int *lcolor, double *fnorm_vol,
                                           double *vec_fnorm, double *upts, double *rhs,
                                           double *dub, double *diag, double *fspr);
UCFD_EXTERN void rans_parallel_upper_sweep(int n0, int ne, int neles, int nface, int *nei_ele,
                                           int *icolor, int *lcolor, double *fnorm_vol,
                                           double *vec_fnorm, double *upts, double *rhs,
                                           double *dub, double *diag, double *fspr);

/* upts[k, i] += rhs[k, i] for the equation set's variables
 * (omp3d.py:22, mpi3d.py:21) */
UCFD_EXTERN void lusgs_serial_ns_update(int neles, double *upts, double *rhs);
UCFD_EXTERN void lusgs_parallel_ns_update(int neles, double *upts, double *rhs);
UCFD_EXTERN void lusgs_serial_rans_update(int neles, double *upts, double *rhs);
UCFD_EXTERN void lusgs_parallel_rans_update(int neles, double *upts, double *rhs);

/* C-example spellings (mpi3d.c:166-174, omp3d.c:180-189): no rhs
 * argument; both sweeps read and write dub in place (the FlowSys in-place
 * form, lusgs.c:201 and 253). */
UCFD_EXTERN void serial_ns_lower_sweep(int neles, int nface, int *nei_ele, double *fnorm_vol,
                                       double *vec_fnorm, double *upts, double *dub,
                                       double *diag, double *fspr);
UCFD_EXTERN void serial_ns_upper_sweep(int neles, int nface, int *nei_ele, double *fnorm_vol,
                                       double *vec_fnorm, double *upts, double *dub,
                                       double *diag, double *fspr);
UCFD_EXTERN void serial_ns_lusgs_update(int neles, double *upts, double *dub);
UCFD_EXTERN void parallel_ns_lower_sweep(int n0, int ne, int neles, int nface, int *nei_ele,
                                         int *icolor, int *lcolor, double *fnorm_vol,
                                         double *vec_fnorm, double *upts, double *dub,
                                         double *diag, double *fspr);
UCFD_EXTERN void parallel_ns_upper_sweep(int n0, int ne, int neles, int nface, int *nei_ele,
                                         int *icolor, int *lcolor, double *fnorm_vol,
                                         double *vec_fnorm, double *upts, double *dub,
                                         double *diag, double *fspr);

/* The void entry points above cannot return a status (their reference
 * signatures are void); the last failure is kept here (UCFD_SUCCESS if the
 * last array-API call succeeded; message via UCFDGetLastError). */
UCFD_EXTERN ucfd_status_t UCFDLegacyLastStatus(void);

#if defined(__cplusplus)
}
#endif
