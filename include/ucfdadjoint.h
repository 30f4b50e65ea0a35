/*
 * ucfdadjoint.h -- differentiable colored LU-SGS step (GB300 extension; the
 * reference has no adjoint).
 *
 * UCFDColoredStep runs the colored step of coloredlusgs.h -- pre, lower
 * sweep colour by colour, upper sweep in reverse colour order -- on device
 * arrays of one precision, without the update (upts + dq is left to the
 * caller), keeping the intermediates the reverse pass needs:
 *   diag [neles], dub = dQ* [nvars][neles] (lower sweep),
 *   dq = dQ [nvars][neles] (upper sweep).
 * Variables [0, nfvars) are swept with the Euler flux.  UCFD_PREC_FP64 uses
 * the bit-exact FP64 kernels (the same arithmetic as the array API),
 * UCFD_PREC_FP64_FMA the fused ones, UCFD_PREC_FP32 float arrays.  icolor
 * lists the cells colour by colour; ranges (a HOST array of ncolors
 * entries) holds the exclusive end of each colour in icolor; lcolor is the
 * colour of each cell.
 *
 * UCFDColoredStepAdjoint is its reverse-mode derivative: given gdq = dL/ddQ
 * it returns grhs = dL/drhs, gdt = dL/ddt and gfspr = dL/dfspr (geometry
 * and upts held fixed), running the transposed upper sweep (colours
 * ascending) and then the transposed lower sweep (colours descending).
 * rface [nface][neles] is the reverse-face map (UCFDReverseFaces); work
 * holds (2*nfvars + 1)*neles elements of the working precision.
 *
 * All arrays except ranges must be device memory.  With stream != NULL the
 * calls are ordered on that CUDA stream and return without synchronising;
 * with NULL they run on the default stream and complete before returning.
 */
#pragma once

#include "ucfd_gb300.h"

#if defined(__cplusplus)
extern "C" {
#endif

/* rface[f][i] = index of the face of cell nei_ele[f][i] that points back
 * to i (f itself for boundary faces, which point to i); host arrays. */
UCFD_EXTERN ucfd_status_t UCFDReverseFaces(int neles, int nface, const int *nei_ele, int *rface);

UCFD_EXTERN ucfd_status_t UCFDColoredStep(int precision, int neles, int nface, int nvars, int nfvars, int ndims,
                                          const int *nei_ele, const int *icolor, int ncolors, const int *ranges,
                                          const int *lcolor, double factor, const void *fnorm_vol,
                                          const void *vec_fnorm, const void *fspr, const void *dt,
                                          const void *upts, const void *rhs, void *diag, void *dub, void *dq,
                                          void *stream);

UCFD_EXTERN ucfd_status_t UCFDColoredStepAdjoint(int precision, int neles, int nface, int nvars, int nfvars,
                                                 int ndims, const int *nei_ele, const int *rface,
                                                 const int *icolor, int ncolors, const int *ranges,
                                                 const int *lcolor, double factor, const void *fnorm_vol,
                                                 const void *vec_fnorm, const void *fspr, const void *dt,
                                                 const void *upts, const void *diag, const void *dub,
                                                 const void *dq, const void *gdq, void *grhs, void *gdt,
                                                 void *gfspr, void *work, void *stream);

#if defined(__cplusplus)
}
#endif
