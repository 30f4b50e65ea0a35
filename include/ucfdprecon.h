/*
 * ucfdprecon.h -- preconditioners of libucfd_gb300.so (Krylov path).
 *
 * Drop-in for src/krylov/include/ucfdprecon.h:5-38, BLU-SGS family:
 *   BLUSGS      natural-order block LU-SGS (precon/blusgs.c:7-128); run on
 *               the GPU level by level with the sequential result;
 *   PBLUSGS     coloured block LU-SGS over contiguous colour ranges
 *               icolors[c]..icolors[c+1] (precon/pblusgs.c:7-127; declared
 *               here, missing from the reference header).  The reference
 *               lower apply reads the diagonal block at idx+blkdim
 *               (pblusgs.c:41); this library uses block idx, the intended
 *               one, i.e. the natural-order result of the colour-ordered
 *               matrix;
 *   CUDABLUSGS  same as PBLUSGS (cublusgs.cu:245-278).
 * The arrays of UCFDPreconCreatefromArrays are the BSR matrix (rowptr,
 * colidx, values) plus diagslots[bn], the position of each diagonal block
 * (precon.c:13-27); they are copied to the GPU at Prepare.
 */
#pragma once

#include "ucfdmat.h"

#if defined(__cplusplus)
extern "C" {
#endif

typedef struct _Precon *Precon;   /* ucfdprecon.h:6 */

typedef const char *PreconType;   /* ucfdprecon.h:8-16 */
#define NONE "none"
#define BLUSGS "blu-sgs"
#define PBLUSGS "pblu-sgs"
#define CUDABLUSGS "cudablusgs"

/* ucfdprecon.h:24-27 (precon.c:13-45, none.c:14-30) */
UCFD_EXTERN ucfd_status_t UCFDPreconCreatefromArrays(Precon *pc, UCFDInt *rowptr,
                                                     UCFDInt *colidx, UCFDInt *diagslots,
                                                     UCFDReal *values);
UCFD_EXTERN ucfd_status_t UCFDPreconCreateNone(Precon *pc);
UCFD_EXTERN ucfd_status_t UCFDPreconPrepare(Precon pc);
UCFD_EXTERN ucfd_status_t UCFDPreconDestroy(Precon *pc);

/* ucfdprecon.h:32, blusgs.c:111-128 */
UCFD_EXTERN ucfd_status_t UCFDPreconSetBLUSGS(Precon *pc, UCFDInt bn, UCFDInt block);
/* pblusgs.c:107-127 */
UCFD_EXTERN ucfd_status_t UCFDPreconSetPBLUSGS(Precon *pc, UCFDInt bn, UCFDInt block,
                                               UCFDInt ncolors, UCFDInt *icolors);
/* ucfdprecon.h:36, cublusgs.cu:245-278 */
UCFD_EXTERN ucfd_status_t UCFDPreconSetCUDABLUSGS(Precon *pc, UCFDInt bn, UCFDInt block,
                                                  UCFDInt ncolors, UCFDInt *icolors);

/* ---- GB300 extensions ------------------------------------------------ */
/* Apply the preconditioner in place to b (host or device), the operation
 * the reference calls through its vtable (ucfdsolverimpl.h:47-51). */
UCFD_EXTERN ucfd_status_t UCFDPreconApply(Precon pc, UCFDReal *b);
/* UCFD_PREC_FP32: FP32 block values and FP32 arithmetic in the apply (the
 * diagonal blocks are factored in FP64, then rounded).  Before Prepare. */
UCFD_EXTERN ucfd_status_t UCFDPreconSetPrecision(Precon pc, int precision);
/* Number of parallel levels the apply runs in (after Prepare). */
UCFD_EXTERN ucfd_status_t UCFDPreconGetLevels(Precon pc, UCFDInt *nlevels);

#if defined(__cplusplus)
}
#endif
