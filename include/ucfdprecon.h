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
 *   CUDABLUSGS  same as PBLUSGS (cublusgs.cu:245-278);
 *   BILU        block ILU(0) (precon/bilu.c:5-158): the factorisation runs on
 *               the GPU level by level (each row once its lower neighbours
 *               are final, the sequential result), the apply as unit-lower
 *               then block-upper triangular sweeps;
 *   PBILU       coloured block ILU(0) over colour ranges (pbilu.c:5-207),
 *               equal to BILU on the colour-ordered matrix (pbilu.c:12,19
 *               shares one column map among its OpenMP threads, so the
 *               reference's own result is defined only with one thread);
 *   CUDABILU    same as PBILU (cubilu.cu:322-351);
 *   ILU         scalar ILU(0) of a CSR matrix (precon/ilu.c:4-117).  The
 *               reference's backward loop starts at the diagonal slot
 *               (ilu.c:81), subtracting a_ii b_i before dividing by a_ii;
 *               this library solves the intended U b = y.
 * As in the reference, Prepare of the ILU types overwrites the values
 * array given to UCFDPreconCreatefromArrays with the factors (do not share
 * it with the matrix).
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
#define ILU "ilu"
#define BILU "bilu"
#define PBILU "pbilu"
#define CUDABILU "cudabilu"

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

/* ucfdprecon.h:30, ilu.c:99-117 */
UCFD_EXTERN ucfd_status_t UCFDPreconSetILU(Precon *pc, UCFDInt n);
/* ucfdprecon.h:31, bilu.c:138-158 */
UCFD_EXTERN ucfd_status_t UCFDPreconSetBILU(Precon *pc, UCFDInt bn, UCFDInt block);
/* ucfdprecon.h:33, pbilu.c:184-207 */
UCFD_EXTERN ucfd_status_t UCFDPreconSetPBILU(Precon *pc, UCFDInt bn, UCFDInt block,
                                             UCFDInt ncolors, UCFDInt *icolors);
/* ucfdprecon.h:35, cubilu.cu:322-351 */
UCFD_EXTERN ucfd_status_t UCFDPreconSetCUDABILU(Precon *pc, UCFDInt bn, UCFDInt block,
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
