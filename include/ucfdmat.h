/*
 * ucfdmat.h -- sparse matrices of libucfd_gb300.so (Krylov path).
 *
 * Drop-in for src/krylov/include/ucfdmat.h:5-48.  Every matrix lives on
 * the GPU: the CPU constructors (CSR, BSR) and the CUDA ones (CUDACSR,
 * CUDABSR) accept host or device arrays and copy them into device memory
 * at creation (the reference keeps the pointers; after changing the values
 * in place call UCFDMatUpdateValues).  UCFDMatMult takes host or device
 * vectors; with beta == 0 it does not read y (the reference forms beta*y
 * regardless).  BSR blocks are row-major [nnzb][blk][blk] and vectors AoS
 * [bn][blk] (sparsemat.c:57-101).
 */
#pragma once

#include "ucfd_gb300.h"

#if defined(__cplusplus)
extern "C" {
#endif

typedef struct _SpMat *SpMat;   /* ucfdmat.h:5 */

typedef const char *SpMatType;  /* ucfdmat.h:7-17 */
#define CSR "csr"
#define BSR "bsr"
#define CSRCUDA "cudacsr"
#define BSRCUDA "cudabsr"

/* ucfdmat.h:25-27, matrix.c:4-31 */
UCFD_EXTERN ucfd_status_t UCFDMatInit(SpMat *mat);
UCFD_EXTERN ucfd_status_t UCFDMatDestroy(SpMat *mat);
UCFD_EXTERN ucfd_status_t UCFDMatMult(UCFDReal alpha, SpMat mat, UCFDReal *x, UCFDReal beta,
                                      UCFDReal *y);

/* ucfdmat.h:30-31 (sparsemat.c:32-50, 104-125) */
UCFD_EXTERN ucfd_status_t UCFDMatCreateCSR(SpMat *mat, UCFDInt n, UCFDInt *rowptr,
                                           UCFDInt *colidx, UCFDReal *values);
UCFD_EXTERN ucfd_status_t UCFDMatCreateBSR(SpMat *mat, UCFDInt bn, UCFDInt blk,
                                           UCFDInt *rowptr, UCFDInt *colidx, UCFDReal *values);
/* ucfdmat.h:40-41 (cusparsemat.cu:45-171) */
UCFD_EXTERN ucfd_status_t UCFDMatCreateCUDACSR(SpMat *mat, UCFDInt n, UCFDInt *rowptr,
                                               UCFDInt *colidx, UCFDReal *values);
UCFD_EXTERN ucfd_status_t UCFDMatCreateCUDABSR(SpMat *mat, UCFDInt bn, UCFDInt blk,
                                               UCFDInt *rowptr, UCFDInt *colidx,
                                               UCFDReal *values);

/* ---- GB300 extensions ------------------------------------------------ */
/* Re-read the values array given at creation (after the caller changed it). */
UCFD_EXTERN ucfd_status_t UCFDMatUpdateValues(SpMat mat);
/* Type name of the matrix (one of the SpMatType strings). */
UCFD_EXTERN ucfd_status_t UCFDMatGetType(SpMat mat, const char **type_name);
/* Matrix-vector product with FP32 values (an FP32 copy of the values made
 * on first use), FP64 vectors and FP64 accumulation. */
UCFD_EXTERN ucfd_status_t UCFDMatMultFP32(UCFDReal alpha, SpMat mat, UCFDReal *x,
                                          UCFDReal beta, UCFDReal *y);
/* The product in a chosen arithmetic: UCFD_PREC_FP64 (= UCFDMatMult, the
 * reference's operation order), UCFD_PREC_FP64_FMA (fused multiply-adds, as
 * the solvers' FMA mode uses it) or UCFD_PREC_FP32 (= UCFDMatMultFP32). */
UCFD_EXTERN ucfd_status_t UCFDMatMultPrecision(UCFDReal alpha, SpMat mat, UCFDReal *x,
                                               UCFDReal beta, UCFDReal *y, int precision);

#if defined(__cplusplus)
}
#endif
