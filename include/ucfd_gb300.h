/*
 * ucfd_gb300.h -- common types of libucfd_gb300.so, a GB300 (sm_103a)
 * implementation of UCFD_SPARSE's implicit hot path behind the library's
 * own C entry points.
 *
 * The scalar types and status codes keep the reference's names and values
 * (src/krylov/include/config.h:15-28, src/krylov/include/ucfdtypes.h:13-30)
 * so existing ctypes / C callers bind unchanged.  Two deliberate
 * differences, both observable by callers:
 *   - errors are returned as a nonzero ucfd_status_t (with a message from
 *     UCFDGetLastError) instead of calling exit() (ucfd macros.h:32-70);
 *   - every array argument may be a host pointer or a CUDA device pointer
 *     (the kind is detected per call with cudaPointerGetAttributes); host
 *     arrays are staged to the GPU and results copied back before return.
 */
#pragma once

#include <stddef.h>
#include <stdint.h>

#if defined(__cplusplus)
extern "C" {
#endif

#define UCFD_EXTERN extern __attribute__((visibility("default")))

typedef int32_t UCFDInt;   /* ucfd config.h:18 (UCFD_INT64 unset) */
typedef double UCFDReal;   /* ucfd config.h:27 (UCFD_FLOAT32 unset) */
typedef int8_t UCFDInt8;   /* ucfd ucfdtypes.h:11 */

/* ucfd ucfdtypes.h:13-17 (0 and 1 keep their meaning; 2.. are new). */
typedef enum {
    UCFD_SUCCESS = 0,
    UCFD_FAILED = 1,
    UCFD_ERR_ARGUMENT = 2,    /* invalid size, null pointer, bad layout     */
    UCFD_ERR_CUDA = 3,        /* a CUDA runtime call failed                 */
    UCFD_ERR_NOMEM = 4,       /* device or host allocation failed           */
    UCFD_ERR_UNSUPPORTED = 5, /* e.g. nvars/ndims combination not built     */
    UCFD_ERR_BREAKDOWN = 6,   /* zero pivot / non-finite value detected     */
    UCFD_ERR_TIMEOUT = 7,     /* a bounded device-side wait gave up         */
    UCFD_ERR_STATE = 8        /* call made on an object in the wrong state  */
} ucfd_status_t;

/* ucfd ucfdtypes.h:22-30 */
typedef enum {
    INITIALIZED = -1,
    CONVERGED = 0,
    HAPPYBREAKDOWN = 1,
    REACH_ITERMAX = 2,
    RHOBREAKDOWN = 3,
    PIBREAKDOWN = 4
} ucfd_solver_t;

/* Arithmetic of the sweeps (an addition of this library).
 *  UCFD_PREC_FP64     FP64, compiled without FMA contraction: every cell's
 *                     arithmetic is the reference's, bit for bit (default).
 *  UCFD_PREC_FP64_FMA FP64 with fused multiply-add (faster, last-bit
 *                     differences from the reference).
 *  UCFD_PREC_FP32     FP32 storage and arithmetic in the sweeps and the
 *                     preconditioner; LU factorisations, residuals and
 *                     Krylov orthogonalisation stay FP64. */
typedef enum {
    UCFD_PREC_FP64 = 0,
    UCFD_PREC_FP64_FMA = 1,
    UCFD_PREC_FP32 = 2
} ucfd_precision_t;

/* Message of the last error raised on the calling thread ("" if none). */
UCFD_EXTERN const char *UCFDGetLastError(void);

/* Gas constants used by the Euler flux (ucfd flux.h:18-26: GAMMA 1.4,
 * PMIN 1e-13, BETAST 0.09 -- compile-time macros in the reference,
 * process-wide runtime values here). */
UCFD_EXTERN ucfd_status_t UCFDSetConstants(UCFDReal gamma, UCFDReal pmin, UCFDReal betast);

/* Host<->device copies of caller arrays made by the library (host-pointer
 * arguments are staged to the GPU and results copied back), timed with CUDA
 * events on the copying stream while timing is on.  No counterpart in the
 * reference.  UCFDSetTransferTiming(1) clears the counters and starts
 * timing (each timed copy then waits for its own completion);
 * UCFDSetTransferTiming(0) stops it.  Counters are process-wide. */
typedef struct {
    double h2d_ms, h2d_bytes;  /* host -> device: summed copy time, bytes */
    double d2h_ms, d2h_bytes;  /* device -> host */
    long long h2d_copies, d2h_copies;
} UCFDTransferStats;
UCFD_EXTERN ucfd_status_t UCFDSetTransferTiming(int on);
UCFD_EXTERN ucfd_status_t UCFDGetTransferStats(UCFDTransferStats *stats);

/* How host-memory array arguments reach the GPU (process-wide).
 * UCFD_HOST_STAGE: copied into library device buffers (cudaMemcpyAsync)
 * before the kernels that read them.  UCFD_HOST_MAP (the default): an
 * array in page-locked host memory (cudaHostAlloc / cudaHostRegister / a
 * pinned torch tensor) is read in place by the kernel that consumes it,
 * over the host link, with no copy and no device staging buffer -- where
 * the library supports it: the face Jacobians of UCFDBLUSGS_NSPrepare /
 * RANSPrepare.  Other arrays, and pageable memory, are staged in either
 * mode.  Results are identical.  No counterpart in the reference (a CPU
 * library). */
typedef enum { UCFD_HOST_STAGE = 0, UCFD_HOST_MAP = 1 } ucfd_host_access_t;
UCFD_EXTERN ucfd_status_t UCFDSetHostArrayAccess(int mode);
UCFD_EXTERN int UCFDGetHostArrayAccess(void);

/* Library version string and the device it runs on (diagnostics). */
UCFD_EXTERN const char *UCFDVersion(void);
UCFD_EXTERN ucfd_status_t UCFDDeviceInfo(char *name, size_t len, int *sm_count);

/* Diagnostics: runs the two bounded device waits of the sweeps (the grid
 * barrier of the persistent scalar sweep, the mbarrier wait of the
 * bulk-copy block sweep) on states that never complete and reports
 * whether each gave up as designed (1) -- instead of hanging -- leaving the
 * context usable.  No counterpart in the reference. */
UCFD_EXTERN ucfd_status_t UCFDSelfTestTimeouts(int *barrier_timed_out, int *mbarrier_timed_out);

#if defined(__cplusplus)
}
#endif
