/*
 * ucfdlusgs.h -- FlowSys LU-SGS / block LU-SGS API of libucfd_gb300.so.
 *
 * Drop-in for the reference header src/lusgs/include/ucfdlusgs.h:5-40:
 * same handle type, function names, argument order and array layouts.
 *   rowptr/colidx/slots/sides  rank-level CSR over faces (flowsys.h:34-59)
 *   face_area [nfaces], face_normal [ndims][nfaces], rcp_vol [nlocal]
 *   element arrays (SetElement): uptsb, rhs, dsrc, resid_out [nvars][neles];
 *   dt, vol [neles]; cell_ids [neles] maps element -> rank cell
 *   LU-SGS fspr/tfspr [nfaces]; BLU-SGS jmat [2][nfvars][nfvars][nfaces],
 *   tjmat [2][nturb][nturb][nfaces]
 *
 * Sweep semantics are the reference's natural-order Gauss-Seidel
 * (lusgs.c:157-257, blusgs.c:273-373).  On the GPU the rank cells are
 * processed level by level: level(i) = 1 + max level of i's lower-indexed
 * neighbours, so every cell sees exactly the neighbour values the
 * sequential sweep would show it and the result is the sequential one.
 * UCFDFlowSysSetColoring replaces natural order by a colour order (the
 * colored LU-SGS of the reference documentation), which equals the natural
 * order of the colour-renumbered mesh.
 *
 * Like the reference, the object keeps the caller's pointers (host or
 * device) without copying.  The mesh arrays (CSR, face_area, face_normal,
 * rcp_vol) are read once, at the first Prepare/sweep; fspr/tfspr and
 * jmat/tjmat are read by each Prepare; element arrays by Pack, Update and
 * SubResidual.  All calls are complete when they return.
 */
#pragma once

#include "ucfd_gb300.h"

#if defined(__cplusplus)
extern "C" {
#endif

typedef struct _FlowSys *FlowSys;   /* ucfdlusgs.h:5 */

/* ---- common (ucfdlusgs.h:8-14, flowsys.c:6-54,120-140) ---------------- */
UCFD_EXTERN ucfd_status_t UCFDFlowSysCreate(FlowSys *sys, UCFDInt nlocal, UCFDInt nvars,
                                            UCFDInt nfvars, UCFDInt ndims, UCFDInt nfaces,
                                            UCFDInt nelem, UCFDInt *rowptr, UCFDInt *colidx,
                                            UCFDInt *slots, UCFDInt8 *sides,
                                            UCFDReal *face_area, UCFDReal *face_normal,
                                            UCFDReal *rcp_vol);
UCFD_EXTERN ucfd_status_t UCFDFlowSysSetElement(FlowSys *sys, UCFDInt eidx, UCFDInt neles,
                                                UCFDInt nface, UCFDInt *cell_ids,
                                                UCFDReal *uptsb, UCFDReal *rhs, UCFDReal *dt,
                                                UCFDReal *dsrc, UCFDReal *vol,
                                                UCFDReal *resid_out);
UCFD_EXTERN ucfd_status_t UCFDFlowSysDestroy(FlowSys *sys);

/* ---- scalar LU-SGS (ucfdlusgs.h:17-25, lusgs.c) ----------------------- */
UCFD_EXTERN ucfd_status_t UCFDFlowSysSetLUSGS(FlowSys *sys, UCFDReal *fspr, UCFDReal *tfspr);
UCFD_EXTERN ucfd_status_t UCFDLUSGS_Pack(FlowSys sys, UCFDInt eidx, UCFDReal turb_factor,
                                         UCFDReal a0);
UCFD_EXTERN ucfd_status_t UCFDLUSGS_Update(FlowSys sys, UCFDInt eidx);
UCFD_EXTERN ucfd_status_t UCFDLUSGS_NSPrepare(FlowSys sys, UCFDReal kappa);
UCFD_EXTERN ucfd_status_t UCFDLUSGS_RANSPrepare(FlowSys sys, UCFDReal kappa);
UCFD_EXTERN ucfd_status_t UCFDLUSGS_NSLowerSweep(FlowSys sys, UCFDReal kappa);
UCFD_EXTERN ucfd_status_t UCFDLUSGS_NSUpperSweep(FlowSys sys, UCFDReal kappa);
UCFD_EXTERN ucfd_status_t UCFDLUSGS_RANSLowerSweep(FlowSys sys, UCFDReal kappa);
UCFD_EXTERN ucfd_status_t UCFDLUSGS_RANSUpperSweep(FlowSys sys, UCFDReal kappa);
/* Both systems in one call: NSRANSPrepare gives the values of NSPrepare
 * followed by RANSPrepare, NSRANSLowerSweep those of NSLowerSweep followed
 * by RANSLowerSweep, NSRANSUpperSweep those of NSUpperSweep followed by
 * RANSUpperSweep (each system's sweep reads only the state and its own
 * increments, so the two are independent).  With one thread per cell
 * (sweep_variant 0-2) one kernel serves both systems and loads each
 * neighbour index, face normal, area and mean-flow state once; the other
 * variants run the two sweeps one after the other.  No counterpart in the
 * reference, whose callers make the NS and RANS calls one by one. */
UCFD_EXTERN ucfd_status_t UCFDLUSGS_NSRANSPrepare(FlowSys sys, UCFDReal kappa);
UCFD_EXTERN ucfd_status_t UCFDLUSGS_NSRANSLowerSweep(FlowSys sys, UCFDReal kappa);
UCFD_EXTERN ucfd_status_t UCFDLUSGS_NSRANSUpperSweep(FlowSys sys, UCFDReal kappa);

/* ---- block LU-SGS (ucfdlusgs.h:28-40, blusgs.c) ----------------------- */
UCFD_EXTERN ucfd_status_t UCFDFlowSysSetBLUSGS(FlowSys *sys, UCFDReal *jmat, UCFDReal *tjmat);
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_Pack(FlowSys sys, UCFDInt eidx, UCFDReal a0);
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_KWSST_Pack(FlowSys sys, UCFDInt eidx, UCFDReal turb_factor,
                                                UCFDReal a0);
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_SA_Pack(FlowSys sys, UCFDInt eidx, UCFDReal turb_factor,
                                             UCFDReal a0);
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_Update(FlowSys sys, UCFDInt eidx);
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_SubResidual(FlowSys sys, UCFDInt eidx);
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_NSPrepare(FlowSys sys);
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_RANSPrepare(FlowSys sys);
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_NSLowerSweep(FlowSys sys);
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_RANSLowerSweep(FlowSys sys);
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_NSUpperSweep(FlowSys sys);
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_RANSUpperSweep(FlowSys sys);
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_Reset(FlowSys sys);

/* ======================================================================
 * GB300 extensions (no counterpart in the reference header).
 * ==================================================================== */

/* Sweep in colour order instead of natural order.  color[r] (0-based, any
 * range) is the colour of rank cell r; cells of one colour must not be
 * neighbours (UCFD_ERR_ARGUMENT otherwise).  Lower sweeps visit colours in
 * increasing order, upper sweeps in decreasing order.  Pass NULL to return
 * to natural order.  Must be called before the first Prepare. */
UCFD_EXTERN ucfd_status_t UCFDFlowSysSetColoring(FlowSys sys, const UCFDInt *color);
/* Greedy first-fit colouring of the CSR graph in rank order, applied as by
 * UCFDFlowSysSetColoring; *ncolors receives the number of colours. */
UCFD_EXTERN ucfd_status_t UCFDFlowSysColorGreedy(FlowSys sys, UCFDInt *ncolors);
/* Number of parallel levels of the current sweep schedule. */
UCFD_EXTERN ucfd_status_t UCFDFlowSysGetLevels(FlowSys sys, UCFDInt *nlevels);
/* Arithmetic of the sweeps (ucfd_precision_t); before the first Prepare. */
UCFD_EXTERN ucfd_status_t UCFDFlowSysSetPrecision(FlowSys sys, int precision);
/* Launch shape of the sweep kernels (0 = autotuned default). */
UCFD_EXTERN ucfd_status_t UCFDFlowSysSetLaunch(FlowSys sys, int threads_per_block);

/* Launch choices of the sweeps.  None of them changes any result: every
 * choice applies the same operations to each cell in the same order.
 * No counterpart in the reference (its launch shape is the compile-time
 * TPB/BLOCK macro of Makefile.inc). */
typedef struct {
    int threads_per_block; /* sweep kernels: 0 (default 256) or 32..256 step 32 */
    int sweep_variant;     /* block sweep: 0 faces unrolled to the ELL width, 1 face loop,
                              2 / 3 FP32 5x5 with J and LU tiles staged in shared memory
                              by bulk copies (2 / 1 buffers per warp; ELL width 6 or 4),
                              4 = 0 launched as a programmatic dependent of the previous
                              colour (its start overlaps the previous colour's tail);
                              5 = 0 for the block sweep;
                              scalar sweeps: 0 default build, 1 / 2 capped at 80 / 64
                              registers (more resident warps), 3 / 4 two threads per
                              cell, 5 one thread per active face (per-level launches;
                              the persistent kernel keeps one thread per cell) */
    int run_mode;          /* UCFDLUSGS_Run with mode -1: 0 CUDA graph, 1 persistent kernel */
    double ms;             /* Autotune: time of the best candidate (one sweep pair, or one
                              Run iteration for scalar LU-SGS); 0 when set by hand */
} UCFDLaunchConfig;

/* Times every launch candidate on the current system and keeps the fastest.
 * Block LU-SGS (after Pack + NSPrepare): threads_per_block x sweep_variant
 * on lower+upper sweep pairs into a scratch correction.  Scalar LU-SGS
 * (after Pack; fspr set): threads_per_block x sweep_variant x run_mode on
 * the iteration of UCFDLUSGS_Run -- with the turbulence system when the
 * handle has one and tfspr is set -- the state saved before and restored
 * after.  reps >= 1
 * timed repetitions per candidate after one untimed one.  Synchronises. */
UCFD_EXTERN ucfd_status_t UCFDFlowSysAutotune(FlowSys sys, int reps, UCFDLaunchConfig *best);
UCFD_EXTERN ucfd_status_t UCFDFlowSysGetLaunchConfig(FlowSys sys, UCFDLaunchConfig *cfg);
UCFD_EXTERN ucfd_status_t UCFDFlowSysSetLaunchConfig(FlowSys sys, const UCFDLaunchConfig *cfg);
/* Run all kernels of a call on the caller's CUDA stream and return without
 * synchronising (stream == NULL restores the private stream and synchronous
 * calls).  Host-pointer arguments still synchronise. */
UCFD_EXTERN ucfd_status_t UCFDFlowSysSetStream(FlowSys sys, void *cuda_stream, int async);

/* Scalar LU-SGS pseudo-time loop on device-resident state: niter times
 * { du = rhs; NS prepare; NS lower; NS upper; [RANS prepare/lower/upper];
 *   u += du }, launched as one CUDA graph (mode 0) or as one persistent
 * grid-synchronised kernel per sweep (mode 1); mode -1 takes the run_mode
 * of the launch configuration (UCFDFlowSysAutotune).  Requires a prior Pack of
 * every element.  resid (optional, [niter]) receives sqrt(sum du^2)
 * accumulated to FP64 accuracy after each iteration.  Update() afterwards
 * writes the final state back to the element arrays.  With UCFD_PREC_FP32
 * the sweeps read the FP32 state while u += du accumulates into a
 * float-float pair (the FP32 state plus an FP32 low part made at Pack, 48
 * significant bits), so increments below the state's FP32 rounding unit
 * are not lost; Update() writes the pair's sum back.  With the
 * turbulence system and one thread per cell (sweep_variant 0-2, and the
 * persistent kernel) one kernel prepares both systems and one launch per
 * level sweeps both: the two sweeps read only the state and their own
 * increments, so the values are those of the separate calls, with each
 * neighbour index, face normal, area and mean-flow state loaded once. */
UCFD_EXTERN ucfd_status_t UCFDLUSGS_Run(FlowSys sys, UCFDInt niter, UCFDReal kappa, int rans,
                                        int mode, UCFDReal *resid);

/* Block LU-SGS linear solve on device-resident state after Pack + Prepare:
 * sweeps (lower+upper pairs) until ||rhs - A du||_2 <= rtol ||rhs||_2 or
 * max_sweeps pairs.  With UCFD_PREC_FP32 the sweeps run in FP32 inside FP64
 * iterative refinement (FP64 true residual every inner_sweeps pairs).
 * Writes the pairs used and the final relative residual. */
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_Solve(FlowSys sys, UCFDReal rtol, UCFDInt max_sweeps,
                                           UCFDInt inner_sweeps, UCFDInt *nsweeps,
                                           UCFDReal *relres);
/* FP64 relative residual ||rhs - A du|| / ||rhs|| of the packed NS system. */
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_Residual(FlowSys sys, UCFDReal *relres);

/* The same residual, computed without allocating anything (no counterpart
 * in the reference).  For callers that may not call cudaMalloc while they
 * run -- a code that gives its whole device memory to its own pool at
 * start-up, or whose time-step loop must not stall on an allocation -- yet
 * monitor the residual every iteration.  The reduction partials live in a
 * fixed 64 KiB device array inside the library (held by every GPU that
 * loads it until exit); systems above 8,388,608 cells are rejected with
 * UCFD_ERR_ARGUMENT.  The system must already be packed and prepared
 * (UCFD_ERR_STATE otherwise).  relres may be host or device memory; the
 * call returns once it is written.  It runs on the device holding the
 * handle's arrays and restores the caller's current device.  The first
 * call on a device looks up the array's address: make it before any stream
 * capture.  All calls share the array, so calls whose kernels overlap on
 * the GPU (unordered streams) race. */
UCFD_EXTERN ucfd_status_t UCFDBLUSGS_ResidualNoAlloc(FlowSys sys, UCFDReal *relres);

#if defined(__cplusplus)
}
#endif
