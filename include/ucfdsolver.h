/*
 * ucfdsolver.h -- Krylov solvers of libucfd_gb300.so.
 *
 * Drop-in for src/krylov/include/ucfdsolver.h:5-31 (GMRES, BiCGSTAB).  GMRES(m) is
 * left-preconditioned with classical Gram-Schmidt plus one
 * re-orthogonalisation and Givens rotations, stopping when the absolute
 * true residual ||b - A x|| <= tol is seen at a restart (gmres.c:42-129).
 * Everything runs on the GPU: Arnoldi passes are fused, the Givens / least-
 * squares step runs on the device, and one restart cycle is replayed as a
 * CUDA graph with a single host synchronisation per restart.  BiCGSTAB is
 * right-preconditioned with the fused five-term reduction and the residual
 * estimate of bicgstab.c:24-128, stopping when the estimate drops below tol
 * (absolute); its scalars stay on the device and the host reads the stop
 * flag every few iterations.  Where s = r - alpha v is exactly zero the
 * reference's omega = (t,s)/(t,t) is 0/0; here omega = 0 and the solve
 * ends converged.  x and b may be host or device arrays of
 * n = bn*blk values.
 */
#pragma once

#include "ucfdprecon.h"

#if defined(__cplusplus)
extern "C" {
#endif

typedef struct _Solver *Solver;   /* ucfdsolver.h:6 */

typedef const char *SolverType;   /* ucfdsolver.h:8-10 */
#define GMRES "gmres"
#define BICGSTAB "bicgstab"

/* ucfdsolver.h:17-23, solver.c:5-69 */
UCFD_EXTERN ucfd_status_t UCFDSolverInit(Solver *solver);
UCFD_EXTERN ucfd_status_t UCFDSolverDestroy(Solver *solver);
UCFD_EXTERN ucfd_status_t UCFDSolve(Solver solver, Precon pc, SpMat A, UCFDReal *x,
                                    UCFDReal *b);
UCFD_EXTERN ucfd_status_t UCFDSolverGetResult(Solver solver, UCFDInt *stat, UCFDInt *iter,
                                              UCFDReal *residual);
UCFD_EXTERN ucfd_status_t UCFDSolverTraceResidualHistory(Solver solver);
UCFD_EXTERN ucfd_status_t UCFDSolverGetResidualHistory(Solver solver, UCFDReal *hist);

/* ucfdsolver.h:25, gmres.c:153-178; ucfdsolver.h:28, cugmres.cu:253-300 */
UCFD_EXTERN ucfd_status_t UCFDSolverCreateGMRES(Solver *solver, UCFDInt n, UCFDInt m,
                                                UCFDInt maxiter, UCFDReal tol);
UCFD_EXTERN ucfd_status_t UCFDSolverCreateCUDAGMRES(Solver *solver, UCFDInt n, UCFDInt m,
                                                    UCFDInt maxiter, UCFDReal tol);
/* ucfdsolver.h:26, bicgstab.c:156-179 */
UCFD_EXTERN ucfd_status_t UCFDSolverCreateBICGSTAB(Solver *solver, UCFDInt n, UCFDInt maxiter,
                                                   UCFDReal tol);

/* ---- GB300 extensions ------------------------------------------------ */
/* UCFD_PREC_FP64 (default): the reference's arithmetic in every product.
 * UCFD_PREC_FP64_FMA: the same sums with fused multiply-adds (not
 * bit-matched to the reference).
 * UCFD_PREC_FP32: mixed-precision GMRES -- inside each restart cycle the
 * matrix-vector products use FP32 values and the preconditioner runs in
 * FP32, while the Arnoldi orthogonalisation, Givens/least-squares solve and
 * the true residual b - A x at every restart stay FP64 (iterative
 * refinement; the residual's product with fused multiply-adds).  Before
 * the first UCFDSolve. */
UCFD_EXTERN ucfd_status_t UCFDSolverSetPrecision(Solver solver, int precision);
/* Happy-breakdown tolerance (default 1e-12, solver.c:11). */
UCFD_EXTERN ucfd_status_t UCFDSolverSetHappyTol(Solver solver, UCFDReal haptol);
/* GMRES in the FP64 modes: with on != 0 a restart cycle also ends once its
 * residual estimate has fallen by the factor the true residual still needs
 * to reach tol (with a margin of 10), instead of always building m Krylov
 * vectors; the restart then checks the true residual as usual.  Default
 * off: the reference's iteration (gmres.c:62-125).  The mixed-precision
 * mode always ends a cycle at the FP32 operator's accuracy. */
UCFD_EXTERN ucfd_status_t UCFDSolverSetCycleExit(Solver solver, int on);
/* Total Arnoldi steps of the last solve. */
UCFD_EXTERN ucfd_status_t UCFDSolverGetArnoldiSteps(Solver solver, UCFDInt *steps);

#if defined(__cplusplus)
}
#endif
