/*
 * accel.h -- SPARC's accelerator hook surface mapped onto libsparc_gpu.so.
 *
 * SPARC compiled with -DSPARCX_ACCEL -DACCEL includes this header (src/eigenSolver.c:51-53,
 * src/forces.c:40, src/pressure.c:46, src/stress.c:45, src/linearScaling/sq.c:36,
 * src/highT/sqHighT.c:29) and calls the ACCEL_* names below instead of its CPU routines;
 * initialization.c then sets pSPARC->useACCEL = 1 (src/initialization.c:384-402). No SPARC
 * source is modified: this file, accel_kpt.h and sparc_gb300_shim.c are the whole binding.
 *
 * What runs where:
 *  - ACCEL_ChebyshevFiltering (src/eigenSolver.c:314-321): the FP64 filter on the GPU, then
 *    H*Y into X, because DP_Project_Hamiltonian skips its own H*Y when the hook is active
 *    (src/eigenSolver.c:953-958);
 *  - DSYGV / DSYEV (src/eigenSolver.c:1276-1281, :483, :1695): the subspace eigenproblem on
 *    the GPU (sgpu_Solve_Generalized_EigenProblem / sgpu_Solve_Standard_EigenProblem);
 *  - ACCEL_Calculate_nonlocal_forces_linear (src/forces.c:726-729): the nonlocal forces on
 *    the GPU for spin-unpolarised runs, SPARC's own routine otherwise;
 *  - ACCEL_DGEMM / ACCEL_DTRSM: the host BLAS, as SPARC's non-accelerated path calls it;
 *  - pressure and stress hooks: SPARC's own CPU routines; the SQ (spectral quadrature) hook
 *    is not provided by this library and stops the run with a message.
 */
#ifndef SPARC_GB300_ACCEL_H
#define SPARC_GB300_ACCEL_H

#include <mpi.h>
#include <cblas.h>
#include <lapacke.h>
#include "isddft.h"
#include "sparc_gpu.h"

void gb300_ChebyshevFiltering(SPARC_OBJ *pSPARC, int *DMVertices, double *X, int ldi,
                              double *Y, int ldo, int ncol, int m, double a, double b,
                              double a0, int k, int spn_i, MPI_Comm comm);
int gb300_dsygv(int layout, int itype, char jobz, char uplo, int n, double *A, int lda,
                double *B, int ldb, double *w);
int gb300_dsyev(int layout, char jobz, char uplo, int n, double *A, int lda, double *w);
void gb300_nonlocal_forces_linear(SPARC_OBJ *pSPARC);
void gb300_not_provided(const char *what);

/* SPARC's own CPU routines used by the hooks this library does not take over */
void Calculate_nonlocal_pressure_linear(SPARC_OBJ *pSPARC);
void Calculate_nonlocal_kinetic_stress_linear(SPARC_OBJ *pSPARC);

#define ACCEL_ChebyshevFiltering gb300_ChebyshevFiltering
#define ACCEL_DGEMM cblas_dgemm
#define ACCEL_DTRSM cblas_dtrsm
#define DSYGV gb300_dsygv
#define DSYEV gb300_dsyev
#define STR_DGEMM "cblas_dgemm (host)"
#define STR_DSYGV "sgpu_Solve_Generalized_EigenProblem (GPU)"
#define STR_DSYEV "sgpu_Solve_Standard_EigenProblem (GPU)"
#define ACCEL_Calculate_nonlocal_forces_linear gb300_nonlocal_forces_linear
#define ACCEL_Calculate_nonlocal_pressure_linear Calculate_nonlocal_pressure_linear
#define ACCEL_Calculate_nonlocal_kinetic_stress_linear Calculate_nonlocal_kinetic_stress_linear
#define ACCEL_SQ_LanczosAlgorithm_gauss(...) gb300_not_provided("spectral-quadrature Lanczos")

#endif
