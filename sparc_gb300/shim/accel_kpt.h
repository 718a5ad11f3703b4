/*
 * accel_kpt.h -- SPARC's k-point accelerator hooks mapped onto libsparc_gpu.so (included by
 * src/eigenSolverKpt.c:54-56, src/forces.c, src/pressure.c and src/stress.c when SPARC is
 * compiled with -DSPARCX_ACCEL -DACCEL).
 *
 *  - ACCEL_ChebyshevFiltering_kpt (src/eigenSolverKpt.c:235-241): the complex128 filter on
 *    the GPU with the block's Bloch vector, then H*Y into X (Project_Hamiltonian_kpt skips its
 *    own H*Y when the hook is active, src/eigenSolverKpt.c:693-697);
 *  - ACCEL_ZGEMM and ZHEGV: the host BLAS and LAPACK;
 *  - k-point force, pressure and stress hooks: SPARC's own CPU routines.
 */
#ifndef SPARC_GB300_ACCEL_KPT_H
#define SPARC_GB300_ACCEL_KPT_H

#include <complex.h>
#include <mpi.h>
#include <cblas.h>
#include <lapacke.h>
#include "isddft.h"
#include "sparc_gpu.h"

void gb300_ChebyshevFiltering_kpt(SPARC_OBJ *pSPARC, int *DMVertices, double _Complex *X,
                                  int ldi, double _Complex *Y, int ldo, int ncol, int m,
                                  double a, double b, double a0, int kpt, int spn_i,
                                  MPI_Comm comm);

void Calculate_nonlocal_forces_kpt(SPARC_OBJ *pSPARC);
void Calculate_nonlocal_pressure_kpt(SPARC_OBJ *pSPARC);
void Calculate_nonlocal_kinetic_stress_kpt(SPARC_OBJ *pSPARC);

#define ACCEL_ChebyshevFiltering_kpt gb300_ChebyshevFiltering_kpt
#define ACCEL_ZGEMM cblas_zgemm
/* the complex subspace eigenproblem stays on the host LAPACK (src/eigenSolverKpt.c:854) */
#define ZHEGV LAPACKE_zhegvd
#define STR_ZGEMM "cblas_zgemm (host)"
#define STR_ZHEGV "LAPACKE_zhegvd (host)"
#define ACCEL_Calculate_nonlocal_forces_kpt Calculate_nonlocal_forces_kpt
#define ACCEL_Calculate_nonlocal_pressure_kpt Calculate_nonlocal_pressure_kpt
#define ACCEL_Calculate_nonlocal_kinetic_stress_kpt Calculate_nonlocal_kinetic_stress_kpt

#endif
