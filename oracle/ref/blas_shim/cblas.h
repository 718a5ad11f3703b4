/*
 * CBLAS declarations for building the reference SPARC sources as the CPU oracle against the
 * OpenBLAS that ships inside scipy (its symbols carry a "scipy_" prefix). Test infrastructure.
 */
#ifndef SPARC_ORACLE_CBLAS_SHIM_H
#define SPARC_ORACLE_CBLAS_SHIM_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef CBLAS_LAYOUT CBLAS_ORDER;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
typedef enum { CblasUpper = 121, CblasLower = 122 } CBLAS_UPLO;
typedef enum { CblasNonUnit = 131, CblasUnit = 132 } CBLAS_DIAG;
typedef enum { CblasLeft = 141, CblasRight = 142 } CBLAS_SIDE;

#define cblas_dcopy scipy_cblas_dcopy
#define cblas_ddot  scipy_cblas_ddot
#define cblas_dgemm scipy_cblas_dgemm
#define cblas_dgemv scipy_cblas_dgemv
#define cblas_dger  scipy_cblas_dger
#define cblas_dscal scipy_cblas_dscal
#define cblas_dsyrk scipy_cblas_dsyrk
#define cblas_dtrsm scipy_cblas_dtrsm
#define cblas_zcopy scipy_cblas_zcopy
#define cblas_zgemm scipy_cblas_zgemm
#define cblas_zgemv scipy_cblas_zgemv
#define cblas_zscal scipy_cblas_zscal
#define cblas_ztrsm scipy_cblas_ztrsm

void cblas_dcopy(const int n, const double *x, const int incx, double *y, const int incy);
double cblas_ddot(const int n, const double *x, const int incx, const double *y, const int incy);
void cblas_dgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, const int m,
                 const int n, const int k, const double alpha, const double *a, const int lda,
                 const double *b, const int ldb, const double beta, double *c, const int ldc);
void cblas_dgemv(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, const int m, const int n,
                 const double alpha, const double *a, const int lda, const double *x,
                 const int incx, const double beta, double *y, const int incy);
void cblas_dger(CBLAS_LAYOUT layout, const int m, const int n, const double alpha,
                const double *x, const int incx, const double *y, const int incy, double *a,
                const int lda);
void cblas_dscal(const int n, const double alpha, double *x, const int incx);
void cblas_dsyrk(CBLAS_LAYOUT layout, CBLAS_UPLO uplo, CBLAS_TRANSPOSE t, const int n,
                 const int k, const double alpha, const double *a, const int lda,
                 const double beta, double *c, const int ldc);
void cblas_dtrsm(CBLAS_LAYOUT layout, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE ta,
                 CBLAS_DIAG diag, const int m, const int n, const double alpha, const double *a,
                 const int lda, double *b, const int ldb);
void cblas_zcopy(const int n, const void *x, const int incx, void *y, const int incy);
void cblas_zgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, const int m,
                 const int n, const int k, const void *alpha, const void *a, const int lda,
                 const void *b, const int ldb, const void *beta, void *c, const int ldc);
void cblas_zgemv(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, const int m, const int n,
                 const void *alpha, const void *a, const int lda, const void *x,
                 const int incx, const void *beta, void *y, const int incy);
void cblas_zscal(const int n, const void *alpha, void *x, const int incx);
void cblas_ztrsm(CBLAS_LAYOUT layout, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE ta,
                 CBLAS_DIAG diag, const int m, const int n, const void *alpha, const void *a,
                 const int lda, void *b, const int ldb);
#ifdef __cplusplus
}
#endif
#endif
