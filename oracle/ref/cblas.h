/*
 * Minimal CBLAS declarations used to compile the reference (ibim-levelset)
 * against the LP64 OpenBLAS that ships inside SciPy's wheel.  That library
 * exports its CBLAS entry points with a `scipy_` prefix, so each name the
 * reference calls (blas_wraper.cpp:14-135, ls_point.h:45-140) is mapped here.
 *
 * Test infrastructure only: this header is used by oracle/Makefile to build
 * oracle/_ref/, the reference's own CPU code that pins the oracle.
 */
#ifndef IBIM_ORACLE_CBLAS_SHIM_H
#define IBIM_ORACLE_CBLAS_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };

void scipy_cblas_dcopy(int n, const double *x, int incx, double *y, int incy);
void scipy_cblas_daxpy(int n, double a, const double *x, int incx, double *y, int incy);
void scipy_cblas_dscal(int n, double a, double *x, int incx);
double scipy_cblas_ddot(int n, const double *x, int incx, const double *y, int incy);
double scipy_cblas_dnrm2(int n, const double *x, int incx);
void scipy_cblas_dgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb,
                       int m, int n, int k, double alpha, const double *a, int lda,
                       const double *b, int ldb, double beta, double *c, int ldc);
void scipy_cblas_dgemv(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, int m, int n,
                       double alpha, const double *a, int lda, const double *x, int incx,
                       double beta, double *y, int incy);
void scipy_cblas_dger(enum CBLAS_ORDER order, int m, int n, double alpha, const double *x,
                      int incx, const double *y, int incy, double *a, int lda);
void scipy_cblas_dsbmv(enum CBLAS_ORDER order, enum CBLAS_UPLO uplo, int n, int k,
                       double alpha, const double *a, int lda, const double *x, int incx,
                       double beta, double *y, int incy);

#ifdef __cplusplus
}
#endif

#define cblas_dcopy scipy_cblas_dcopy
#define cblas_daxpy scipy_cblas_daxpy
#define cblas_dscal scipy_cblas_dscal
#define cblas_ddot scipy_cblas_ddot
#define cblas_dnrm2 scipy_cblas_dnrm2
#define cblas_dgemm scipy_cblas_dgemm
#define cblas_dgemv scipy_cblas_dgemv
#define cblas_dger scipy_cblas_dger
#define cblas_dsbmv scipy_cblas_dsbmv

#endif
