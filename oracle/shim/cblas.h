/*
 * Stand-in for <cblas.h>: the CBLAS subset the reference calls
 * (src/vector.hpp:157, src/vector.cpp:95,161,176, src/symmmatrix.cpp:95,237).
 * Implemented in oracle/linalg.c from the BLAS definitions.
 * ORACLE / TEST INFRASTRUCTURE.
 */
#ifndef BMG_SHIM_CBLAS_H_
#define BMG_SHIM_CBLAS_H_

#ifdef __cplusplus
extern "C" {
#endif

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 };

double cblas_ddot(const int n, const double* x, const int incx,
                  const double* y, const int incy);
void cblas_dgemv(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE trans,
                 const int m, const int n, const double alpha, const double* a,
                 const int lda, const double* x, const int incx,
                 const double beta, double* y, const int incy);
void cblas_dtrmv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO uplo,
                 const enum CBLAS_TRANSPOSE trans, const enum CBLAS_DIAG diag,
                 const int n, const double* a, const int lda, double* x,
                 const int incx);
void cblas_dtrsv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO uplo,
                 const enum CBLAS_TRANSPOSE trans, const enum CBLAS_DIAG diag,
                 const int n, const double* a, const int lda, double* x,
                 const int incx);
void cblas_dsyrk(const enum CBLAS_ORDER order, const enum CBLAS_UPLO uplo,
                 const enum CBLAS_TRANSPOSE trans, const int n, const int k,
                 const double alpha, const double* a, const int lda,
                 const double beta, double* c, const int ldc);
void cblas_drotg(double* a, double* b, double* c, double* s);

#ifdef __cplusplus
}
#endif

#endif
