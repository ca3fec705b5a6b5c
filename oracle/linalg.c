/*
 * oracle/linalg.c -- FP64 dense kernels for the CPU oracle.
 *
 * ORACLE / TEST INFRASTRUCTURE: linked only into the oracle (the compiled
 * reference in oracle/_ref and the CPU port in oracle/port).  Nothing in the
 * product links it.
 *
 * The reference links an unpinned system BLAS/LAPACK (makefile:10) and a
 * vendored LINPACK routine (src/dchex.f).  These are restatements written from
 * the published definitions, column-major, in the loop order of the netlib
 * reference BLAS, so the oracle's rounding is fixed:
 *   ddot/dgemv/dtrmv/dtrsv/dsyrk/drotg  -- netlib BLAS level 1/2/3 semantics
 *   dpotrf_ ('U')                        -- unblocked upper Cholesky (dpotf2)
 *   dchex_ (job 2, left circular shift)  -- src/dchex.f:130-245
 */
#include <math.h>
#include <stddef.h>
#include "shim/cblas.h"

#define A_(i, j) a[(size_t)(j) * (size_t)lda + (size_t)(i)]

double cblas_ddot(const int n, const double* x, const int incx,
                  const double* y, const int incy)
{
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += x[(size_t)i * incx] * y[(size_t)i * incy];
  return s;
}

void cblas_dgemv(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE trans,
                 const int m, const int n, const double alpha, const double* a,
                 const int lda, const double* x, const int incx,
                 const double beta, double* y, const int incy)
{
  (void)order; /* column-major only */
  if (trans == CblasNoTrans) {
    for (int i = 0; i < m; ++i) y[(size_t)i * incy] = (beta == 0.0) ? 0.0 : beta * y[(size_t)i * incy];
    for (int j = 0; j < n; ++j) {
      double t = alpha * x[(size_t)j * incx];
      for (int i = 0; i < m; ++i) y[(size_t)i * incy] += t * A_(i, j);
    }
  } else {
    for (int j = 0; j < n; ++j) {
      double t = 0.0;
      for (int i = 0; i < m; ++i) t += A_(i, j) * x[(size_t)i * incx];
      y[(size_t)j * incy] = (beta == 0.0) ? alpha * t : alpha * t + beta * y[(size_t)j * incy];
    }
  }
}

/* upper triangular only (the reference passes CblasUpper everywhere) */
void cblas_dtrmv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO uplo,
                 const enum CBLAS_TRANSPOSE trans, const enum CBLAS_DIAG diag,
                 const int n, const double* a, const int lda, double* x,
                 const int incx)
{
  (void)order; (void)uplo;
  int unit = (diag == CblasUnit);
  if (trans == CblasNoTrans) {
    for (int j = 0; j < n; ++j) {
      double t = x[(size_t)j * incx];
      for (int i = 0; i < j; ++i) x[(size_t)i * incx] += t * A_(i, j);
      if (!unit) x[(size_t)j * incx] = t * A_(j, j);
    }
  } else {
    for (int j = n - 1; j >= 0; --j) {
      double t = x[(size_t)j * incx];
      if (!unit) t *= A_(j, j);
      for (int i = j - 1; i >= 0; --i) t += A_(i, j) * x[(size_t)i * incx];
      x[(size_t)j * incx] = t;
    }
  }
}

void cblas_dtrsv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO uplo,
                 const enum CBLAS_TRANSPOSE trans, const enum CBLAS_DIAG diag,
                 const int n, const double* a, const int lda, double* x,
                 const int incx)
{
  (void)order; (void)uplo;
  int unit = (diag == CblasUnit);
  if (trans == CblasNoTrans) {
    /* solve U x = b, back substitution in column (axpy) form */
    for (int j = n - 1; j >= 0; --j) {
      if (x[(size_t)j * incx] != 0.0) {
        if (!unit) x[(size_t)j * incx] /= A_(j, j);
        double t = x[(size_t)j * incx];
        for (int i = j - 1; i >= 0; --i) x[(size_t)i * incx] -= t * A_(i, j);
      }
    }
  } else {
    /* solve U' x = b, forward substitution in dot form */
    for (int j = 0; j < n; ++j) {
      double t = x[(size_t)j * incx];
      for (int i = 0; i < j; ++i) t -= A_(i, j) * x[(size_t)i * incx];
      if (!unit) t /= A_(j, j);
      x[(size_t)j * incx] = t;
    }
  }
}

/* C := alpha A' A + beta C, upper part (trans = CblasTrans, A is k x n) */
void cblas_dsyrk(const enum CBLAS_ORDER order, const enum CBLAS_UPLO uplo,
                 const enum CBLAS_TRANSPOSE trans, const int n, const int k,
                 const double alpha, const double* a, const int lda,
                 const double beta, double* c, const int ldc)
{
  (void)order; (void)uplo; (void)trans;
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i <= j; ++i) {
      double t = 0.0;
      for (int l = 0; l < k; ++l) t += A_(l, i) * A_(l, j);
      double* cij = &c[(size_t)j * ldc + i];
      *cij = (beta == 0.0) ? alpha * t : alpha * t + beta * *cij;
    }
  }
}

/* Givens rotation, netlib drotg semantics: on exit a = r, b = z. */
void cblas_drotg(double* a, double* b, double* c, double* s)
{
  double sa = *a, sb = *b;
  double roe = (fabs(sa) > fabs(sb)) ? sa : sb;
  double scale = fabs(sa) + fabs(sb);
  double r, z;
  if (scale == 0.0) {
    *c = 1.0; *s = 0.0; r = 0.0; z = 0.0;
  } else {
    double ta = sa / scale, tb = sb / scale;
    r = scale * sqrt(ta * ta + tb * tb);
    if (roe < 0.0) r = -r;
    *c = sa / r;
    *s = sb / r;
    z = 1.0;
    if (fabs(sa) > fabs(sb)) z = *s;
    if (fabs(sb) >= fabs(sa) && *c != 0.0) z = 1.0 / *c;
  }
  *a = r;
  *b = z;
}

/* Upper Cholesky A = U'U in place (LAPACK dpotrf with uplo 'U'). */
void dpotrf_(char* uplo, int* np, double* a, int* ldap, int* info)
{
  (void)uplo;
  int n = *np, lda = *ldap;
  *info = 0;
  for (int j = 0; j < n; ++j) {
    double ajj = A_(j, j);
    for (int l = 0; l < j; ++l) ajj -= A_(l, j) * A_(l, j);
    if (ajj <= 0.0 || isnan(ajj)) {
      A_(j, j) = ajj;
      *info = j + 1;
      return;
    }
    ajj = sqrt(ajj);
    A_(j, j) = ajj;
    /* row j to the right: (a(j, j+1:n) - a(0:j-1, j)' a(0:j-1, j+1:n)) / ajj */
    for (int c = j + 1; c < n; ++c) {
      double t = A_(j, c);
      for (int l = 0; l < j; ++l) t -= A_(l, j) * A_(l, c);
      A_(j, c) = t / ajj;
    }
  }
}

/* declared by the reference (src/symmmatrix.hpp:35) but never called */
void dpotri_(char* uplo, int* n, double* a, int* lda, int* info)
{
  (void)uplo; (void)n; (void)a; (void)lda;
  *info = -1;
}

/*
 * dchex_: update an upper Cholesky factor R (p x p, leading dim ldr) under a
 * circular shift of columns k..l (1-based).  Only job 2 (left circular shift:
 * column k moves to position l, columns k+1..l move one left) is used by the
 * reference (src/symmmatrix.cpp:178 with k = removed column, l = p), and only
 * job 2 is restated here (src/dchex.f:130-220); z is not used (nz = 0).
 * c, s receive the rotations (length >= l - k).
 */
void dchex_(double* r, int* ldrp, int* pp, int* kp, int* lp, double* z,
            int* ldz, int* nz, double* c, double* s, int* job)
{
  (void)z; (void)ldz; (void)nz;
  if (*job != 2) return;
  const int ldr = *ldrp, p = *pp, k = *kp, l = *lp;
#define R_(i, j) r[(size_t)((j) - 1) * (size_t)ldr + (size_t)((i) - 1)]
  const int km1 = k - 1, lmk = l - k;
  /* reorder the columns: save column k (rows 1..k) at s(lmk+1..lmk+k) */
  for (int i = 1; i <= k; ++i) s[(lmk + i) - 1] = R_(i, k);
  for (int j = k; j <= l - 1; ++j) {
    for (int i = 1; i <= j; ++i) R_(i, j) = R_(i, j + 1);
    s[(j - km1) - 1] = R_(j + 1, j + 1);
  }
  for (int i = 1; i <= k; ++i) R_(i, l) = s[(lmk + i) - 1];
  for (int i = k + 1; i <= l; ++i) R_(i, l) = 0.0;
  /* reduction loop */
  for (int j = k; j <= p; ++j) {
    if (j != k) {
      int iu = (j - 1 < l - 1) ? j - 1 : l - 1;
      for (int i = k; i <= iu; ++i) {
        int ii = i - k + 1;
        double t = c[ii - 1] * R_(i, j) + s[ii - 1] * R_(i + 1, j);
        R_(i + 1, j) = c[ii - 1] * R_(i + 1, j) - s[ii - 1] * R_(i, j);
        R_(i, j) = t;
      }
    }
    if (j < l) {
      int jj = j - k + 1;
      double t = s[jj - 1];
      cblas_drotg(&R_(j, j), &t, &c[jj - 1], &s[jj - 1]);
    }
  }
#undef R_
}
