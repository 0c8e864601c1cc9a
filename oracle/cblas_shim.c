/*
 * TEST INFRASTRUCTURE ONLY (part of the oracle).
 *
 * A minimal CBLAS subset so that the reference's own FP64 hot-path sources
 * (src/d2/centroid_Bregman.c, src/d2/centroid_util.c, src/d2/centroid_rand.c,
 * src/utils/blas_like64.c) link without an external BLAS.  The reference
 * binds OpenBLAS (make.inc.Linux64:11); its summation order is unpinned, so
 * this shim fixes one: the netlib reference-BLAS loop order, i.e. plain
 * left-to-right accumulation.  The C restatement in d2_oracle.c follows the
 * same order, which is what makes the two bit-identical.
 *
 * Prototypes follow include/utils/cblas.h:31,55,90,92,132,446 of the
 * reference (enums at :10-11).
 */
#include <stddef.h>

enum CBLAS_ORDER {CblasRowMajor = 101, CblasColMajor = 102};
enum CBLAS_TRANSPOSE {CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113};

double cblas_ddot(const int n, const double *x, const int incx,
                  const double *y, const int incy) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += x[(size_t)i * incx] * y[(size_t)i * incy];
  return s;
}

double cblas_dasum(const int n, const double *x, const int incx) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) {
    double v = x[(size_t)i * incx];
    s += v < 0 ? -v : v;
  }
  return s;
}

void cblas_dcopy(const int n, const double *x, const int incx, double *y, const int incy) {
  for (int i = 0; i < n; ++i) y[(size_t)i * incy] = x[(size_t)i * incx];
}

void cblas_daxpy(const int n, const double alpha, const double *x, const int incx,
                 double *y, const int incy) {
  if (alpha == 0.0) return;
  for (int i = 0; i < n; ++i) y[(size_t)i * incy] += alpha * x[(size_t)i * incx];
}

void cblas_dscal(const int n, const double alpha, double *x, const int incx) {
  for (int i = 0; i < n; ++i) x[(size_t)i * incx] *= alpha;
}

/* Column-major C(m x n) = alpha * op(A) op(B) + beta * C, netlib DGEMM loop
 * order: for each column j, scale C(:,j) by beta, then for l ascending add
 * alpha*op(B)(l,j) * op(A)(:,l).  Row-major calls are mapped onto the
 * column-major kernel by the usual transpose identity. */
static void dgemm_colmajor(int ta, int tb, int m, int n, int k, double alpha,
                           const double *a, int lda, const double *b, int ldb,
                           double beta, double *c, int ldc) {
  for (int j = 0; j < n; ++j) {
    double *cj = c + (size_t)j * ldc;
    if (beta == 0.0) {
      for (int i = 0; i < m; ++i) cj[i] = 0.0;
    } else if (beta != 1.0) {
      for (int i = 0; i < m; ++i) cj[i] *= beta;
    }
    if (!ta) {
      for (int l = 0; l < k; ++l) {
        double blj = tb ? b[j + (size_t)l * ldb] : b[l + (size_t)j * ldb];
        double t = alpha * blj;
        const double *al = a + (size_t)l * lda;
        for (int i = 0; i < m; ++i) cj[i] += t * al[i];
      }
    } else {
      for (int i = 0; i < m; ++i) {
        double s = 0.0;
        const double *ai = a + (size_t)i * lda;
        for (int l = 0; l < k; ++l) {
          double blj = tb ? b[j + (size_t)l * ldb] : b[l + (size_t)j * ldb];
          s += ai[l] * blj;
        }
        cj[i] += alpha * s;
      }
    }
  }
}

void cblas_dgemm(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE ta,
                 const enum CBLAS_TRANSPOSE tb, const int m, const int n, const int k,
                 const double alpha, const double *a, const int lda,
                 const double *b, const int ldb, const double beta,
                 double *c, const int ldc) {
  int tA = ta != CblasNoTrans, tB = tb != CblasNoTrans;
  if (order == CblasColMajor)
    dgemm_colmajor(tA, tB, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
  else /* C^T = op(B)^T op(A)^T in column-major terms */
    dgemm_colmajor(tB, tA, n, m, k, alpha, b, ldb, a, lda, beta, c, ldc);
}
