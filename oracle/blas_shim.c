/*
 * Test infrastructure, not product code.
 *
 * Minimal column-major BLAS (dgemm_, dgemv_, dger_) used only to link the
 * reference's own grid library (built from its sources into oracle/_ref/) in
 * a container that has no system BLAS.  The reference calls dgemm_ from
 * src/grid/ref/grid_ref_task_list.c:216-231 (load_pab / store_hab) and its
 * DGEMM backend also references dgemv_ and dger_.  Plain triple loops:
 * correctness only, no blocking.
 */
#include <stddef.h>

static int is_t(char c) { return c == 'T' || c == 't' || c == 'C' || c == 'c'; }

void dgemm_(const char *transa, const char *transb, const int *m, const int *n,
            const int *k, const double *alpha, const double *a, const int *lda,
            const double *b, const int *ldb, const double *beta, double *c,
            const int *ldc) {
  const int ta = is_t(*transa), tb = is_t(*transb);
  for (int j = 0; j < *n; j++) {
    for (int i = 0; i < *m; i++) {
      double acc = 0.0;
      for (int p = 0; p < *k; p++) {
        const double av = ta ? a[p + (size_t)i * *lda] : a[i + (size_t)p * *lda];
        const double bv = tb ? b[j + (size_t)p * *ldb] : b[p + (size_t)j * *ldb];
        acc += av * bv;
      }
      double *cij = &c[i + (size_t)j * *ldc];
      *cij = (*beta == 0.0) ? *alpha * acc : *alpha * acc + *beta * *cij;
    }
  }
}

void dgemv_(const char *trans, const int *m, const int *n, const double *alpha,
            const double *a, const int *lda, const double *x, const int *incx,
            const double *beta, double *y, const int *incy) {
  const int t = is_t(*trans);
  const int ny = t ? *n : *m, nx = t ? *m : *n;
  for (int i = 0; i < ny; i++) {
    double acc = 0.0;
    for (int p = 0; p < nx; p++) {
      const double av = t ? a[p + (size_t)i * *lda] : a[i + (size_t)p * *lda];
      acc += av * x[(size_t)p * *incx];
    }
    double *yi = &y[(size_t)i * *incy];
    *yi = (*beta == 0.0) ? *alpha * acc : *alpha * acc + *beta * *yi;
  }
}

void dger_(const int *m, const int *n, const double *alpha, const double *x,
           const int *incx, const double *y, const int *incy, double *a,
           const int *lda) {
  for (int j = 0; j < *n; j++)
    for (int i = 0; i < *m; i++)
      a[i + (size_t)j * *lda] +=
          *alpha * x[(size_t)i * *incx] * y[(size_t)j * *incy];
}
