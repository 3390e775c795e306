/*
 * Plain BLAS/LAPACK entry points linked into the reference build
 * (oracle/_ref) in place of Intel oneMKL, which the reference links
 * (reference src/Matrix.cpp:243-246 calls cblas_dgemm/cblas_dgemv with
 * CblasColMajor).  This is TEST INFRASTRUCTURE: it only serves the
 * reference build that pins the oracle and is never part of the product
 * path.
 *
 * Loop order is the textbook one (k innermost, ascending); MKL's blocked
 * order is unknown and unpinned, so results agree with an MKL build to
 * rounding, not bit for bit.
 */
#include <stdio.h>
#include <stdlib.h>

enum { RowMajor = 101, ColMajor = 102, NoTrans = 111, Trans = 112 };

static double at(const double* a, int lda, int i, int j, int trans) {
  return trans ? a[j + (size_t)i * lda] : a[i + (size_t)j * lda];
}

void cblas_dgemm(int layout, int ta, int tb, int m, int n, int k, double alpha,
                 const double* a, int lda, const double* b, int ldb, double beta,
                 double* c, int ldc) {
  if (layout != ColMajor) { fprintf(stderr, "ref_blas: row-major dgemm unsupported\n"); abort(); }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      double s = 0.0;
      for (int p = 0; p < k; ++p) s += at(a, lda, i, p, ta != NoTrans) * at(b, ldb, p, j, tb != NoTrans);
      c[i + (size_t)j * ldc] = alpha * s + (beta == 0.0 ? 0.0 : beta * c[i + (size_t)j * ldc]);
    }
}

void cblas_dgemv(int layout, int ta, int m, int n, double alpha, const double* a, int lda,
                 const double* x, int incx, double beta, double* y, int incy) {
  if (layout != ColMajor) { fprintf(stderr, "ref_blas: row-major dgemv unsupported\n"); abort(); }
  int rows = ta == NoTrans ? m : n, cols = ta == NoTrans ? n : m;
  for (int i = 0; i < rows; ++i) {
    double s = 0.0;
    for (int p = 0; p < cols; ++p) s += at(a, lda, i, p, ta != NoTrans) * x[(size_t)p * incx];
    y[(size_t)i * incy] = alpha * s + (beta == 0.0 ? 0.0 : beta * y[(size_t)i * incy]);
  }
}

/* Dense LU with partial pivoting (column-major), the LAPACK dgetrf contract. */
void dgetrf(const int* pm, const int* pn, double* a, const int* plda, int* ipiv, int* info) {
  int m = *pm, n = *pn, lda = *plda, mn = m < n ? m : n;
  *info = 0;
  for (int j = 0; j < mn; ++j) {
    int p = j;
    double best = -1.0;
    for (int i = j; i < m; ++i) {
      double v = a[i + (size_t)j * lda];
      v = v < 0 ? -v : v;
      if (v > best) { best = v; p = i; }
    }
    ipiv[j] = p + 1;
    if (a[p + (size_t)j * lda] == 0.0) { if (!*info) *info = j + 1; continue; }
    if (p != j)
      for (int c = 0; c < n; ++c) {
        double t = a[j + (size_t)c * lda];
        a[j + (size_t)c * lda] = a[p + (size_t)c * lda];
        a[p + (size_t)c * lda] = t;
      }
    double piv = a[j + (size_t)j * lda];
    for (int i = j + 1; i < m; ++i) a[i + (size_t)j * lda] /= piv;
    for (int c = j + 1; c < n; ++c) {
      double u = a[j + (size_t)c * lda];
      if (u != 0.0)
        for (int i = j + 1; i < m; ++i) a[i + (size_t)c * lda] -= a[i + (size_t)j * lda] * u;
    }
  }
}

void dgetrs(const char* trans, const int* pn, const int* nrhs, const double* a, const int* plda,
            const int* ipiv, double* b, const int* pldb, int* info) {
  int n = *pn, lda = *plda, ldb = *pldb;
  (void)trans;
  *info = 0;
  for (int r = 0; r < *nrhs; ++r) {
    double* x = b + (size_t)r * ldb;
    for (int i = 0; i < n; ++i) {
      int p = ipiv[i] - 1;
      if (p != i) { double t = x[i]; x[i] = x[p]; x[p] = t; }
    }
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < i; ++k) x[i] -= a[i + (size_t)k * lda] * x[k];
    for (int i = n - 1; i >= 0; --i) {
      for (int k = i + 1; k < n; ++k) x[i] -= a[i + (size_t)k * lda] * x[k];
      x[i] /= a[i + (size_t)i * lda];
    }
  }
}

static void unsupported(const char* what) {
  fprintf(stderr, "ref_blas: %s is not provided by the oracle build\n", what);
  abort();
}
void dgbtrf(void) { unsupported("dgbtrf"); }
void dgbtrs(void) { unsupported("dgbtrs"); }
void dsyev(void) { unsupported("dsyev"); }
void dsyevr(void) { unsupported("dsyevr"); }
void cblas_sgemm(void) { unsupported("cblas_sgemm"); }
void cblas_sgemv(void) { unsupported("cblas_sgemv"); }
void MKL_Set_Num_Threads(int n) { (void)n; }
void mkl_set_num_threads(int n) { (void)n; }
