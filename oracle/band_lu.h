/*
 * Banded LU with partial pivoting in LAPACK general-band (GB) storage, FP64.
 * TEST INFRASTRUCTURE (oracle): the checker's linear solver, never shipped on
 * the product path.
 *
 * Storage follows the reference's BandMatrix (reference src/BandMatrix.cpp:
 * 214,246 — entry (i,j) at m[(kl+ku+i-j) + j*ldab], ldab = 2*kl+ku+1,
 * column-major, the top kl rows hold the fill created by row swaps) and the
 * LAPACK dgbtrf/dgbtrs contract that reference src/BandMatrix.cpp:257-287
 * calls.  The reference's live Newton path calls PARDISO (reference
 * src/SparseMatrix.cpp:74-166), which is not available here; a direct FP64
 * LU with partial pivoting on the same matrix is the stated substitute.
 */
#ifndef GIRAFFE_ORACLE_BAND_LU_H
#define GIRAFFE_ORACLE_BAND_LU_H
#include <math.h>
#include <stddef.h>

#define GB_AT(ab, ldab, kl, ku, i, j) ((ab)[(size_t)((kl) + (ku) + (i) - (j)) + (size_t)(j) * (size_t)(ldab)])

/* Factor in place.  Returns 0, or j+1 for the first exactly-zero pivot
 * (dgbtrf's info > 0), after which the factor is incomplete. */
static inline int oracle_gbtrf(int n, int kl, int ku, double* ab, int ldab, int* ipiv) {
  const int kv = kl + ku;
  int info = 0;
  /* the fill rows (0..kl-1 of every column) start at zero */
  for (int j = 0; j < n; ++j)
    for (int r = 0; r < kl; ++r) ab[(size_t)r + (size_t)j * ldab] = 0.0;
  int ju = 0; /* last column touched by the U part so far */
  for (int j = 0; j < n; ++j) {
    int km = kl < n - 1 - j ? kl : n - 1 - j;
    double* col = ab + (size_t)j * ldab;
    int jp = 0;
    double best = fabs(col[kv]);
    for (int r = 1; r <= km; ++r) {
      double v = fabs(col[kv + r]);
      if (v > best) { best = v; jp = r; }
    }
    ipiv[j] = j + jp;
    if (col[kv + jp] == 0.0) {
      if (!info) info = j + 1;
      continue;
    }
    int jl = j + ku + jp < n - 1 ? j + ku + jp : n - 1;
    if (jl > ju) ju = jl;
    if (jp != 0)
      for (int c = j; c <= ju; ++c) {
        double* a = &GB_AT(ab, ldab, kl, ku, j, c);
        double* b = &GB_AT(ab, ldab, kl, ku, j + jp, c);
        double t = *a; *a = *b; *b = t;
      }
    double inv = 1.0 / col[kv];
    for (int r = 1; r <= km; ++r) col[kv + r] *= inv;
    for (int c = j + 1; c <= ju; ++c) {
      double u = GB_AT(ab, ldab, kl, ku, j, c);
      if (u == 0.0) continue;
      for (int r = 1; r <= km; ++r) GB_AT(ab, ldab, kl, ku, j + r, c) -= col[kv + r] * u;
    }
  }
  return info;
}

/* Solve A x = b with the factor from oracle_gbtrf; b is overwritten by x. */
static inline void oracle_gbtrs(int n, int kl, int ku, const double* ab, int ldab, const int* ipiv,
                                double* b) {
  const int kv = kl + ku;
  for (int j = 0; j < n; ++j) {
    int p = ipiv[j];
    if (p != j) { double t = b[j]; b[j] = b[p]; b[p] = t; }
    int km = kl < n - 1 - j ? kl : n - 1 - j;
    const double* col = ab + (size_t)j * ldab;
    for (int r = 1; r <= km; ++r) b[j + r] -= col[kv + r] * b[j];
  }
  for (int j = n - 1; j >= 0; --j) {
    const double* col = ab + (size_t)j * ldab;
    b[j] /= col[kv];
    int top = j - kv > 0 ? j - kv : 0;
    for (int i = top; i < j; ++i) b[i] -= col[kv + i - j] * b[j];
  }
}
#endif
