/*
 * Banded LU with partial pivoting in LAPACK general-band (GB) storage, FP64.
 * TEST INFRASTRUCTURE (oracle): the oracle's linear solver, never shipped on
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
#include <stdlib.h>
#include <string.h>

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
/* ---- reverse Cuthill-McKee reordering ----
 * PARDISO, the reference's solver, reorders the matrix before factoring
 * (nested dissection, reference src/SparseMatrix.cpp:93-94); this banded
 * substitute reorders by reverse Cuthill-McKee where that narrows the band,
 * so decks whose numbering spreads coupled DOFs far apart (corner nodes
 * first, midside nodes after) keep a narrow band. */

static int oracle_cmp_int(const void* a, const void* b) {
  int x = *(const int*)a, y = *(const int*)b;
  return (x > y) - (x < y);
}

/* Symmetric adjacency (CSR, 0-based, no self loops, sorted, unique) of n
 * vertices from np pairs (pi[k], pj[k]).  *xadj and *adj are malloc'ed. */
static inline void oracle_graph(int n, size_t np, const int* pi, const int* pj, int** xadj, int** adj) {
  int* deg = (int*)calloc((size_t)n + 1, sizeof(int));
  for (size_t k = 0; k < np; ++k)
    if (pi[k] != pj[k]) { deg[pi[k]]++; deg[pj[k]]++; }
  int* x = (int*)malloc(sizeof(int) * ((size_t)n + 1));
  x[0] = 0;
  for (int i = 0; i < n; ++i) x[i + 1] = x[i] + deg[i];
  int* a = (int*)malloc(sizeof(int) * ((size_t)x[n] + 1));
  memset(deg, 0, sizeof(int) * (size_t)n);
  for (size_t k = 0; k < np; ++k)
    if (pi[k] != pj[k]) {
      a[x[pi[k]] + deg[pi[k]]++] = pj[k];
      a[x[pj[k]] + deg[pj[k]]++] = pi[k];
    }
  /* sort and compact each row */
  int w = 0;
  for (int i = 0; i < n; ++i) {
    int lo = x[i], hi = x[i + 1];
    qsort(a + lo, (size_t)(hi - lo), sizeof(int), oracle_cmp_int);
    x[i] = w;
    for (int p = lo; p < hi; ++p)
      if (p == lo || a[p] != a[p - 1]) a[w++] = a[p];
  }
  x[n] = w;
  free(deg);
  *xadj = x;
  *adj = a;
}

/* Breadth-first levels from r over the unvisited component; returns the
 * last vertex of minimum degree in the deepest level and its depth. */
static inline int oracle_bfs_far(int r, const int* x, const int* a, const char* done, int* lvl, int* q, int* depth,
                                 int* nq) {
  int h = 0, t = 0;
  q[t++] = r;
  lvl[r] = 0;
  while (h < t) {
    int v = q[h++];
    for (int p = x[v]; p < x[v + 1]; ++p) {
      int u = a[p];
      if (!done[u] && lvl[u] < 0) { lvl[u] = lvl[v] + 1; q[t++] = u; }
    }
  }
  int d = lvl[q[t - 1]], best = q[t - 1];
  for (int k = t - 1; k >= 0 && lvl[q[k]] == d; --k)
    if (x[q[k] + 1] - x[q[k]] <= x[best + 1] - x[best]) best = q[k];
  for (int k = 0; k < t; ++k) lvl[q[k]] = -1;
  *depth = d;
  *nq = t;
  return best;
}

/* perm[old] = new position under reverse Cuthill-McKee: each component
 * starts at a pseudo-peripheral vertex (George and Liu: repeated
 * breadth-first search from a minimum-degree vertex of the last level while
 * the depth grows), neighbours are queued by increasing degree, and the
 * whole order is reversed. */
static inline void oracle_rcm(int n, const int* x, const int* a, int* perm) {
  char* done = (char*)calloc((size_t)n + 1, 1);
  int* lvl = (int*)malloc(sizeof(int) * ((size_t)n + 1));
  int* q = (int*)malloc(sizeof(int) * ((size_t)n + 1));
  int* order = (int*)malloc(sizeof(int) * ((size_t)n + 1));
  for (int i = 0; i < n; ++i) lvl[i] = -1;
  int placed = 0;
  while (placed < n) {
    int r = -1;
    for (int i = 0; i < n; ++i)
      if (!done[i] && (r < 0 || x[i + 1] - x[i] < x[r + 1] - x[r])) r = i;
    int d, nq, d2;
    int far = oracle_bfs_far(r, x, a, done, lvl, q, &d, &nq);
    for (int guard = 0; guard < n; ++guard) {
      int far2 = oracle_bfs_far(far, x, a, done, lvl, q, &d2, &nq);
      if (d2 <= d) break;
      r = far;
      far = far2;
      d = d2;
    }
    r = far;
    int h = placed, t = placed;
    order[t++] = r;
    done[r] = 1;
    while (h < t) {
      int v = order[h++];
      int s0 = t;
      for (int p = x[v]; p < x[v + 1]; ++p) {
        int u = a[p];
        if (!done[u]) { done[u] = 1; order[t++] = u; }
      }
      /* by increasing degree (insertion sort: rows are short) */
      for (int i = s0 + 1; i < t; ++i) {
        int u = order[i], du = x[u + 1] - x[u], j = i - 1;
        while (j >= s0 && x[order[j] + 1] - x[order[j]] > du) { order[j + 1] = order[j]; --j; }
        order[j + 1] = u;
      }
    }
    placed = t;
  }
  for (int k = 0; k < n; ++k) perm[order[k]] = n - 1 - k;
  free(done); free(lvl); free(q); free(order);
}

/* Half-bandwidth max |perm[i] - perm[j]| over the graph's edges. */
static inline int oracle_perm_bandwidth(int n, const int* x, const int* a, const int* perm) {
  int b = 0;
  for (int i = 0; i < n; ++i)
    for (int p = x[i]; p < x[i + 1]; ++p) {
      int d = perm[i] - perm[a[p]];
      if (d < 0) d = -d;
      if (d > b) b = d;
    }
  return b;
}
#endif