/*
 * Shared helpers of the CPU oracle.  TEST INFRASTRUCTURE: the oracle gives
 * the values the CUDA path is tested against and the timed CPU baseline; only tests/, the
 * smoke check and bench.py's CPU legs load it.  It is a plain restatement of
 * the reference's algorithm, not part of the product.
 *
 * Conventions: 3x3 matrices are row-major double[9]; element matrices are
 * column-major like the reference's Matrix class (reference
 * src/Matrix.cpp:97 stores (i,j) at i + j*lines).
 */
#ifndef GIRAFFE_ORACLE_COMMON_H
#define GIRAFFE_ORACLE_COMMON_H
#include <math.h>
#include <string.h>

#include "../include/giraffe_model.h"

#define OR_PI 3.1415926535897932384626433832795

static inline void m3_zero(double* a) { memset(a, 0, 9 * sizeof(double)); }
static inline void m3_eye(double* a) { m3_zero(a); a[0] = a[4] = a[8] = 1.0; }
static inline void m3_copy(double* d, const double* s) { memcpy(d, s, 9 * sizeof(double)); }
static inline void m3_mul(double* c, const double* a, const double* b) {
  double t[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t[i * 3 + j] = a[i * 3] * b[j] + a[i * 3 + 1] * b[3 + j] + a[i * 3 + 2] * b[6 + j];
  m3_copy(c, t);
}
/* c = a^T b */
static inline void m3_tmul(double* c, const double* a, const double* b) {
  double t[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t[i * 3 + j] = a[i] * b[j] + a[3 + i] * b[3 + j] + a[6 + i] * b[6 + j];
  m3_copy(c, t);
}
/* c = a b^T */
static inline void m3_mult(double* c, const double* a, const double* b) {
  double t[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      t[i * 3 + j] = a[i * 3] * b[j * 3] + a[i * 3 + 1] * b[j * 3 + 1] + a[i * 3 + 2] * b[j * 3 + 2];
  m3_copy(c, t);
}
static inline void m3_transpose(double* d, const double* a) {
  double t[9] = {a[0], a[3], a[6], a[1], a[4], a[7], a[2], a[5], a[8]};
  m3_copy(d, t);
}
static inline void m3_vec(double* y, const double* a, const double* x) {
  double t0 = a[0] * x[0] + a[1] * x[1] + a[2] * x[2];
  double t1 = a[3] * x[0] + a[4] * x[1] + a[5] * x[2];
  double t2 = a[6] * x[0] + a[7] * x[1] + a[8] * x[2];
  y[0] = t0; y[1] = t1; y[2] = t2;
}
/* y = a^T x */
static inline void m3_tvec(double* y, const double* a, const double* x) {
  double t0 = a[0] * x[0] + a[3] * x[1] + a[6] * x[2];
  double t1 = a[1] * x[0] + a[4] * x[1] + a[7] * x[2];
  double t2 = a[2] * x[0] + a[5] * x[1] + a[8] * x[2];
  y[0] = t0; y[1] = t1; y[2] = t2;
}
/* Inverse of a 3x3 matrix (row-major) by its adjugate over the determinant. */
static inline void m3_inverse(double* r, const double* a) {
  const double c00 = a[4] * a[8] - a[5] * a[7], c01 = a[5] * a[6] - a[3] * a[8], c02 = a[3] * a[7] - a[4] * a[6];
  const double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
  const double id = 1.0 / det;
  r[0] = c00 * id;
  r[1] = (a[2] * a[7] - a[1] * a[8]) * id;
  r[2] = (a[1] * a[5] - a[2] * a[4]) * id;
  r[3] = c01 * id;
  r[4] = (a[0] * a[8] - a[2] * a[6]) * id;
  r[5] = (a[2] * a[3] - a[0] * a[5]) * id;
  r[6] = c02 * id;
  r[7] = (a[1] * a[6] - a[0] * a[7]) * id;
  r[8] = (a[0] * a[4] - a[1] * a[3]) * id;
}
static inline void m3_skew(double* a, const double* v) {
  a[0] = 0.0;   a[1] = -v[2]; a[2] = v[1];
  a[3] = v[2];  a[4] = 0.0;   a[5] = -v[0];
  a[6] = -v[1]; a[7] = v[0];  a[8] = 0.0;
}
static inline double v3_dot(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline void v3_cross(double* c, const double* a, const double* b) {
  double t0 = a[1] * b[2] - a[2] * b[1], t1 = a[2] * b[0] - a[0] * b[2], t2 = a[0] * b[1] - a[1] * b[0];
  c[0] = t0; c[1] = t1; c[2] = t2;
}
static inline double v3_norm(const double* a) { return sqrt(v3_dot(a, a)); }

/* Rodrigues rotation tensor Q = I + g (A + A^2/2), g = 4/(4+|a|^2)
 * (reference src/Beam_1.cpp:748-752, src/Node.cpp:362-365). */
static inline void rodrigues_Q(double* Q, const double* a) {
  double A[9], A2[9];
  double n = v3_norm(a);
  double g = 4.0 / (4.0 + n * n);
  m3_skew(A, a);
  m3_mul(A2, A, A);
  for (int k = 0; k < 9; ++k) Q[k] = g * (A[k] + 0.5 * A2[k]);
  Q[0] += 1.0; Q[4] += 1.0; Q[8] += 1.0;
}

/* Composition of Rodrigues vectors a_new = 4/(4 - a2.a1) (a2 + a1 + a2 x a1 / 2)
 * (reference src/Node.cpp:342, src/Beam_1.cpp:1502-1503). */
static inline void rodrigues_compose(double* out, const double* a2, const double* a1) {
  double c[3];
  v3_cross(c, a2, a1);
  double f = 4.0 / (4.0 - v3_dot(a2, a1));
  for (int k = 0; k < 3; ++k) out[k] = f * (a2[k] + a1[k] + 0.5 * c[k]);
}

/* V operator for the geometric stiffness (reference src/Matrix.cpp:1999-2012):
 * V(x,t) = (h8 t - h4 x*t) x^T + h2 skew(t), h = 4/(4+|x|^2). */
static inline void op_V(double* V, const double* x, const double* t, double xn) {
  double h = 4.0 / (4.0 + xn * xn);
  double h2 = 0.5 * h, h4 = -0.25 * h * h, h8 = -0.5 * h * h;
  double xt[3], a[3], S[9];
  v3_cross(xt, x, t);
  for (int i = 0; i < 3; ++i) a[i] = h8 * t[i] - h4 * xt[i];
  m3_skew(S, t);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) V[i * 3 + j] = a[i] * x[j] + h2 * S[i * 3 + j];
}

/* d_V operator (reference src/Matrix.cpp:2014-2032), terms with the vanishing
 * coefficients h3, h5, h7 omitted:
 * d_V = (x.dx)(h9 t - h6 x*t) x^T + (h8 t - h4 x*t) dx^T - h4 (dx*t) x^T
 *       + h4 (x.dx) skew(t). */
static inline void op_dV(double* W, const double* x, const double* dx, const double* t, double xn) {
  double h = 4.0 / (4.0 + xn * xn);
  double h4 = -0.25 * h * h, h6 = 0.25 * h * h * h, h8 = -0.5 * h * h, h9 = 0.5 * h * h * h;
  double xt[3], dxt[3], S[9];
  v3_cross(xt, x, t);
  v3_cross(dxt, dx, t);
  double xdx = v3_dot(x, dx);
  m3_skew(S, t);
  for (int i = 0; i < 3; ++i) {
    double a = xdx * (h9 * t[i] - h6 * xt[i]);
    double b = h8 * t[i] - h4 * xt[i];
    double c = -h4 * dxt[i];
    for (int j = 0; j < 3; ++j) W[i * 3 + j] = a * x[j] + b * dx[j] + c * x[j] + h4 * xdx * S[i * 3 + j];
  }
}

/* Piecewise-linear table lookup (reference src/Table.cpp:73-102). */
static inline double table_at(const gf_table* t, double time, int col) {
  if (t->n_times == 0) return 0.0;
  if (time >= t->times[t->n_times - 1]) return t->values[(t->n_times - 1) * t->n_cols + col];
  if (time <= t->times[0]) return t->values[col];
  int idx = 0;
  while (time >= t->times[idx]) idx++;
  double f = (time - t->times[idx - 1]) / (t->times[idx] - t->times[idx - 1]);
  double a = t->values[(idx - 1) * t->n_cols + col], b = t->values[idx * t->n_cols + col];
  return a + f * (b - a);
}

/* Rows E1, E2, E3 of a coordinate system (reference
 * src/CoordinateSystem.cpp:68-92: E2 = E3 x E1, each normalised, Q rows). */
static inline void cs_matrix(double* Q, const double* e1e3) {
  double e1[3] = {e1e3[0], e1e3[1], e1e3[2]}, e3[3] = {e1e3[3], e1e3[4], e1e3[5]}, e2[3];
  v3_cross(e2, e3, e1);
  double n1 = v3_norm(e1), n2 = v3_norm(e2), n3 = v3_norm(e3);
  for (int k = 0; k < 3; ++k) {
    Q[k] = n1 != 1.0 ? e1[k] * (1.0 / n1) : e1[k];
    Q[3 + k] = n2 != 1.0 ? e2[k] * (1.0 / n2) : e2[k];
    Q[6 + k] = n3 != 1.0 ? e3[k] * (1.0 / n3) : e3[k];
  }
}
#endif
