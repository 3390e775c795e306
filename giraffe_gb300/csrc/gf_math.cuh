// Small fixed-size linear algebra used by the element kernels.  Row-major
// 3x3 matrices in registers; everything is inlined.  The rotation helpers
// restate reference src/Matrix.cpp:1812-2032 (skew, V, d_V) and the
// Rodrigues formulas of reference src/Beam_1.cpp:748-754 and
// src/Node.cpp:325-365.
#pragma once
#include <cuda_runtime.h>

#define GF_HD __host__ __device__ __forceinline__

namespace gf {

template <typename T> struct M3 {
  T a[9];
  GF_HD T& operator[](int i) { return a[i]; }
  GF_HD const T& operator[](int i) const { return a[i]; }
};
template <typename T> struct V3 {
  T a[3];
  GF_HD T& operator[](int i) { return a[i]; }
  GF_HD const T& operator[](int i) const { return a[i]; }
};

template <typename T> GF_HD M3<T> eye3() {
  M3<T> r;
#pragma unroll
  for (int i = 0; i < 9; ++i) r[i] = T(0);
  r[0] = r[4] = r[8] = T(1);
  return r;
}
template <typename T> GF_HD M3<T> mul(const M3<T>& a, const M3<T>& b) {
  M3<T> c;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) c[i * 3 + j] = a[i * 3] * b[j] + a[i * 3 + 1] * b[3 + j] + a[i * 3 + 2] * b[6 + j];
  return c;
}
// a^T b
template <typename T> GF_HD M3<T> tmul(const M3<T>& a, const M3<T>& b) {
  M3<T> c;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) c[i * 3 + j] = a[i] * b[j] + a[3 + i] * b[3 + j] + a[6 + i] * b[6 + j];
  return c;
}
template <typename T> GF_HD M3<T> transpose(const M3<T>& a) {
  M3<T> r;
  r[0] = a[0]; r[1] = a[3]; r[2] = a[6];
  r[3] = a[1]; r[4] = a[4]; r[5] = a[7];
  r[6] = a[2]; r[7] = a[5]; r[8] = a[8];
  return r;
}
template <typename T> GF_HD V3<T> mv(const M3<T>& a, const V3<T>& x) {
  V3<T> y;
  y[0] = a[0] * x[0] + a[1] * x[1] + a[2] * x[2];
  y[1] = a[3] * x[0] + a[4] * x[1] + a[5] * x[2];
  y[2] = a[6] * x[0] + a[7] * x[1] + a[8] * x[2];
  return y;
}
// a^T x
template <typename T> GF_HD V3<T> tmv(const M3<T>& a, const V3<T>& x) {
  V3<T> y;
  y[0] = a[0] * x[0] + a[3] * x[1] + a[6] * x[2];
  y[1] = a[1] * x[0] + a[4] * x[1] + a[7] * x[2];
  y[2] = a[2] * x[0] + a[5] * x[1] + a[8] * x[2];
  return y;
}
template <typename T> GF_HD M3<T> skew(const V3<T>& v) {
  M3<T> a;
  a[0] = T(0);  a[1] = -v[2]; a[2] = v[1];
  a[3] = v[2];  a[4] = T(0);  a[5] = -v[0];
  a[6] = -v[1]; a[7] = v[0];  a[8] = T(0);
  return a;
}
template <typename T> GF_HD T dot(const V3<T>& a, const V3<T>& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
template <typename T> GF_HD V3<T> cross(const V3<T>& a, const V3<T>& b) {
  V3<T> c;
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
  return c;
}
template <typename T, typename S> GF_HD M3<T> cvt(const M3<S>& a) {
  M3<T> r;
#pragma unroll
  for (int i = 0; i < 9; ++i) r[i] = T(a[i]);
  return r;
}
template <typename T, typename S> GF_HD V3<T> cvt(const V3<S>& a) {
  V3<T> r;
#pragma unroll
  for (int i = 0; i < 3; ++i) r[i] = T(a[i]);
  return r;
}

// Rodrigues tensor Q = I + g (A + A^2 / 2), g = 4 / (4 + |a|^2)
template <typename T> GF_HD M3<T> rodrigues(const V3<T>& a) {
  T n2 = dot(a, a);
  T g = T(4) / (T(4) + n2);
  M3<T> A = skew(a), A2 = mul(A, A), Q;
#pragma unroll
  for (int i = 0; i < 9; ++i) Q[i] = g * (A[i] + T(0.5) * A2[i]);
  Q[0] += T(1); Q[4] += T(1); Q[8] += T(1);
  return Q;
}

// Rodrigues composition 4/(4 - a2.a1) (a2 + a1 + a2 x a1 / 2)
template <typename T> GF_HD V3<T> rodrigues_compose(const V3<T>& a2, const V3<T>& a1) {
  V3<T> c = cross(a2, a1), r;
  T f = T(4) / (T(4) - dot(a2, a1));
#pragma unroll
  for (int i = 0; i < 3; ++i) r[i] = f * (a2[i] + a1[i] + T(0.5) * c[i]);
  return r;
}

// V(x, t) = (h8 t - h4 x*t) x^T + h2 skew(t)
template <typename T> GF_HD M3<T> opV(const V3<T>& x, const V3<T>& t, T h) {
  T h2 = T(0.5) * h, h4 = T(-0.25) * h * h, h8 = T(-0.5) * h * h;
  V3<T> xt = cross(x, t);
  M3<T> V;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    T a = h8 * t[i] - h4 * xt[i];
#pragma unroll
    for (int j = 0; j < 3; ++j) V[i * 3 + j] = a * x[j];
  }
  V[1] += -h2 * t[2]; V[2] += h2 * t[1];
  V[3] += h2 * t[2];  V[5] += -h2 * t[0];
  V[6] += -h2 * t[1]; V[7] += h2 * t[0];
  return V;
}

// d_V(x, dx, t) = (x.dx)(h9 t - h6 x*t) x^T + (h8 t - h4 x*t) dx^T
//                 - h4 (dx*t) x^T + h4 (x.dx) skew(t)
template <typename T> GF_HD M3<T> opdV(const V3<T>& x, const V3<T>& dx, const V3<T>& t, T h) {
  T h4 = T(-0.25) * h * h, h6 = T(0.25) * h * h * h, h8 = T(-0.5) * h * h, h9 = T(0.5) * h * h * h;
  V3<T> xt = cross(x, t), dxt = cross(dx, t);
  T xdx = dot(x, dx);
  M3<T> W;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    T a = xdx * (h9 * t[i] - h6 * xt[i]) - h4 * dxt[i];
    T b = h8 * t[i] - h4 * xt[i];
#pragma unroll
    for (int j = 0; j < 3; ++j) W[i * 3 + j] = a * x[j] + b * dx[j];
  }
  T s = h4 * xdx;
  W[1] += -s * t[2]; W[2] += s * t[1];
  W[3] += s * t[2];  W[5] += -s * t[0];
  W[6] += -s * t[1]; W[7] += s * t[0];
  return W;
}

}  // namespace gf
