// FP32-pair ("double-float") numbers: a value is the unevaluated sum h + l
// of two floats with |l| <= ulp(h)/2, about 48 significant bits.  The
// operations are the error-free transformations of Dekker and Knuth (two-sum,
// and two-product through a fused multiply-add), so they run on the FP32
// pipe, which on this part has about 58 times the FP64 pipe's throughput.
// Rounding is explicit (__fadd_rn / __fmul_rn / __fmaf_rn) so that the
// compiler cannot contract the transformations.
//
// Used as the TK type of the Beam_1 tangent's rotation to the global frame
// and K_e expansion in the mixed-precision path: the tangent only steers the
// Newton iteration, while the Gauss-point operator, the internal force, the
// residual and the convergence checks stay FP64.
#pragma once
#include <cuda_runtime.h>

namespace gf {

struct f2 {
  float h, l;
  __host__ __device__ __forceinline__ f2() : h(0.f), l(0.f) {}
  __host__ __device__ __forceinline__ f2(float a, float b) : h(a), l(b) {}
  __device__ __forceinline__ f2(int x) : h((float)x), l(0.f) {}
  __device__ __forceinline__ f2(double x) {
    h = __double2float_rn(x);
    l = __double2float_rn(x - (double)h);
  }
  __device__ __forceinline__ explicit operator double() const { return (double)h + (double)l; }
};

__device__ __forceinline__ f2 f2_quick_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  return f2(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ f2 operator+(f2 a, f2 b) {
  float s = __fadd_rn(a.h, b.h);
  float bb = __fsub_rn(s, a.h);
  float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  return f2_quick_two_sum(s, e);
}
__device__ __forceinline__ f2 operator-(f2 a) { return f2(-a.h, -a.l); }
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return a + (-b); }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) {
  float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return f2_quick_two_sum(p, e);
}
__device__ __forceinline__ f2& operator+=(f2& a, f2 b) { return a = a + b; }
__device__ __forceinline__ f2& operator-=(f2& a, f2 b) { return a = a - b; }
__device__ __forceinline__ f2& operator*=(f2& a, f2 b) { return a = a * b; }

}  // namespace gf
