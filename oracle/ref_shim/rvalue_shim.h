// Force-included ahead of every reference translation unit built into the
// oracle.  The reference is written for MSVC, which binds temporaries to
// non-const references; g++ does not.  These forwarding overloads take the
// temporary by rvalue reference and hand it on as an lvalue, so the
// reference's own arithmetic runs unchanged.
#pragma once
#include <cstring>
#include <cctype>
#include "omp.h"
#include <cstdlib>
#include <typeinfo>
#include <cmath>
#include <algorithm>
#include "Matrix.h"
using std::abs;
#define RV2(OP)                                                                   \
  inline Matrix OP(Matrix&& a, Matrix& b) { return OP(static_cast<Matrix&>(a), b); } \
  inline Matrix OP(Matrix& a, Matrix&& b) { return OP(a, static_cast<Matrix&>(b)); } \
  inline Matrix OP(Matrix&& a, Matrix&& b) {                                     \
    return OP(static_cast<Matrix&>(a), static_cast<Matrix&>(b));                 \
  }
RV2(operator+)
RV2(operator-)
RV2(operator*)
RV2(cross)
RV2(dyadic)
RV2(Dot)
#undef RV2
inline Matrix operator*(double s, Matrix&& a) { return s * static_cast<Matrix&>(a); }
inline Matrix operator*(Matrix&& a, double s) { return static_cast<Matrix&>(a) * s; }
inline double dot(Matrix&& a, Matrix& b) { return dot(static_cast<Matrix&>(a), b); }
inline double dot(Matrix& a, Matrix&& b) { return dot(a, static_cast<Matrix&>(b)); }
inline double dot(Matrix&& a, Matrix&& b) {
  return dot(static_cast<Matrix&>(a), static_cast<Matrix&>(b));
}
#define RV1(RET, F) inline RET F(Matrix&& a) { return F(static_cast<Matrix&>(a)); }
RV1(Matrix, skew)
RV1(Matrix, axial)
RV1(Matrix, transp)
RV1(double, norm)
RV1(double, norm4)
RV1(Matrix, invert2x2)
RV1(Matrix, invert3x3)
RV1(Matrix, invert4x4)
RV1(Matrix, invert5x5)
RV1(Matrix, invert6x6)
RV1(Matrix, invert)
#undef RV1
