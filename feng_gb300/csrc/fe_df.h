// Double-float arithmetic for the device residuals (shared by the triangle
// and tetrahedron kernels).
#pragma once

#include <cuda_runtime.h>

namespace feng {

// Double-float arithmetic: a value is hi + lo, two floats (~44-bit
// significand) computed on the FP32 pipes.  Knuth's error-free sum
// (TwoSum, The Art of Computer Programming vol. 2, 4.2.2), Dekker's product
// ("A floating-point technique for extending the available precision",
// Numer. Math. 18, 1971) with the error of hi * hi from a fused
// multiply-add, and the pair addition of Dekker (the same paper) as in
// Bailey's double-double library, whose error is relative to the operands (u^2 |x| + u^2 |y|,
// u = 2^-24): enough for element sums, which do not cancel to the size of
// a converged residual (that cancellation happens in the FP64 sums across
// elements).  Every operation is an explicit round-to-nearest intrinsic so
// that no multiply and add are contracted into one.
struct dfl {
  float hi, lo;
};

__device__ __forceinline__ dfl df_from(double x)
{
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ double df_to(dfl a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ dfl df_zero() { return {0.f, 0.f}; }
__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.hi, -a.lo}; }
// s + e with |a| >= |b|
__device__ __forceinline__ dfl df_fast2(float a, float b)
{
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dfl df_add(dfl x, dfl y)
{
  const float s = __fadd_rn(x.hi, y.hi);
  const float v = __fsub_rn(s, x.hi);
  float e = __fadd_rn(__fsub_rn(x.hi, __fsub_rn(s, v)), __fsub_rn(y.hi, v));
  e = __fadd_rn(e, __fadd_rn(x.lo, y.lo));
  return df_fast2(s, e);
}
__device__ __forceinline__ dfl df_sub(dfl x, dfl y) { return df_add(x, df_neg(y)); }
__device__ __forceinline__ dfl df_mul(dfl x, dfl y)
{
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  return df_fast2(p, e);
}
__device__ __forceinline__ dfl df_fma(dfl a, dfl b, dfl c) { return df_add(df_mul(a, b), c); }


}  // namespace feng
