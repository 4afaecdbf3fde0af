// Double-float numbers for the Davidson subspace of the mixed-precision
// solver: x = hi + lo stored as a float2 (8 bytes, like a double), about 48
// significant bits.  The FP64 pipe of this GPU retires far fewer operations
// per byte than HBM delivers, so vector kernels that spend one double FMA per
// double loaded are bound by it; in double-float form the same kernels spend
// about a dozen FP32 operations per element and stay bound by memory.
//
// Building blocks are the error-free transformations TwoSum (Knuth) and
// TwoProduct via FMA, and the compensated dot product Dot2 of Ogita, Rump and
// Oishi (SIAM J. Sci. Comput. 26, 2005): a sum of products computed as if in
// twice the working precision.  Every operation goes through the _rn
// intrinsics, which the compiler neither contracts into FMAs nor reorders.
#pragma once
#include <cuda_runtime.h>

namespace qdkgb {
namespace df {

// s + e = a + b exactly
__device__ __forceinline__ float2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return make_float2(s, e);
}
// the same when |a| >= |b| (or a == 0): the normalised pair
__device__ __forceinline__ float2 quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}

// Dot2 accumulator: the running sum is s.x + s.y, s.x carrying the TwoSum
// chain of the leading products and s.y the collected rounding errors and
// low-order products (not normalised until `value`)
__device__ __forceinline__ void mac(float2& s, float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  const float2 t = two_sum(s.x, p);
  s.x = t.x;
  s.y = __fadd_rn(s.y, __fadd_rn(t.y, e));
}
__device__ __forceinline__ float2 normalise(float2 s) { return two_sum(s.x, s.y); }
__device__ __forceinline__ double to_double(float2 s) { return (double)s.x + (double)s.y; }
// nearest double-float of a double
__device__ __forceinline__ float2 split(double x) {
  const float h = __double2float_rn(x);
  return make_float2(h, __double2float_rn(x - (double)h));
}
// a - b
__device__ __forceinline__ float2 sub(float2 a, float2 b) {
  const float2 t = two_sum(a.x, -b.x);
  return quick_two_sum(t.x, __fadd_rn(t.y, __fsub_rn(a.y, b.y)));
}
// a + b
__device__ __forceinline__ float2 add(float2 a, float2 b) {
  const float2 t = two_sum(a.x, b.x);
  return quick_two_sum(t.x, __fadd_rn(t.y, __fadd_rn(a.y, b.y)));
}
// a * b
__device__ __forceinline__ float2 mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  return quick_two_sum(p, e);
}

}  // namespace df
}  // namespace qdkgb
