// dfloat.cuh -- double-float arithmetic: a value is the unevaluated sum
// hi + lo of two float32 numbers with |lo| <= ulp(hi) / 2, about 48
// significant bits.  GB300 runs float64 at 1/64 of the float32 rate, so the
// re-contraction of rows whose float32 margin is inside the rounding bound
// runs on pairs of float32 instead.
//
// The algorithms are the classical error-free transformations: Knuth's
// two-sum, Dekker's fast two-sum (|a| >= |b|), and the product's exact
// error from one fused multiply-add (Ogita, Rump and Oishi, "Accurate sum
// and dot product", SIAM J. Sci. Comput. 26, 2005).  All operations use the
// round-to-nearest intrinsics so that the compiler cannot contract a
// multiply and an add of the transformations into one fma.
//
// Error bound (all operands non-negative, as every tensor entry of the
// decoder is): fma(a, b, c) below returns c + a*b times (1 + d) with
// |d| <= 15 * 2^-48 < 2^-44 -- the dropped a.lo*b.lo term (2^-48), the two
// roundings inside the product's low part (5 * 2^-48) and the two roundings
// of the low-order sum (9 * 2^-48); the fast two-sums are exact.  The host
// bounds the re-contraction with 2^-43 per operation, in place of float32's
// 2^-24, over the same operation count; as for float32, values below the
// normal range are outside the bound.
#pragma once

#include <cuda_runtime.h>

namespace tqec {

struct dfloat {
  float hi, lo;
  dfloat() = default;
  __host__ __device__ constexpr dfloat(int v) : hi(float(v)), lo(0.0f) {}
  __host__ __device__ constexpr dfloat(float v) : hi(v), lo(0.0f) {}
  __host__ __device__ constexpr dfloat(float h, float l) : hi(h), lo(l) {}
  // the leading part: the float32 bits of the value (maxima, normalisers)
  __host__ __device__ explicit operator float() const { return hi; }
  __host__ __device__ explicit operator double() const { return double(hi) + double(lo); }
};

// hi + lo = a + b exactly (|a| >= |b|).
__device__ __forceinline__ dfloat fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return dfloat(s, __fsub_rn(b, __fsub_rn(s, a)));
}

// hi + lo = a + b exactly.
__device__ __forceinline__ dfloat two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return dfloat(s, e);
}

__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
  const dfloat s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = __fmaf_rn(a.hi, b.hi, -p);  // p + e = a.hi * b.hi exactly
  const float t = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
  return fast_two_sum(p, t);
}

// c + a * b (the float and double overloads stay visible next to this one)
using ::fma;
__device__ __forceinline__ dfloat fma(dfloat a, dfloat b, dfloat c) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = __fmaf_rn(a.hi, b.hi, -p);
  const float t = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
  const dfloat s = two_sum(c.hi, p);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(c.lo, t)));
}

__device__ __forceinline__ bool operator>(dfloat a, dfloat b) {
  return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo);
}

// (the built-in overloads stay visible next to this one)
using ::__shfl_xor_sync;
__device__ __forceinline__ dfloat __shfl_xor_sync(unsigned mask, dfloat v, int lane_mask) {
  return dfloat(::__shfl_xor_sync(mask, v.hi, lane_mask), ::__shfl_xor_sync(mask, v.lo, lane_mask));
}

// x times a power of two (the per-tensor normalisers): exact.
template <typename T>
__device__ __forceinline__ T scale(T x, T s) {
  return x * s;
}
template <>
__device__ __forceinline__ dfloat scale<dfloat>(dfloat x, dfloat s) {
  return dfloat(__fmul_rn(x.hi, s.hi), __fmul_rn(x.lo, s.hi));
}

}  // namespace tqec
