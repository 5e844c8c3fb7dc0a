// Device helpers of the FP32 evaluators: FP64 -> FP32 conversion on the
// integer pipes and compensated FP32 summation.
#pragma once

#include <cuda_runtime.h>

namespace smx {

// FP64 -> FP32 with integer operations (truncation of the mantissa; |v| below
// 2^-126 is raised to a value in [2^-126, 2^-125) of the same sign; |v| of
// 2^128 and above, infinities and NaNs give NaN, so that a non-finite
// coordinate makes the point's value NaN as in the FP64 path).  Keeps the
// conversions off the FP64 pipe.  Layout facts used: IEEE-754 binary64 =
// sign, 11-bit exponent (bias 1023), 52-bit fraction; binary32 = sign, 8-bit
// exponent (bias 127), 23-bit fraction.  The magnitude's high word is clamped
// below at the exponent of 2^-126; its top 9 exponent bits and 23 fraction
// bits are then shifted into place together, adding 2^30 re-biases the
// exponent modulo 2^32, and the sign is merged back.
__device__ __forceinline__ float f64_to_f32(double v) {
  const unsigned hi = static_cast<unsigned>(__double2hiint(v));
  const unsigned lo = static_cast<unsigned>(__double2loint(v));
  const unsigned a = hi & 0x7fffffffu;
  const unsigned mag = max(a, 0x38100000u);
  const unsigned t = a >= 0x47f00000u ? 0x7fc00000u : __funnelshift_l(lo, mag, 3) + 0x40000000u;
  return __uint_as_float((t & 0x7fffffffu) | (hi & 0x80000000u));
}

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  const float yv = v - c;
  const float t = s + yv;
  c = (t - s) - yv;
  s = t;
}

}  // namespace smx
