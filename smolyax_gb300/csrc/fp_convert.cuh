// Device helpers of the FP32 evaluators: FP64 -> FP32 conversion on the
// integer pipes and compensated FP32 summation.
#pragma once

#include <cuda_runtime.h>

namespace smx {

// FP64 -> FP32 with integer operations (truncation of the mantissa; |v| below
// 2^-126 is raised to a value in [2^-126, 2^-125) of the same sign; |v| of
// 2^128 (1 + 2^-20) and above, infinities and NaNs give NaN, so that a
// non-finite coordinate makes the point's value NaN as in the FP64 path).
// Keeps the conversions off the FP64 pipe.  Layout facts used: IEEE-754
// binary64 = sign, 11-bit exponent (bias 1023), 52-bit fraction; binary32 =
// sign, 8-bit exponent (bias 127), 23-bit fraction.  The magnitude's high word
// is clamped to [exponent of 2^-126, exponent 255 + one fraction bit]; its top
// 9 exponent bits and 23 fraction bits are then shifted into place together,
// adding 2^30 re-biases the exponent modulo 2^32 (the clamp keeps it in 1..255,
// so bit 31 stays clear), and the sign is merged back: six integer operations.
__device__ __forceinline__ float f64_to_f32(double v) {
  const unsigned hi = static_cast<unsigned>(__double2hiint(v));
  const unsigned lo = static_cast<unsigned>(__double2loint(v));
  const unsigned mag = min(max(hi & 0x7fffffffu, 0x38100000u), 0x47f00001u);
  const unsigned t = __funnelshift_l(lo, mag, 3) + 0x40000000u;
  return __uint_as_float(t | (hi & 0x80000000u));
}

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  const float yv = v - c;
  const float t = s + yv;
  c = (t - s) - yv;
  s = t;
}

}  // namespace smx
