// 16-bit operands of the tensor-core trailing updates: rounding to FP16 or
// BF16 and back, and the power-of-two FP16 scale of an operand from its
// largest magnitude.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace mgb {

template <int BF16>
__device__ __forceinline__ uint16_t to16(float v) {
  if (BF16) return __bfloat16_as_ushort(__float2bfloat16_rn(v));
  return __half_as_ushort(__float2half_rn(v));
}

template <int BF16>
__device__ __forceinline__ float from16(uint16_t h) {
  if (BF16) return __bfloat162float(__ushort_as_bfloat16(h));
  return __half2float(__ushort_as_half(h));
}

// s = 2^(14 - e) for max|x| = f 2^e (f in [0.5, 1)): the scaled maximum sits
// in [2^13, 2^14), far from FP16's overflow and, for the entries near it,
// from its subnormal range.  1 for 0, Inf or NaN (NaN then propagates).
// The exponent is capped at 2^100 so that the scale and its inverse stay
// finite for maxima near FLT_MIN.
__device__ __forceinline__ float fp16_scale(unsigned amax_bits) {
  const float a = __uint_as_float(amax_bits);
  if (!(a > 0.f) || isinf(a)) return 1.f;
  int e;
  frexpf(a, &e);  // a = f * 2^e, f in [0.5, 1)
  return ldexpf(1.f, 14 - e < 100 ? 14 - e : 100);
}

}  // namespace mgb
