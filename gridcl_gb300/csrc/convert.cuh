// f32 <-> f64 conversions in integer operations, shared by the split kernels and their self-test.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace tlg {

// f32 <-> f64 conversions in integer operations. On this part the conversion instructions run
// on the FP64 pipe (about 2 lanes per clock per SM) and queue behind its throttle; the split
// kernels convert every node coordinate of every cell. Both functions return exactly what the
// conversion instructions return: IEEE round-to-nearest-even, by exponent rebias and the
// discarded mantissa bits; operands outside the normal range take the instruction.

// f64 -> f32, round to nearest even.
__device__ __forceinline__ float d2f_rn(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7FFu;
  // Biased f64 exponents 897 .. 1150 are the f32 normal exponents 1 .. 254.
  if (e - 897u >= 254u) return __double2float_rn(x);
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  unsigned r = ((unsigned)(b >> 63) << 31) | ((e - 896u) << 23) | (unsigned)(m >> 29);
  const unsigned rest = (unsigned)(m & 0x1FFFFFFFull);  // the 29 discarded bits; half = 2^28
  // Round up above half, and at half to even; a carry out of the mantissa raises the exponent
  // (to infinity past the largest finite f32, as the instruction does).
  r += (unsigned)(rest > 0x10000000u) | ((unsigned)(rest == 0x10000000u) & r & 1u);
  return __uint_as_float(r);
}

// f32 -> f64 (exact).
__device__ __forceinline__ double f2d_exact(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xFFu;
  const uint64_t sign = (uint64_t)(b >> 31) << 63;
  if ((b << 1) == 0u) return __longlong_as_double((long long)sign);
  if (e == 0u || e == 0xFFu) return (double)f;
  return __longlong_as_double(
      (long long)(sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(b & 0x7FFFFFu) << 29)));
}

}  // namespace tlg
