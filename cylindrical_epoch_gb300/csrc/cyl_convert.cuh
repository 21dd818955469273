// cyl_convert.cuh -- FP64 <-> FP32 conversions done with integer operations.
//
// On GB300 the FP64 pipe is narrow and the F2F conversion instructions run
// on it; the mixed-precision kernels convert the FP64 currents and their
// FP32 partial sums with the integer bit manipulations below instead.
// Normal numbers only: values below the FP32 normal range become zero,
// values above it infinity (currents and fields stay many decades inside).
#pragma once

#include <cuda_runtime.h>

namespace cyl {

// FP64 -> FP32, rounding the 29 dropped mantissa bits half up.
__device__ __forceinline__ float d2f_bits(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
  if (e <= 0) return __uint_as_float(sign);
  if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
  unsigned f = sign | ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  f += (lo >> 28) & 1u;  // a carry into the exponent is the correct result
  return __uint_as_float(f);
}

// FP32 -> FP64, exact for normal numbers.
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  if (e == 0u) return __longlong_as_double((long long)sign);
  const unsigned long long de = (e == 255u) ? 2047ull : (unsigned long long)(e + 896u);
  return __longlong_as_double((long long)(sign | (de << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
}

}  // namespace cyl
