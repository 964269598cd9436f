// 32-bit fixed-point window sums for the DTS iteration and its adjoint.
//
// Values convert to integers at a power-of-two scale 2^F chosen from the
// largest magnitude m among them and the largest number n of values one
// window adds up: n * m * 2^F < 2^31, so every window sum fits an int32.
// Prefix sums are kept in wrapping (mod 2^32) unsigned arithmetic: a
// difference of two prefixes is then the exact window sum of the converted
// values even when the prefixes themselves wrap.  The only roundings are the
// conversion of each value (at most 2^-F / 2 <= n * m * 2^-32) and of the
// sum back to float: for windows of up to 17 pixels that is below 1/8 ulp
// of m per value, more accurate than a float running sum.  Conversions and
// adds are single native 32-bit instructions.
#pragma once

#include <cuda_runtime.h>

namespace dtsgb {

// ceil(log2(n)) for n >= 1.
__host__ __device__ __forceinline__ int ceil_log2(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return l;
}

// F for values of magnitude <= m, windows of up to 2^lg_n of them (clamped
// so that 2^F and 2^-F are normal floats).
__device__ __forceinline__ int fx_shift(float m, int lg_n) {
  const int e = (int)((__float_as_uint(m) >> 23) & 0xff) - 127;  // m < 2^(e+1)
  return max(min(30 - lg_n - e, 126), -126);
}

// 2^k as a float, k in [-126, 127].
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }

// Value -> fixed point (|v * sF| < 2^31 by the choice of F).
__device__ __forceinline__ unsigned fx_from(float v, float sF) {
  return (unsigned)__float2int_rn(v * sF);
}

// Window sum (difference of two wrapping prefixes) -> float, times `scale`.
__device__ __forceinline__ float fx_window(unsigned hi, unsigned lo, float scale) {
  return __int2float_rn((int)(hi - lo)) * scale;
}

// Inclusive prefix sum over the 32 lanes of a warp (all lanes active).
__device__ __forceinline__ unsigned warp_incl_scan(unsigned v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned n = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += n;
  }
  return v;
}

// Bits of |v|: they order like the magnitude, and every infinity or NaN
// lies at or above kNonFiniteBits, so an integer max over them both finds the
// fixed-point scale and flags a non-finite value (a float max would skip a
// NaN, whose conversion to fixed point is then undefined).
__device__ __forceinline__ unsigned mag_bits(float v) {
  return __float_as_uint(v) & 0x7fffffffu;
}
constexpr unsigned kNonFiniteBits = 0x7f800000u;

// Largest of a non-negative float over the warp (all lanes active).
__device__ __forceinline__ float warp_max_nonneg(float m) {
  return __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(m)));
}

}  // namespace dtsgb
