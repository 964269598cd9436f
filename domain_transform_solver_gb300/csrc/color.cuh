// Bit-exact colour-space conversion of an RGBA8 guide.
//
// The reference converts in double and truncates to unsigned char
// (src/color_space.cuh:11-40):
//   Y  = R*0.299 + 0.587*G + 0.114*B
//   Cb = 128 - R*0.168736 - 0.331264*G + 0.5*B
//   Cr = 128 + R*0.5 - 0.418688*G - 0.081312*B
// Every exact value is a rational N/1000 (Y) or N/10^6 (Cb, Cr) with an
// integer N, and the double evaluation is within ~1e-13 of it.  So wherever
// N is not a multiple of the denominator, the truncated result is exactly
// floor(N/den), computed here in integer arithmetic.  Where N is a multiple
// (the exact value is an integer k, e.g. every grey pixel), the double result
// can land on either side of k, so those pixels evaluate the double
// expression itself, in the order nvcc compiles the reference source
// (multiply-add pairs contracted to fma).  Which of the two possible orders
// of Y applies is pinned on the GPU by tests/test_gpu_color_pin.py.
#pragma once

#include <stdint.h>

namespace dtsgb {

// Evaluation order of Y = R*0.299 + 0.587*G + 0.114*B:
//   1: fma(0.114,B, fma(R,0.299, 0.587*G))
//   2: fma(0.114,B, fma(0.587,G, R*0.299))
#ifndef DTSGB_Y_ORDER
#define DTSGB_Y_ORDER 1
#endif

__host__ __device__ inline double dmul_rn(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
__host__ __device__ inline double dfma_rn(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return __builtin_fma(a, b, c);
#endif
}

__host__ __device__ inline uint8_t luma_exact(int r, int g, int b) {
  const int n = 299 * r + 587 * g + 114 * b;
  const int q = n / 1000;
  if (n != q * 1000) return (uint8_t)q;
  const double R = r, G = g, B = b;
#if DTSGB_Y_ORDER == 1
  const double v = dfma_rn(0.114, B, dfma_rn(R, 0.299, dmul_rn(0.587, G)));
#else
  const double v = dfma_rn(0.114, B, dfma_rn(0.587, G, dmul_rn(R, 0.299)));
#endif
  return (uint8_t)(int)v;
}

__host__ __device__ inline uint8_t cb_exact(int r, int g, int b) {
  const int n = 128000000 - 168736 * r - 331264 * g + 500000 * b;
  const int q = n / 1000000;
  if (n != q * 1000000) return (uint8_t)q;
  const double R = r, G = g, B = b;
  const double v = dfma_rn(0.5, B, dfma_rn(-0.331264, G, dfma_rn(-R, 0.168736, 128.0)));
  return (uint8_t)(int)v;
}

__host__ __device__ inline uint8_t cr_exact(int r, int g, int b) {
  const int n = 128000000 + 500000 * r - 418688 * g - 81312 * b;
  const int q = n / 1000000;
  if (n != q * 1000000) return (uint8_t)q;
  const double R = r, G = g, B = b;
  const double v = dfma_rn(-0.081312, B, dfma_rn(-0.418688, G, dfma_rn(R, 0.5, 128.0)));
  return (uint8_t)(int)v;
}

// color_space: 0 RGB (unchanged), 1 YCbCr, 2 YYY.  Alpha is kept.
__host__ __device__ inline uchar4 convert_pixel(uchar4 p, int color_space) {
  if (color_space == 1) {
    return make_uchar4(luma_exact(p.x, p.y, p.z), cb_exact(p.x, p.y, p.z),
                       cr_exact(p.x, p.y, p.z), p.w);
  }
  if (color_space == 2) {
    const uint8_t y = luma_exact(p.x, p.y, p.z);
    return make_uchar4(y, y, y, p.w);
  }
  return p;
}

}  // namespace dtsgb
