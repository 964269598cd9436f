// Host-side helpers for the benchmark drivers' image formats (no GPU work).
// The reference decodes its PNG inputs with OpenCV; the drivers of this
// library decode them in Python and undo the PNG row filters here.
#include <cstdint>
#include <cstdlib>

#include "../../include/dtsgb.h"

extern "C" {

DTSGB_API int dtsgb_png_unfilter(const unsigned char* raw, int height, int stride,
                                 int bpp, unsigned char* out) {
  if (!raw || !out || height < 0 || stride < 0 || bpp < 1 || bpp > 8)
    return DTSGB_ERR_INVALID_ARGUMENT;
  const unsigned char* prev = nullptr;
  for (int y = 0; y < height; ++y) {
    const unsigned char ftype = raw[(size_t)y * (stride + 1)];
    const unsigned char* f = raw + (size_t)y * (stride + 1) + 1;
    unsigned char* cur = out + (size_t)y * stride;
    for (int i = 0; i < stride; ++i) {
      const int a = i >= bpp ? cur[i - bpp] : 0;
      const int b = prev ? prev[i] : 0;
      const int c = (prev && i >= bpp) ? prev[i - bpp] : 0;
      int pred;
      switch (ftype) {
        case 0: pred = 0; break;
        case 1: pred = a; break;
        case 2: pred = b; break;
        case 3: pred = (a + b) >> 1; break;
        case 4: {
          const int p = a + b - c;
          const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
          pred = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
          break;
        }
        default: return DTSGB_ERR_INVALID_ARGUMENT;
      }
      cur[i] = (unsigned char)((f[i] + pred) & 0xff);
    }
    prev = cur;
  }
  return DTSGB_OK;
}

}  // extern "C"
