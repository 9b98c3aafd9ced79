// Host helper of the command-line tool's image files: the PNG row filters (plain C++, built with
// the host compiler and linked into the same library as the CUDA translation units).
//
// The reference reads and writes its photographs with the image crate (image 0.25, png feature;
// image::open at src/image_pipeline.rs:1141, GrayImage/RgbImage::save at :1087-1133).  The tool's
// PNG codec lives in Python (fgrain_gb300/imageio.py: chunks, zlib, Adam7 passes, bit depths);
// the per-byte recurrences of the Average and Paeth filters are the one part that needs native
// code to be fast on large scans.  Nothing here touches the GPU.
#include <cstddef>
#include <cstdint>
#include <cstdlib>

#include "fgrain_cuda.h"

namespace {

// The Paeth predictor of the PNG specification (ISO/IEC 15948:2003 section 9.4).
inline uint8_t paeth(int a, int b, int c) {
  const int p = a + b - c;
  const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
  if (pa <= pb && pa <= pc) return static_cast<uint8_t>(a);
  if (pb <= pc) return static_cast<uint8_t>(b);
  return static_cast<uint8_t>(c);
}

}  // namespace

extern "C" fg_status fg_png_unfilter(uint8_t* rows, uint32_t h, uint32_t stride, uint32_t bpp) {
  if ((!rows && h) || bpp == 0 || bpp > 8) return FG_ERR_INVALID_ARG;
  const size_t pitch = static_cast<size_t>(stride) + 1;
  const uint8_t* prior = nullptr;  // the previous row's reconstructed bytes (none for the first row)
  for (uint32_t y = 0; y < h; ++y) {
    uint8_t* row = rows + y * pitch;
    const uint8_t type = row[0];
    uint8_t* x = row + 1;
    switch (type) {
      case 0:  // None
        break;
      case 1:  // Sub
        for (uint32_t i = bpp; i < stride; ++i) x[i] = static_cast<uint8_t>(x[i] + x[i - bpp]);
        break;
      case 2:  // Up
        if (prior)
          for (uint32_t i = 0; i < stride; ++i) x[i] = static_cast<uint8_t>(x[i] + prior[i]);
        break;
      case 3:  // Average
        for (uint32_t i = 0; i < stride; ++i) {
          const int a = i >= bpp ? x[i - bpp] : 0, b = prior ? prior[i] : 0;
          x[i] = static_cast<uint8_t>(x[i] + ((a + b) >> 1));
        }
        break;
      case 4:  // Paeth
        for (uint32_t i = 0; i < stride; ++i) {
          const int a = i >= bpp ? x[i - bpp] : 0, b = prior ? prior[i] : 0;
          const int c = (prior && i >= bpp) ? prior[i - bpp] : 0;
          x[i] = static_cast<uint8_t>(x[i] + paeth(a, b, c));
        }
        break;
      default:
        return FG_ERR_INVALID_ARG;
    }
    row[0] = 0;
    prior = x;
  }
  return FG_OK;
}
