// vh_frames.cpp - host-side preparation of colour frames (vh_resize_colour).
//
// The reference scales every colour frame to 640 x 480 with cv::resize's
// default bilinear interpolation before fusing it with the depth frame
// (src/SaveFrame.cpp:164-171); colour and depth then share one pixel grid,
// which is what the integration kernel indexes.  vh_resize_colour brings a
// colour image to the depth image's size by the same geometry: pixel centres
// at half-integer positions, source position (x + 0.5) * src_w / dst_w - 0.5,
// clamped to the first and last column (rows alike), and the four
// neighbours weighted bilinearly.  The weights are evaluated in double and
// rounded to the nearest level; OpenCV's 11-bit fixed-point weights can land
// one level away on some pixels.
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/vhsdf.h"

namespace {

// One axis of the bilinear map: destination index -> first source index and
// the weight of the second one (0 at the clamped borders).
struct Tap {
  int32_t i0, i1;
  double a;
};

std::vector<Tap> taps(int32_t src, int32_t dst) {
  std::vector<Tap> t((size_t)dst);
  const double scale = (double)src / (double)dst;
  for (int32_t d = 0; d < dst; ++d) {
    const double f = ((double)d + 0.5) * scale - 0.5;
    int32_t i = (int32_t)std::floor(f);
    double a = f - (double)i;
    if (i < 0) {
      i = 0;
      a = 0.0;
    }
    if (i >= src - 1) {
      i = src - 1;
      a = 0.0;
    }
    t[(size_t)d] = Tap{i, i + 1 < src ? i + 1 : i, a};
  }
  return t;
}

}  // namespace

extern "C" vh_status vh_resize_colour(const uint8_t *src, int32_t src_width, int32_t src_height,
                                      uint8_t *dst, int32_t dst_width, int32_t dst_height) {
  if (!src || !dst || src_width <= 0 || src_height <= 0 || dst_width <= 0 || dst_height <= 0 ||
      src_width > 32768 || src_height > 32768 || dst_width > 32768 || dst_height > 32768)
    return VH_ERR_INVALID_ARG;
  const std::vector<Tap> tx = taps(src_width, dst_width), ty = taps(src_height, dst_height);
  const size_t sstride = (size_t)src_width * 3;
  for (int32_t y = 0; y < dst_height; ++y) {
    const Tap &v = ty[(size_t)y];
    const uint8_t *r0 = src + (size_t)v.i0 * sstride, *r1 = src + (size_t)v.i1 * sstride;
    uint8_t *out = dst + (size_t)y * (size_t)dst_width * 3;
    for (int32_t x = 0; x < dst_width; ++x) {
      const Tap &u = tx[(size_t)x];
      const size_t c0 = (size_t)u.i0 * 3, c1 = (size_t)u.i1 * 3;
      for (int c = 0; c < 3; ++c) {
        const double top = (1.0 - u.a) * r0[c0 + c] + u.a * r0[c1 + c];
        const double bot = (1.0 - u.a) * r1[c0 + c] + u.a * r1[c1 + c];
        const double val = (1.0 - v.a) * top + v.a * bot;  // within [0, 255]
        out[(size_t)x * 3 + c] = (uint8_t)std::floor(val + 0.5);
      }
    }
  }
  return VH_OK;
}
