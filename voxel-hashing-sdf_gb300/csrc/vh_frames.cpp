// vh_frames.cpp - host-side frame preparation: colour resizing
// (vh_resize_colour) and whole frames read from the reference's frame
// folders (vh_load_frame).
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
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
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

// ---- frames in the reference's folder layout -----------------------------
//
// SaveFrame::frameLoad (src/SaveFrame.cpp:154-218) reads frame i as
// <root>/RGB/<i>.jpg (colour), <root>/depth/<i>.png (16-bit millimetres)
// and <root>/tcw/<i>.txt (16 numbers read with operator>> into floats, a
// row-major 4 x 4 camera-to-world pose, which it inverts and
// PointCloudGenerator::PushFrame inverts back, src/SaveFrame.cpp:206,
// src/PointCloudGenerator.cpp:140; Reproject then sets the last row to
// 0 0 0 1, src/PointCloudGenerator.cpp:118-125).

namespace {

bool read_file(const std::string &path, std::vector<uint8_t> &out) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  out.clear();
  uint8_t chunk[1 << 16];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) out.insert(out.end(), chunk, chunk + got);
  const bool ok = !std::ferror(f);
  std::fclose(f);
  return ok;
}

bool exists(const std::string &path) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fclose(f);
  return true;
}

// 16 numbers separated by white space, each read as a float the way
// operator>> reads one (strtof: the nearest float to the decimal)
vh_status parse_pose(const std::vector<uint8_t> &text, float *c2w) {
  std::string s(text.begin(), text.end());
  const char *p = s.c_str();
  for (int i = 0; i < 16; ++i) {
    char *end = nullptr;
    const float v = std::strtof(p, &end);
    if (end == p) return VH_ERR_INVALID_ARG;
    if (!std::isfinite(v)) return VH_ERR_NOT_FINITE;
    c2w[i] = v;
    p = end;
  }
  c2w[12] = c2w[13] = c2w[14] = 0.0f;
  c2w[15] = 1.0f;
  return VH_OK;
}

}  // namespace

extern "C" vh_status vh_load_frame(const char *root, int32_t frame_id, uint16_t *depth,
                                   int64_t depth_capacity, uint8_t *rgb, int64_t rgb_capacity,
                                   float *c2w, int32_t *width, int32_t *height) {
  if (!root || !width || !height || depth_capacity < 0 || rgb_capacity < 0 || frame_id < 0)
    return VH_ERR_INVALID_ARG;
  const std::string id = std::to_string(frame_id), base(root);
  const std::string depth_path = base + "/depth/" + id + ".png";
  const std::string pose_path = base + "/tcw/" + id + ".txt";
  std::string colour_path = base + "/RGB/" + id + ".jpg";
  if (!exists(colour_path)) colour_path = base + "/RGB/" + id + ".png";
  std::vector<uint8_t> file;
  if (!exists(colour_path) || !exists(pose_path) || !read_file(depth_path, file))
    return VH_ERR_IO;  // the frame is missing
  int32_t w = 0, h = 0;
  vh_status s = vh_decode_depth_png(file.data(), (int64_t)file.size(), nullptr, 0, &w, &h);
  if (s != VH_OK) return s;
  *width = w;
  *height = h;
  if (!depth) return VH_OK;  // size query
  const int64_t npx = (int64_t)w * (int64_t)h;
  if (depth_capacity < npx || !rgb || rgb_capacity < 3 * npx || !c2w) {
    return (!rgb || !c2w) ? VH_ERR_INVALID_ARG : VH_ERR_CAPACITY;
  }
  if ((s = vh_decode_depth_png(file.data(), (int64_t)file.size(), depth, depth_capacity, &w,
                               &h)) != VH_OK)
    return s;
  if (!read_file(colour_path, file)) return VH_ERR_IO;
  const bool png = file.size() >= 8 && file[0] == 0x89 && file[1] == 'P';
  const bool jpeg = file.size() >= 2 && file[0] == 0xFF && file[1] == 0xD8;
  if (!png && !jpeg) return VH_ERR_UNSUPPORTED;
  int32_t cw = 0, ch = 0;
  s = png ? vh_decode_colour_png(file.data(), (int64_t)file.size(), nullptr, 0, &cw, &ch)
          : vh_decode_colour_jpeg(file.data(), (int64_t)file.size(), nullptr, 0, &cw, &ch);
  if (s != VH_OK) return s;
  std::vector<uint8_t> colour((size_t)cw * (size_t)ch * 3);
  uint8_t *dst = (cw == w && ch == h) ? rgb : colour.data();
  const int64_t cap = 3 * (int64_t)cw * (int64_t)ch;
  s = png ? vh_decode_colour_png(file.data(), (int64_t)file.size(), dst, cap, &cw, &ch)
          : vh_decode_colour_jpeg(file.data(), (int64_t)file.size(), dst, cap, &cw, &ch);
  if (s != VH_OK) return s;
  if (dst != rgb && (s = vh_resize_colour(colour.data(), cw, ch, rgb, w, h)) != VH_OK) return s;
  if (!read_file(pose_path, file)) return VH_ERR_IO;
  return parse_pose(file, c2w);
}
