// Sanitizer fuzzing of the frame decoders (test side only): each seed file
// (PNG or JPEG; the first argument is the number of mutations per seed) is
// damaged by seeded bit flips, byte overwrites, insertions, truncations and
// planted markers, then decoded: a size query, then the pixels when the
// size is modest; a decoded image is then resized to a random size
// (vh_resize_colour).  Built with -fsanitize=address,undefined by
// tests/test_decoder_fuzz.py; an out-of-bounds access or undefined
// behaviour ends the run with a report and a non-zero exit.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <random>
#include <vector>

#include "vhsdf.h"

static void mutate(std::vector<uint8_t> &d, std::mt19937_64 &rng) {
  const int n = 1 + (int)(rng() % 8);
  for (int m = 0; m < n && d.size() >= 4; ++m) {
    const int kind = (int)(rng() % 5);
    const size_t at = rng() % d.size();
    if (kind == 0) {
      d[at] ^= (uint8_t)(1u << (rng() % 8));
    } else if (kind == 1) {
      d[at] = (uint8_t)rng();
    } else if (kind == 2 && at > 2) {
      d.resize(at);
    } else if (kind == 3) {
      d.insert(d.begin() + (long)at, (uint8_t)rng());
    } else if (kind == 4 && at + 4 < d.size()) {
      d[at] = 0xFF;
      d[at + 1] = (uint8_t)(0xC0 + rng() % 64);
    }
  }
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  const int iters = atoi(argv[1]);
  std::mt19937_64 rng(12345);
  long decoded = 0, rejected = 0;
  for (int f = 2; f < argc; ++f) {
    FILE *fp = fopen(argv[f], "rb");
    if (!fp) return 2;
    std::vector<uint8_t> seed;
    for (int c; (c = fgetc(fp)) != EOF;) seed.push_back((uint8_t)c);
    fclose(fp);
    if (seed.size() < 4) return 2;
    const bool png = seed[0] == 0x89;
    for (int it = 0; it < iters; ++it) {
      std::vector<uint8_t> m = seed;
      mutate(m, rng);
      // an allocation of exactly the file's size, so that a read one byte
      // past the end is outside the heap block the sanitizer tracks
      const int64_t n = (int64_t)m.size();
      std::unique_ptr<uint8_t[]> file(new uint8_t[m.size()]);
      std::memcpy(file.get(), m.data(), m.size());
      const uint8_t *d = file.get();
      int32_t w = 0, h = 0;
      vh_status s = png ? vh_decode_colour_png(d, n, nullptr, 0, &w, &h)
                        : vh_decode_colour_jpeg(d, n, nullptr, 0, &w, &h);
      if (s == VH_OK && (int64_t)w * h <= (1 << 22)) {
        std::vector<uint8_t> rgb((size_t)w * (size_t)h * 3);
        const int64_t cap = (int64_t)rgb.size();
        s = png ? vh_decode_colour_png(d, n, rgb.data(), cap, &w, &h)
                : vh_decode_colour_jpeg(d, n, rgb.data(), cap, &w, &h);
        if (png) {
          std::vector<uint16_t> depth((size_t)w * (size_t)h);
          vh_decode_depth_png(d, n, depth.data(), (int64_t)depth.size(), &w, &h);
        }
        if (s == VH_OK) {
          const int32_t dw = 1 + (int32_t)(rng() % 70), dh = 1 + (int32_t)(rng() % 70);
          std::unique_ptr<uint8_t[]> out(new uint8_t[(size_t)dw * (size_t)dh * 3]);
          if (vh_resize_colour(rgb.data(), w, h, out.get(), dw, dh) != VH_OK) return 3;
        }
      }
      (s == VH_OK ? decoded : rejected)++;
    }
  }
  printf("decoded %ld, rejected %ld\n", decoded, rejected);
  return 0;
}
