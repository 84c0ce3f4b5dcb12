// vh_mesh.cpp - PLY export and volume snapshots.
//
// write_ply follows GpuTsdfGenerator::tsdf2mesh (src/tsdf.cu:1760-1888):
// vertices are merged when their (x, y, z) are exactly equal (the reference
// keys an unordered_map on the three floats, src/tsdf.cu:1777,1810-1821), the
// first occurrence keeps its colour, positions are scaled by the voxel size
// with no origin offset (src/tsdf.cu:1815-1817), and the ASCII layout is the
// reference's header and "x y z r g b" / "3 i j k" lines (src/tsdf.cu:1870-1885).
// Triangles are sorted first so the file does not depend on GPU scheduling.

#include "vh_mesh.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <unordered_map>

namespace vh {

namespace {

struct PosKey {
  uint32_t x, y, z;
  bool operator==(const PosKey &o) const { return x == o.x && y == o.y && z == o.z; }
};
struct PosHash {
  size_t operator()(const PosKey &k) const {
    uint64_t h = k.x * 0x9E3779B97F4A7C15ull;
    h ^= (k.y + 0x632BE59BD9B4E019ull) * 0xBF58476D1CE4E5B9ull;
    h ^= (k.z + 0x94D049BB133111EBull) * 0xD6E8FEB86659FD93ull;
    return (size_t)(h ^ (h >> 29));
  }
};

uint32_t bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

// +0.0 and -0.0 compare equal as floats; merge them like the reference does.
uint32_t canon(float f) { return f == 0.0f ? 0u : bits(f); }

}  // namespace

bool write_ply(const char *path, const float *tris, int64_t n, float voxel_size, bool binary) {
  std::vector<int64_t> order((size_t)n);
  for (int64_t i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
    const float *ta = tris + 12 * a, *tb = tris + 12 * b;
    for (int k = 0; k < 12; ++k) {
      if ((k & 3) == 3) continue;
      if (ta[k] < tb[k]) return true;
      if (ta[k] > tb[k]) return false;
    }
    for (int k = 3; k < 12; k += 4) {
      if (bits(ta[k]) != bits(tb[k])) return bits(ta[k]) < bits(tb[k]);
    }
    return false;
  });
  std::unordered_map<PosKey, int32_t, PosHash> index;
  index.reserve((size_t)n * 2);
  std::vector<float> vx;
  std::vector<uint8_t> vc;
  std::vector<int32_t> faces((size_t)n * 3);
  for (int64_t t = 0; t < n; ++t) {
    const float *tri = tris + 12 * order[t];
    for (int j = 0; j < 3; ++j) {
      const float *v = tri + 4 * j;
      PosKey k{canon(v[0]), canon(v[1]), canon(v[2])};
      auto it = index.find(k);
      int32_t id;
      if (it == index.end()) {
        id = (int32_t)(vx.size() / 3);
        index.emplace(k, id);
        vx.push_back(v[0] * voxel_size);
        vx.push_back(v[1] * voxel_size);
        vx.push_back(v[2] * voxel_size);
        uint32_t c = bits(v[3]);
        vc.push_back((uint8_t)(c & 0xFF));
        vc.push_back((uint8_t)((c >> 8) & 0xFF));
        vc.push_back((uint8_t)((c >> 16) & 0xFF));
      } else {
        id = it->second;
      }
      faces[3 * t + j] = id;
    }
  }
  const size_t nv = vx.size() / 3;
  std::ofstream f(path, binary ? std::ios::binary : std::ios::out);
  if (!f) return false;
  f << "ply\nformat " << (binary ? "binary_little_endian" : "ascii") << " 1.0\n";
  f << "comment stanford bunny\nelement vertex " << nv << "\n";
  f << "property float x\nproperty float y\nproperty float z\nproperty uchar red\n"
       "property uchar green\nproperty uchar blue\n";
  f << "element face " << n << "\nproperty list uchar int vertex_index\nend_header\n";
  if (binary) {
    for (size_t i = 0; i < nv; ++i) {
      f.write(reinterpret_cast<const char *>(&vx[3 * i]), 12);
      f.write(reinterpret_cast<const char *>(&vc[3 * i]), 3);
    }
    for (int64_t t = 0; t < n; ++t) {
      const uint8_t three = 3;
      f.write(reinterpret_cast<const char *>(&three), 1);
      f.write(reinterpret_cast<const char *>(&faces[3 * t]), 12);
    }
  } else {
    for (size_t i = 0; i < nv; ++i)
      f << vx[3 * i] << " " << vx[3 * i + 1] << " " << vx[3 * i + 2] << " " << (int)vc[3 * i] << " "
        << (int)vc[3 * i + 1] << " " << (int)vc[3 * i + 2] << "\n";
    for (int64_t t = 0; t < n; ++t)
      f << "3 " << faces[3 * t] << " " << faces[3 * t + 1] << " " << faces[3 * t + 2] << "\n";
  }
  return (bool)f;
}

namespace {
const char kMagic[8] = {'V', 'H', 'S', 'D', 'F', 'S', 'N', 'P'};
}

bool write_snapshot(const char *path, float voxel, float trunc, const int32_t *xyz,
                    const float *sdf, const float *w, const uint8_t *rgb, int64_t n) {
  std::ofstream f(path, std::ios::binary);
  if (!f) return false;
  const uint32_t version = 1, edge = 8;
  f.write(kMagic, 8);
  f.write(reinterpret_cast<const char *>(&version), 4);
  f.write(reinterpret_cast<const char *>(&edge), 4);
  f.write(reinterpret_cast<const char *>(&voxel), 4);
  f.write(reinterpret_cast<const char *>(&trunc), 4);
  f.write(reinterpret_cast<const char *>(&n), 8);
  f.write(reinterpret_cast<const char *>(xyz), (std::streamsize)(12 * n));
  f.write(reinterpret_cast<const char *>(sdf), (std::streamsize)(2048 * n));
  f.write(reinterpret_cast<const char *>(w), (std::streamsize)(2048 * n));
  f.write(reinterpret_cast<const char *>(rgb), (std::streamsize)(1536 * n));
  return (bool)f;
}

bool read_snapshot(const char *path, float *voxel, float *trunc, std::vector<int32_t> &xyz,
                   std::vector<float> &sdf, std::vector<float> &w, std::vector<uint8_t> &rgb) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  char magic[8];
  uint32_t version = 0, edge = 0;
  int64_t n = 0;
  f.read(magic, 8);
  f.read(reinterpret_cast<char *>(&version), 4);
  f.read(reinterpret_cast<char *>(&edge), 4);
  f.read(reinterpret_cast<char *>(voxel), 4);
  f.read(reinterpret_cast<char *>(trunc), 4);
  f.read(reinterpret_cast<char *>(&n), 8);
  if (!f || std::memcmp(magic, kMagic, 8) != 0 || version != 1 || edge != 8 || n < 0 ||
      n > (1ll << 28))
    return false;
  xyz.resize(3 * (size_t)n);
  sdf.resize(512 * (size_t)n);
  w.resize(512 * (size_t)n);
  rgb.resize(1536 * (size_t)n);
  f.read(reinterpret_cast<char *>(xyz.data()), (std::streamsize)(12 * n));
  f.read(reinterpret_cast<char *>(sdf.data()), (std::streamsize)(2048 * n));
  f.read(reinterpret_cast<char *>(w.data()), (std::streamsize)(2048 * n));
  f.read(reinterpret_cast<char *>(rgb.data()), (std::streamsize)(1536 * n));
  return (bool)f;
}

}  // namespace vh
