// vh_mesh.cpp - PLY export and volume snapshots.
//
// write_ply writes the mesh that vh_meshindex.cu indexed on the GPU the way
// GpuTsdfGenerator::tsdf2mesh does (src/tsdf.cu:1760-1888: exact-position
// merge, first occurrence keeps its colour, positions scaled by the voxel
// size with no origin offset) in the reference's layout: its header and
// "x y z r g b" / "3 i j k" lines (src/tsdf.cu:1870-1885), or the same
// elements as binary little endian.

#include "vh_mesh.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>

namespace vh {

bool write_ply(const char *path, const std::vector<float> &vx, const std::vector<uint8_t> &vc,
               const std::vector<int32_t> &faces, bool binary) {
  const int64_t n = (int64_t)(faces.size() / 3);
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
