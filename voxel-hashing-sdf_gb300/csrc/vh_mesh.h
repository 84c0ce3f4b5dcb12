// vh_mesh.h - host-side mesh and snapshot files.
#pragma once
#include <stdint.h>
#include <vector>

namespace vh {

// Writes a triangle soup (12 floats per triangle: 3 x {x, y, z, rgb bits},
// voxel units) as PLY with vertices merged by exact position.
bool write_ply(const char *path, const float *tris, int64_t n, float voxel_size, bool binary);

// Binary volume snapshot: header, keys, sdf, weight, rgb.
bool write_snapshot(const char *path, float voxel, float trunc, const int32_t *xyz,
                    const float *sdf, const float *w, const uint8_t *rgb, int64_t n);
bool read_snapshot(const char *path, float *voxel, float *trunc, std::vector<int32_t> &xyz,
                   std::vector<float> &sdf, std::vector<float> &w, std::vector<uint8_t> &rgb);

}  // namespace vh
