// vh_mesh.h - host-side mesh and snapshot files.
#pragma once
#include <stdint.h>
#include <vector>

namespace vh {

// Writes an indexed mesh (vertices in metres, 3 colour bytes each, 3 vertex
// numbers per face) as PLY in the reference's layout.
bool write_ply(const char *path, const std::vector<float> &vert, const std::vector<uint8_t> &col,
               const std::vector<int32_t> &faces, bool binary);

// Binary volume snapshot: header, keys, sdf, weight, rgb.
bool write_snapshot(const char *path, float voxel, float trunc, const int32_t *xyz,
                    const float *sdf, const float *w, const uint8_t *rgb, int64_t n);
bool read_snapshot(const char *path, float *voxel, float *trunc, std::vector<int32_t> &xyz,
                   std::vector<float> &sdf, std::vector<float> &w, std::vector<uint8_t> &rgb);

}  // namespace vh
