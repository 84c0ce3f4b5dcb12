/*
 * ark_tsdf.h - header-only C++ front end with the reference's class name and
 * method signatures, forwarding to the C ABI in vhsdf.h.
 *
 * A caller written against ark::GpuTsdfGenerator (include/tsdf.cuh:548-683 of
 * E-BAO/Voxel-Hashing-SDF), such as PointCloudGenerator::Reproject
 * (src/PointCloudGenerator.cpp:93-129), compiles unchanged against this
 * header and links against libvhsdf.so.
 *
 * Differences a caller can observe:
 *   - blocks are 8^3 voxels and the volume stays resident on the GPU;
 *   - processFrame allocates the blocks of every pixel's truncation band
 *     (the reference walks subsampled rays) and averages sdf with the old
 *     weight (the reference uses the new one, src/tsdf.cu:739-742);
 *   - render() draws nothing: OpenGL is not available (it sets last_status);
 *   - errors never exit the process: every method records a vh_status in
 *     last_status() and processFrame returns it instead of aborting;
 *   - getHashMap() holds the merged vertices of the full-volume mesh (the
 *     reference's insert_vertex works on a copy of the bucket,
 *     src/tsdf.cu:1935, and leaves its map empty).
 */
#ifndef ARK_TSDF_H
#define ARK_TSDF_H

#include <cmath>
#include <cstring>
#include <list>
#include <string>
#include <utility>
#include <vector>

#include "vhsdf.h"

namespace ark {

/* include/tsdf.cuh:65-77: position and colour of one mesh vertex. */
struct Vertex {
  float x, y, z;
  unsigned char r, g, b;
};

/* include/tsdf.cuh:111-113 */
struct Face {
  int vIdx[3];
};

/* Host stand-ins for CUDA's float3 / int3 members of MarchingCubeParam. */
struct Float3 {
  float x, y, z;
};
struct Int3 {
  int x, y, z;
};

/* include/tsdf.cuh:220-534: the volume and camera settings and the
 * marching-cubes tables (the engine's own, equal to the reference's). */
struct MarchingCubeParam {
  Float3 vox_origin;  // the reference's dense grid; unused by the hash path
  float vox_size;
  float trunc_margin;
  Int3 vox_dim;
  int total_vox;
  float max_depth;
  float min_depth;
  float block_size;  // 8 voxels
  int im_width;
  int im_height;
  float fx, fy, cx, cy;
  int idxMap[8][3];
  int edgeTable[256];
  int triTable[256][16];
};

class GpuTsdfGenerator {
 public:
  /* include/tsdf.cuh:606-607, defaults src/tsdf.cu:1249-1252.  origin and
   * vox_dim describe the reference's unused dense grid and are ignored. */
  GpuTsdfGenerator(int width, int height, float fx, float fy, float cx, float cy,
                   float max_depth, float origin_x = -1.5f, float origin_y = -1.5f,
                   float origin_z = 0.5f, float vox_size = 0.006f, float trunc_m = 0.03f,
                   int vox_dim_x = 500, int vox_dim_y = 500, int vox_dim_z = 500) {
    mc_ = MarchingCubeParam{};
    mc_.vox_origin = Float3{origin_x, origin_y, origin_z};
    mc_.vox_dim = Int3{vox_dim_x, vox_dim_y, vox_dim_z};
    mc_.total_vox = vox_dim_x * vox_dim_y * vox_dim_z;
    vh_params_default(&params_);
    params_.width = width;
    params_.height = height;
    params_.fx = fx;
    params_.fy = fy;
    params_.cx = cx;
    params_.cy = cy;
    params_.max_depth = max_depth;
    params_.voxel_size = vox_size;
    params_.trunc = trunc_m;
    status_ = vh_create(&params_, &handle_);
    mc_.vox_size = vox_size;
    mc_.trunc_margin = trunc_m;
    mc_.max_depth = max_depth;
    mc_.min_depth = params_.min_depth;
    mc_.block_size = 8.0f * vox_size;
    mc_.im_width = width;
    mc_.im_height = height;
    mc_.fx = fx;
    mc_.fy = fy;
    mc_.cx = cx;
    mc_.cy = cy;
    vh_mc_tables(&mc_.idxMap[0][0], mc_.edgeTable, &mc_.triTable[0][0]);
  }

  ~GpuTsdfGenerator() { Shutdown(); }
  GpuTsdfGenerator(const GpuTsdfGenerator &) = delete;
  GpuTsdfGenerator &operator=(const GpuTsdfGenerator &) = delete;

  /* include/tsdf.cuh:610: depth H*W float metres, rgb H*W*3 (RGB order),
   * c2w row-major 4x4 camera-to-world, all host memory. */
  vh_status processFrame(float *depth, unsigned char *rgb, float *c2w) {
    if (!handle_) return status_ = VH_ERR_INVALID_ARG;
    status_ = vh_process_frame(handle_, depth, VH_DEPTH_F32_M, rgb, c2w, VH_MEM_HOST, nullptr);
    mesh_valid_ = map_valid_ = false;
    return status_;
  }

  /* include/tsdf.cuh:628: full-volume mesh as ASCII PLY. */
  void SavePLY(std::string filename) {
    status_ = handle_ ? vh_save_ply(handle_, filename.c_str(), 0) : VH_ERR_INVALID_ARG;
  }

  /* include/tsdf.cuh:619: needs OpenGL, which this engine does not use. */
  void render() { status_ = handle_ ? vh_render(handle_) : VH_ERR_INVALID_ARG; }

  /* include/tsdf.cuh:622 */
  void Shutdown() {
    if (handle_) vh_destroy(handle_);
    handle_ = nullptr;
  }

  /* include/tsdf.cuh:631-634: vertices (metres) and faces of the full-volume
   * mesh, vertices merged by exact position like tsdf2mesh. */
  std::vector<Vertex> *getVertices() {
    build_mesh();
    return &vertices_;
  }
  std::vector<Face> *getFaces() {
    build_mesh();
    return &faces_;
  }

  /* include/tsdf.cuh:637: the vertex hash of the mesh export - buckets of
   * (vertex, index) keyed by the vertex's voxel cell. */
  std::vector<std::list<std::pair<Vertex, int>>> *getHashMap() {
    build_mesh();
    if (!map_valid_) {
      const size_t nb = vertices_.empty() ? 1 : vertices_.size();
      map_.assign(nb, std::list<std::pair<Vertex, int>>());
      const float inv = 1.0f / params_.voxel_size;
      for (size_t i = 0; i < vertices_.size(); ++i) {
        const Vertex &v = vertices_[i];
        const long long cx = (long long)std::floor(v.x * inv), cy = (long long)std::floor(v.y * inv),
                        cz = (long long)std::floor(v.z * inv);
        const unsigned long long key =
            (unsigned long long)(cx * 73856093LL ^ cy * 19349669LL ^ cz * 83492791LL);
        map_[key % nb].push_back(std::make_pair(v, (int)i));
      }
      map_valid_ = true;
    }
    return &map_;
  }

  /* include/tsdf.cuh:640 */
  MarchingCubeParam *getMarchingCubeParam() { return &mc_; }

  vh_status last_status() const { return status_; }
  vh_handle *handle() { return handle_; }

 private:
  void build_mesh() {
    if (mesh_valid_ || !handle_) return;
    vertices_.clear();
    faces_.clear();
    int64_t nv = 0, nf = 0;
    status_ = vh_mesh_indexed(handle_, nullptr, nullptr, 0, nullptr, 0, &nv, &nf);
    if (status_ != VH_OK) return;
    std::vector<float> xyz((size_t)nv * 3);
    std::vector<unsigned char> rgb((size_t)nv * 3);
    std::vector<int> idx((size_t)nf * 3);
    status_ = vh_mesh_indexed(handle_, xyz.data(), rgb.data(), nv, idx.data(), nf, &nv, &nf);
    if (status_ != VH_OK) return;
    vertices_.resize((size_t)nv);
    for (int64_t i = 0; i < nv; ++i)
      vertices_[i] = Vertex{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], rgb[3 * i], rgb[3 * i + 1],
                            rgb[3 * i + 2]};
    faces_.resize((size_t)nf);
    for (int64_t t = 0; t < nf; ++t)
      for (int j = 0; j < 3; ++j) faces_[t].vIdx[j] = idx[3 * t + j];
    mesh_valid_ = true;
  }

  vh_params params_{};
  vh_handle *handle_ = nullptr;
  vh_status status_ = VH_OK;
  bool mesh_valid_ = false;
  bool map_valid_ = false;
  std::vector<Vertex> vertices_;
  std::vector<Face> faces_;
  std::vector<std::list<std::pair<Vertex, int>>> map_;
  MarchingCubeParam mc_{};
};

}  // namespace ark

#endif /* ARK_TSDF_H */
