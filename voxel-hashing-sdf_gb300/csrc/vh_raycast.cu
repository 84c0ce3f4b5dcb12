// vh_raycast.cu - headless ray casting of the TSDF into depth, normal and
// colour images.
//
// The reference draws its mesh with OpenGL (GpuTsdfGenerator::render,
// src/tsdf.cu:1710-1758); what a tracker consumes instead is a ray-cast
// depth / normal map of the fused surface (the natural input of ICP-style
// tracking and of the pose refinement in vh_adjoint.cu).  One thread per
// pixel marches its ray through the trilinear TSDF:
//   * the ray of pixel (u, v) is parametrised by camera-frame depth t (its
//     camera direction ((u - cx) / fx, (v - cy) / fy, 1) has z = 1), world
//     point c2w * (t * dir);
//   * where the sample is unknown (a corner block missing or a corner
//     weight below max(1, mc_min_weight)) the ray advances by T (it cannot
//     step over a +-T band); where it is known and positive it advances by
//     0.8 of the sampled distance T * phi, at least half a voxel;
//   * the first known sign change + -> - is the surface: the depth is
//     interpolated linearly between the two samples; negative space entered
//     without a positive sample before it (a surface seen from behind, or
//     voxels that other views saw behind an occluder - projective fusion
//     leaves such patches in free space) is crossed in half-voxel steps;
//   * the normal is the normalised TSDF gradient at the hit (world frame,
//     towards free space), the colour that of the nearest voxel.

#include <cmath>
#include <cstring>

#include "vh_device.cuh"
#include "vh_internal.h"

namespace vh {
namespace {

__device__ __forceinline__ uint32_t voxel_rgb(const VolumeView &V, float x, float y, float z,
                                              float inv_voxel) {
  const int ix = (int)floorf(x * inv_voxel + 0.5f), iy = (int)floorf(y * inv_voxel + 0.5f),
            iz = (int)floorf(z * inv_voxel + 0.5f);
  const int bx = ix >> 3, by = iy >> 3, bz = iz >> 3;
  if (!key_in_range(bx, by, bz)) return 0u;
  const uint32_t b = block_of(V, pack_key(bx, by, bz));
  if (b == kNoBlock) return 0u;
  const int li = (ix & 7) + 8 * (iy & 7) + 64 * (iz & 7);
  return __ldg(reinterpret_cast<const uint32_t *>(V.pool + (size_t)b * kBlockWords + 2 * kB3) + li);
}

__global__ void __launch_bounds__(128) k_raycast(VolumeView V, CamParams C, const float *__restrict__ pose,
                                                 float *__restrict__ depth,
                                                 float *__restrict__ normal,
                                                 uint8_t *__restrict__ rgb) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= C.width * C.height) return;
  float P[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) P[k] = __ldg(pose + k);
  const int u = idx % C.width, v = idx / C.width;
  const float dx = ((float)u - C.cx) / C.fx, dy = ((float)v - C.cy) / C.fy;
  const float wx = P[0] * dx + P[1] * dy + P[2];
  const float wy = P[4] * dx + P[5] * dy + P[6];
  const float wz = P[8] * dx + P[9] * dy + P[10];
  const float len = sqrtf(dx * dx + dy * dy + 1.0f);  // world distance per unit of t
  const float inv_voxel = 1.0f / C.voxel;
  const float min_w = C.mc_min_weight < 1.0f ? 1.0f : C.mc_min_weight;
  const float far_step = C.trunc / len, min_step = 0.5f * C.voxel / len;
  const int max_steps = (int)((C.max_depth - C.min_depth) / min_step) + 2;
  float t = C.min_depth, prev_t = 0.0f, prev_phi = 0.0f, t_hit = 0.0f;
  bool prev_ok = false, hit = false;
  Sample last{};
  for (int it = 0; it < max_steps && t <= C.max_depth; ++it) {
    const float x = P[3] + t * wx, y = P[7] + t * wy, z = P[11] + t * wz;
    const Sample s = sample_tsdf(V, inv_voxel, min_w, x, y, z);
    if (!s.ok) {
      prev_ok = false;
      t += far_step;
      continue;
    }
    if (s.phi <= 0.0f) {
      if (prev_ok) {  // + -> - crossing
        t_hit = prev_t + (t - prev_t) * (prev_phi / (prev_phi - s.phi));
        hit = true;
        last = s;
        break;
      }
      // negative space not entered from positive space (a surface seen from
      // behind, or a voxel other views saw behind an occluder): cross it
      t += min_step;
      continue;
    }
    prev_ok = true;
    prev_phi = s.phi;
    prev_t = t;
    last = s;
    t += fmaxf(0.8f * s.phi * C.trunc / len, min_step);
  }
  float n[3] = {0.0f, 0.0f, 0.0f};
  uint32_t c = 0u;
  if (hit) {
    const float x = P[3] + t_hit * wx, y = P[7] + t_hit * wy, z = P[11] + t_hit * wz;
    const Sample s = sample_tsdf(V, inv_voxel, min_w, x, y, z);
    const Sample &g = s.ok ? s : last;
    const float gn = sqrtf(g.gx * g.gx + g.gy * g.gy + g.gz * g.gz);
    if (gn > 0.0f) {
      n[0] = g.gx / gn;
      n[1] = g.gy / gn;
      n[2] = g.gz / gn;
    }
    c = voxel_rgb(V, x, y, z, inv_voxel);
  }
  depth[idx] = hit ? t_hit : 0.0f;
  if (normal) {
    normal[3 * (size_t)idx] = n[0];
    normal[3 * (size_t)idx + 1] = n[1];
    normal[3 * (size_t)idx + 2] = n[2];
  }
  if (rgb) {
    rgb[3 * (size_t)idx] = (uint8_t)(c & 0xFFu);
    rgb[3 * (size_t)idx + 1] = (uint8_t)((c >> 8) & 0xFFu);
    rgb[3 * (size_t)idx + 2] = (uint8_t)((c >> 16) & 0xFFu);
  }
}

}  // namespace
}  // namespace vh

using namespace vh;

extern "C" vh_status vh_raycast(vh_handle *h, const float *c2w, float *depth, float *normal,
                                uint8_t *rgb, int32_t mem) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_raycast");
  if (!h || !c2w || !depth) return VH_ERR_INVALID_ARG;
  if (mem != VH_MEM_HOST && mem != VH_MEM_DEVICE) return VH_ERR_INVALID_ARG;
  for (int i = 0; i < 16; ++i)
    if (!std::isfinite(c2w[i])) return VH_ERR_NOT_FINITE;
  const CamParams C = handle_cam(h);
  const cudaStream_t st = handle_stream(h);
  const size_t npx = (size_t)C.width * C.height;
  // workspace: pose (16 floats) | depth | normals | rgb (host outputs only)
  const size_t bytes = 64 + (mem == VH_MEM_HOST ? npx * (4 + 12 + 3) + 64 : 0);
  void *p = nullptr;
  vh_status s = handle_workspace(h, bytes, &p);
  if (s != VH_OK) return s;
  float *dpose = static_cast<float *>(p);
  float *dd = depth, *dn = normal;
  uint8_t *dc = rgb;
  if (mem == VH_MEM_HOST) {
    dd = dpose + 16;
    dn = normal ? dd + npx : nullptr;
    dc = rgb ? reinterpret_cast<uint8_t *>(dd + 4 * npx) : nullptr;
  }
  if (cudaMemcpyAsync(dpose, c2w, 16 * sizeof(float), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return handle_fail(h, VH_ERR_CUDA, "pose upload failed");
  k_raycast<<<(unsigned)((npx + 127) / 128), 128, 0, st>>>(handle_view(h), C, dpose, dd, dn, dc);
  if (cudaGetLastError() != cudaSuccess) return handle_fail(h, VH_ERR_CUDA, "raycast launch failed");
  if (mem == VH_MEM_HOST) {
    bool ok = cudaMemcpyAsync(depth, dd, sizeof(float) * npx, cudaMemcpyDeviceToHost, st) == cudaSuccess;
    if (normal)
      ok = ok && cudaMemcpyAsync(normal, dn, sizeof(float) * 3 * npx, cudaMemcpyDeviceToHost, st) ==
                     cudaSuccess;
    if (rgb) ok = ok && cudaMemcpyAsync(rgb, dc, 3 * npx, cudaMemcpyDeviceToHost, st) == cudaSuccess;
    if (!ok) return handle_fail(h, VH_ERR_CUDA, "raycast download failed");
  }
  return handle_sync(h);
}
