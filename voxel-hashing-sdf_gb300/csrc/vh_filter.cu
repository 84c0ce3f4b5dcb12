// vh_filter.cu - optional depth pre-filter (VH_FLAG_DEPTH_FILTER).
//
// The reference only scales its depth (SaveFrame::frameLoad,
// src/SaveFrame.cpp:179-180).  With the flag set, every staged frame is
// smoothed before allocation by an edge-preserving bilateral filter over a
// 5x5 window: weights exp(-r^2 / (2 s^2)) exp(-(d - d0)^2 / (2 sr^2)) with
// s = 2 pixels and sr = 5 mm + 3 * 1.5e-3 d0^2 (three standard deviations of
// structured-light depth noise), neighbours that are invalid or farther than
// 3 sr from the centre depth left out.  Invalid centre pixels stay invalid.
// The result is float metres, read by allocation and integration.

#include "vh_common.cuh"

namespace vh {
namespace {

template <typename DepthT>
__device__ __forceinline__ float depth_at(const DepthT *d, int i, float scale);
template <>
__device__ __forceinline__ float depth_at<uint16_t>(const uint16_t *d, int i, float scale) {
  return (float)__ldg(d + i) * scale;
}
template <>
__device__ __forceinline__ float depth_at<float>(const float *d, int i, float) {
  return __ldg(d + i);
}

template <typename DepthT>
__global__ void __launch_bounds__(256) k_depth_filter(CamParams C, const DepthT *__restrict__ depth,
                                                      const FrameIn *__restrict__ fin,
                                                      float *__restrict__ out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= C.width * C.height) return;
  const DepthT *in = depth ? depth : static_cast<const DepthT *>(fin->depth);
  const int u = idx % C.width, v = idx / C.width;
  const float d0 = depth_at<DepthT>(in, idx, C.depth_scale);
  if (!(d0 > C.min_depth && d0 <= C.max_depth)) {
    out[idx] = 0.0f;
    return;
  }
  const float sr = 0.005f + 4.5e-3f * d0 * d0;
  const float inv_2sr2 = 1.0f / (2.0f * sr * sr), inv_2ss2 = 1.0f / 8.0f;  // s = 2 px
  float sum = 0.0f, wsum = 0.0f;
#pragma unroll
  for (int dy = -2; dy <= 2; ++dy)
#pragma unroll
    for (int dx = -2; dx <= 2; ++dx) {
      const int x = u + dx, y = v + dy;
      if (x < 0 || x >= C.width || y < 0 || y >= C.height) continue;
      const float d = depth_at<DepthT>(in, y * C.width + x, C.depth_scale);
      if (!(d > C.min_depth && d <= C.max_depth) || fabsf(d - d0) >= 3.0f * sr) continue;
      const float w = expf(-(float)(dx * dx + dy * dy) * inv_2ss2 - (d - d0) * (d - d0) * inv_2sr2);
      sum += w * d;
      wsum += w;
    }
  out[idx] = sum / wsum;  // the centre contributes weight 1
}

}  // namespace

void launch_depth_filter(const CamParams &C, const void *depth, const FrameIn *fin, int fmt,
                         float *out, cudaStream_t s) {
  const unsigned grid = (unsigned)(((size_t)C.width * C.height + 255) / 256);
  if (fmt == 0)
    k_depth_filter<uint16_t><<<grid, 256, 0, s>>>(C, static_cast<const uint16_t *>(depth), fin, out);
  else
    k_depth_filter<float><<<grid, 256, 0, s>>>(C, static_cast<const float *>(depth), fin, out);
}

}  // namespace vh
