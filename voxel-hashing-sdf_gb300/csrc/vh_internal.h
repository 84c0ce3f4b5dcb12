// vh_internal.h - handle accessors for entry points implemented outside
// vh_api.cpp (host code only).
#pragma once
#include "../../include/vhsdf.h"
#include "vh_common.cuh"

#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

namespace vh {
// NVTX range over one entry point (named after it): visible in Nsight
// Systems timelines, a no-op without a profiler attached.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};
#define VH_NVTX(name) ::vh::NvtxRange vh_nvtx_range__(name)

VolumeView handle_view(const vh_handle *h);
cudaStream_t handle_stream(const vh_handle *h);
int handle_device(const vh_handle *h);
// Records `msg` as the handle's last error and returns `s`.
vh_status handle_fail(vh_handle *h, vh_status s, const char *msg);
// Passes an error message to the log callback (vh_set_log_callback), if any.
void log_error(const std::string &msg);
// Waits for the handle's stream and reports sticky device errors.
vh_status handle_sync(vh_handle *h);
CamParams handle_cam(const vh_handle *h);
int handle_sm_count(const vh_handle *h);
// Copies one depth image into the handle's staging buffer (stream-ordered)
// and returns its device address.
vh_status handle_stage_depth(vh_handle *h, const void *depth, int fmt, int mem, const void **dev);
// Device workspace owned by the handle, grown on demand, freed with it.
vh_status handle_workspace(vh_handle *h, size_t bytes, void **ptr);
// Frame buffers and launch shapes of a handle, for the batched frame step.
struct FrameBuffers {
  void *depth;
  uint8_t *rgb;
  uint2 *pix;
  float4 *tris;
  int64_t tri_cap;
  int integrate_per_sm;
  int mc_per_sm;
  int mc_variant;
};
FrameBuffers handle_frame_buffers(const vh_handle *h);
const vh_params &handle_params(const vh_handle *h);
// Bookkeeping after a batched frame step ran on the handle's volume.
void handle_note_frame(vh_handle *h);
int64_t handle_frames(const vh_handle *h);
// Reports sticky device error bits as a status (and records the message).
vh_status handle_status_of_bits(vh_handle *h, uint32_t bits);
// Vertices merged by exact position and numbered by first occurrence over
// the sorted triangles (vh_meshindex.cu); positions scaled to metres.
vh_status index_mesh(vh_handle *h, const float4 *tris, int64_t n, float voxel,
                     std::vector<float> &vert, std::vector<uint8_t> &col,
                     std::vector<int32_t> &faces);
// Host store of streamed-out blocks (vh_stream.cu), released with the handle.
struct StreamStore;
StreamStore *&handle_stream_store(vh_handle *h);
void stream_store_free(StreamStore *s);
// Waits for pending asynchronous evictions and moves them into the store.
vh_status stream_store_settle(vh_handle *h);
// The device state as of the last synchronising call.
const DevState &handle_state(const vh_handle *h);
// The frame list's neighbour table no longer matches the hash table.
void handle_invalidate_nb(vh_handle *h);
// Pose-refinement state (buffers, cached graph) created on first use by
// vh_adjoint.cu and released with the handle.
struct RefineCtx;
RefineCtx *&handle_refine(vh_handle *h);
void refine_ctx_free(RefineCtx *ctx);
}  // namespace vh

namespace vh {
// Makes `device` the calling thread's current GPU for the scope's lifetime
// and restores the caller's device after it, so that an entry point works on
// its handle's GPU whatever device the caller has current, and leaves that
// setting as it found it.  device < 0: no change (a null handle).
class DeviceScope {
 public:
  explicit DeviceScope(int device) {
    if (device < 0) return;
    ok_ = cudaGetDevice(&prev_) == cudaSuccess;
    if (ok_ && prev_ != device) ok_ = switched_ = cudaSetDevice(device) == cudaSuccess;
  }
  ~DeviceScope() {
    if (switched_) cudaSetDevice(prev_);
  }
  DeviceScope(const DeviceScope &) = delete;
  DeviceScope &operator=(const DeviceScope &) = delete;
  bool ok() const { return ok_; }

 private:
  int prev_ = 0;
  bool ok_ = true, switched_ = false;
};
}  // namespace vh

// First statement of an entry point that works on a handle's GPU (the
// handle may be null; the argument checks that follow report that).
#define VH_HANDLE_DEVICE(h)                                                   \
  vh::DeviceScope vh_device_scope_((h) ? vh::handle_device(h) : -1);          \
  if (!vh_device_scope_.ok())                                                 \
  return vh::handle_fail((h), VH_ERR_CUDA, "cannot make the handle's GPU current")
