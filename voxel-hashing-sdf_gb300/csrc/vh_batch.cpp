// vh_batch.cpp - many independent scenes stepped together (include/vhsdf.h,
// vh_batch_*).
//
// Each scene is an ordinary handle (own hash table, pool, staging buffers).
// A batched step runs the per-frame stages of every scene that has a frame
// as one launch per stage: the kernels walk a flattened (scene, item) index
// (pixels for allocation, listed blocks for integration and marching cubes)
// and apply the single-scene bodies with that scene's volume and camera.
// Per step the host fills one pinned block - the scene descriptors, the
// poses and the active flags - and sends it with one copy; the stage
// launches replay as one CUDA graph whose arguments never change.
//
// The scenes are split into a few contiguous groups of about equal pixel
// count.  Each group has its own stream, which is also the stream of its
// scenes' handles, and runs its stage launches there as one CUDA graph per
// step: a scene depends only on its own earlier frames, so groups move on
// from step to step independently (no step-wide join), one group's
// latency-bound allocation overlapping another's issue-bound integration.
// The per-step descriptor blocks live in a ring on the device; a block is
// rewritten only after every group has finished the step that read it.
//
// With VH_FLAG_BATCH_FUSED the scenes form one group whose step is one
// persistent launch over all stages of all scenes (k_batch_step): one
// scene's latency-bound allocation overlaps another's issue-bound
// integration inside that launch instead of across group streams.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/vhsdf.h"
#include "vh_common.cuh"
#include "vh_internal.h"

using namespace vh;

namespace {
constexpr int kRing = 4;  // per-step upload blocks in flight
// Concurrent scene groups per step.  Measured on the 64-scene configuration
// (GB300): 1 group 29.9k, 2 31.0k, 4 32.2k, 8 33.1k, 16 33.6k frames/s; on
// 256 small scenes 133k .. 159k.  Each group's persistent kernels keep
// full-GPU grids (grids split by group count measured slower).
constexpr int kMaxGroups = 16;

// Scenes [s0, s0 + n) with their own work prefixes and stream.
struct BatchGroup {
  int s0 = 0, n = 0;
  uint32_t total_px = 0;
  uint32_t *d_px_start = nullptr;  // n + 1, relative to the group
  uint32_t *d_prefix = nullptr;    // n + 1 prefix words, then the MC block counter
  cudaStream_t stream = nullptr;
  cudaEvent_t done[kRing] = {};    // this group's step that read ring block k
  bool used[kRing] = {};
  cudaEvent_t last = nullptr;      // this group's latest work
  // step graphs per depth format, mesh flag and ring block
  cudaGraphExec_t graphs[2][2][kRing] = {};
};
}

struct vh_batch {
  int n = 0;
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;  // descriptor uploads and the state gather
  std::vector<vh_handle *> scenes;
  // per-step upload block: SceneDesc[n] | float pose[16 n] | uint8 active[n]
  size_t desc_bytes = 0, pose_bytes = 0, block_bytes = 0;
  unsigned char *d_block = nullptr;  // kRing blocks
  unsigned char *h_block = nullptr;  // pinned, kRing blocks
  cudaEvent_t ring_ev[kRing] = {};   // upload of ring block k done
  int ring_pos = 0;
  SceneDesc *d_static = nullptr;     // n: every scene's volume view (state gather)
  std::vector<BatchGroup> groups;
  cudaEvent_t joined = nullptr;      // the batch stream after a state gather
  DevState *d_states = nullptr;  // n
  DevState *h_states = nullptr;  // pinned, n
  int graph_shape[3] = {0, 0, -1};  // integrate grid, MC grid, MC variant the graphs hold
  bool fused = false;                // VH_FLAG_BATCH_FUSED: one persistent launch per step
  StepSched *d_sched = nullptr;      // fused: per-scene work hand-out (n)
  StepGlobal *d_glob = nullptr;      // fused: scenes left in the step
  int step_grid[2] = {0, 0};         // fused: persistent CTAs without / with meshes
  std::string last_error;

  unsigned char *block(int k) const { return d_block + block_bytes * (size_t)k; }
  SceneDesc *desc(int k) const { return reinterpret_cast<SceneDesc *>(block(k)); }
  const float *pose(int k, int i) const {
    return reinterpret_cast<const float *>(block(k) + desc_bytes) + 16 * (size_t)i;
  }
  const uint8_t *active(int k) const { return block(k) + desc_bytes + pose_bytes; }
};

namespace {

void drop_step_graphs(vh_batch *b) {
  for (BatchGroup &g : b->groups)
    for (auto &a : g.graphs)
      for (auto &m : a)
        for (auto &x : m)
          if (x) {
            cudaGraphExecDestroy(x);
            x = nullptr;
          }
}

void free_batch(vh_batch *b) {
  drop_step_graphs(b);
  for (BatchGroup &g : b->groups)
    if (g.stream) cudaStreamSynchronize(g.stream);
  for (vh_handle *h : b->scenes)
    if (h) vh_destroy(h);
  cudaFree(b->d_block);
  cudaFree(b->d_static);
  cudaFree(b->d_sched);
  cudaFree(b->d_glob);
  for (BatchGroup &g : b->groups) {
    cudaFree(g.d_px_start);
    cudaFree(g.d_prefix);
    for (auto &e : g.done)
      if (e) cudaEventDestroy(e);
    if (g.last) cudaEventDestroy(g.last);
    if (g.stream) cudaStreamDestroy(g.stream);
  }
  if (b->joined) cudaEventDestroy(b->joined);
  cudaFree(b->d_states);
  if (b->h_block) cudaFreeHost(b->h_block);
  if (b->h_states) cudaFreeHost(b->h_states);
  for (auto &e : b->ring_ev)
    if (e) cudaEventDestroy(e);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

// Launch shapes: the first scene's tuning, capped by the batched kernels'
// own occupancy.  {integrate grid, MC grid, MC variant}.
void batch_shape(const vh_batch *b, int out[3]) {
  const FrameBuffers f0 = handle_frame_buffers(b->scenes[0]);
  out[0] = b->sm_count * std::max(1, std::min(f0.integrate_per_sm, batch_integrate_ctas_per_sm()));
  out[1] = b->sm_count * std::max(1, std::min(f0.mc_per_sm, batch_mc_ctas_per_sm(f0.mc_variant)));
  out[2] = f0.mc_variant;
}

// One group's stages of one step, reading ring block k, on the group's
// stream (also inside a stream capture).
void enqueue_group_step(vh_batch *b, BatchGroup &g, int k, int fmt, bool with_mesh,
                        const int shape[3]) {
  const SceneDesc *d = b->desc(k) + g.s0;
  const uint8_t *act = b->active(k) + g.s0;
  cudaStream_t s = g.stream;
  if (b->fused) {
    launch_batch_step(d, act, g.n, b->d_sched, b->d_glob, fmt, with_mesh,
                      b->step_grid[with_mesh ? 1 : 0], s);
    return;
  }
  launch_batch_frame_begin(d, act, g.n, s);
  launch_batch_allocate(d, act, g.d_px_start, g.total_px, g.n, fmt, s);
  launch_batch_resolve(d, act, g.n, g.d_prefix, with_mesh, b->sm_count * 2, s);
  launch_batch_integrate(d, g.d_prefix, g.n, shape[0], s);
  if (with_mesh) launch_batch_mc(d, g.d_prefix, g.n, shape[1], shape[2], s);
}

vh_status fail(vh_batch *b, vh_status s, const std::string &msg) {
  b->last_error = msg;
  vh::log_error(msg);
  return s;
}

vh_status check_batch(vh_batch *b, vh_status *status, vh_stats *stats, bool clear);

}  // namespace

extern "C" {

vh_status vh_batch_create(const vh_params *params, int32_t n, vh_batch **out) {
  if (!out) return VH_ERR_INVALID_ARG;
  *out = nullptr;
  if (!params || n < 1 || n > VH_BATCH_MAX_SCENES) return VH_ERR_INVALID_ARG;
  for (int i = 0; i < n; ++i) {
    const vh_status s = vh_params_validate(params + i);
    if (s != VH_OK) return s;
    if (params[i].device != params[0].device) return VH_ERR_INVALID_ARG;
    if (params[i].flags & VH_FLAG_DEPTH_FILTER) return VH_ERR_UNSUPPORTED;  // not in batches
  }
  DeviceScope on_device(params[0].device);  // the caller's current device is restored
  if (!on_device.ok()) return VH_ERR_CUDA;
  vh_batch *b = new vh_batch();
  b->n = n;
  b->device = params[0].device;
  b->scenes.assign(n, nullptr);
  for (int i = 0; i < n; ++i) {
    const vh_status s = vh_create(params + i, &b->scenes[i]);
    if (s != VH_OK) {
      free_batch(b);
      return s;
    }
  }
  if (cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device) !=
          cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    free_batch(b);
    return VH_ERR_CUDA;
  }
  b->desc_bytes = sizeof(SceneDesc) * (size_t)n;
  b->pose_bytes = 16 * sizeof(float) * (size_t)n;
  b->block_bytes = (b->desc_bytes + b->pose_bytes + (size_t)n + 15) & ~(size_t)15;
  // pixels per scene, rounded to whole allocation CTAs
  std::vector<uint64_t> spx(n);
  uint64_t all_px = 0;
  for (int i = 0; i < n; ++i) {
    const uint64_t npx = (uint64_t)params[i].width * (uint64_t)params[i].height;
    spx[i] = (npx + kBatchPixelThreads - 1) / kBatchPixelThreads * kBatchPixelThreads;
    all_px += spx[i];
  }
  // contiguous groups of about equal pixel count, at least one scene each
  b->fused = (params[0].flags & VH_FLAG_BATCH_FUSED) != 0;
  const int ng = b->fused ? 1 : std::min(kMaxGroups, n);
  b->groups.resize(ng);
  for (int g = 0, i = 0; g < ng; ++g) {
    BatchGroup &G = b->groups[g];
    G.s0 = i;
    uint64_t acc = 0;
    const uint64_t want = all_px * (uint64_t)(g + 1) / (uint64_t)ng;
    uint64_t before = 0;
    for (int k = 0; k < i; ++k) before += spx[k];
    do {
      acc += spx[i++];
    } while (i < n - (ng - 1 - g) && before + acc < want);
    if (g == ng - 1) {
      while (i < n) acc += spx[i++];
    }
    G.n = i - G.s0;
  }
  bool ok = cudaMalloc(&b->d_block, b->block_bytes * kRing) == cudaSuccess &&
            cudaMallocHost(&b->h_block, b->block_bytes * kRing) == cudaSuccess &&
            cudaMalloc(&b->d_static, b->desc_bytes) == cudaSuccess &&
            cudaMalloc(&b->d_states, sizeof(DevState) * n) == cudaSuccess &&
            cudaMallocHost(&b->h_states, sizeof(DevState) * n) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->joined, cudaEventDisableTiming) == cudaSuccess;
  if (ok && b->fused) {
    ok = cudaMalloc(&b->d_sched, sizeof(StepSched) * n) == cudaSuccess &&
         cudaMalloc(&b->d_glob, sizeof(StepGlobal)) == cudaSuccess &&
         cudaMemset(b->d_sched, 0, sizeof(StepSched) * n) == cudaSuccess &&
         cudaMemset(b->d_glob, 0, sizeof(StepGlobal)) == cudaSuccess;
    b->step_grid[0] = b->sm_count * batch_step_ctas_per_sm(false);
    b->step_grid[1] = b->sm_count * batch_step_ctas_per_sm(true);
  }
  for (auto &e : b->ring_ev)
    ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
  for (BatchGroup &G : b->groups) {
    std::vector<uint32_t> px(G.n + 1, 0);
    for (int k = 0; k < G.n; ++k) px[k + 1] = px[k] + (uint32_t)spx[G.s0 + k];
    G.total_px = px[G.n];
    ok = ok && cudaMalloc(&G.d_px_start, sizeof(uint32_t) * (G.n + 1)) == cudaSuccess &&
         cudaMalloc(&G.d_prefix, sizeof(uint32_t) * (G.n + 2)) == cudaSuccess &&
         cudaStreamCreateWithFlags(&G.stream, cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&G.last, cudaEventDisableTiming) == cudaSuccess &&
         cudaMemcpy(G.d_px_start, px.data(), sizeof(uint32_t) * (G.n + 1),
                    cudaMemcpyHostToDevice) == cudaSuccess;
    for (auto &e : G.done) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    // a scene's own calls run on its group's stream, in order with its steps
    for (int k = 0; ok && k < G.n; ++k) ok = vh_set_stream(b->scenes[G.s0 + k], G.stream) == VH_OK;
  }
  if (ok) {  // every scene's volume view, for the state gather
    std::vector<SceneDesc> sd((size_t)n);
    std::memset(sd.data(), 0, b->desc_bytes);
    for (int i = 0; i < n; ++i) {
      sd[i].V = handle_view(b->scenes[i]);
      sd[i].C = handle_cam(b->scenes[i]);
    }
    ok = cudaMemcpy(b->d_static, sd.data(), b->desc_bytes, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemset(b->d_block, 0, b->block_bytes * kRing) == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    free_batch(b);
    return VH_ERR_CUDA;
  }
  for (auto &e : b->ring_ev) cudaEventRecord(e, b->stream);
  for (BatchGroup &G : b->groups) cudaEventRecord(G.last, G.stream);
  *out = b;
  return VH_OK;
}

vh_status vh_batch_destroy(vh_batch *b) {
  DeviceScope on_device(b ? b->device : -1);
  if (!on_device.ok()) return VH_ERR_CUDA;
  if (!b) return VH_ERR_INVALID_ARG;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (BatchGroup &g : b->groups) cudaStreamSynchronize(g.stream);
  free_batch(b);
  return VH_OK;
}

int32_t vh_batch_size(const vh_batch *b) { return b ? b->n : 0; }

vh_handle *vh_batch_scene(vh_batch *b, int32_t i) {
  return b && i >= 0 && i < b->n ? b->scenes[i] : nullptr;
}

vh_status vh_batch_process(vh_batch *b, const void *const *depth, int32_t depth_fmt,
                           const uint8_t *const *rgb, const float *c2w, int32_t mem,
                           int32_t with_mesh) {
  VH_NVTX("vh_batch_process");
  DeviceScope on_device(b ? b->device : -1);
  if (!on_device.ok()) return VH_ERR_CUDA;
  if (!b || !depth || !rgb || !c2w) return VH_ERR_INVALID_ARG;
  if (depth_fmt != VH_DEPTH_U16_MM && depth_fmt != VH_DEPTH_F32_M)
    return fail(b, VH_ERR_INVALID_ARG, "unknown depth format");
  if (mem != VH_MEM_HOST && mem != VH_MEM_DEVICE)
    return fail(b, VH_ERR_INVALID_ARG, "unknown memory kind");
  for (int i = 0; i < b->n; ++i) {
    if (!depth[i]) continue;
    if (!rgb[i]) return fail(b, VH_ERR_INVALID_ARG, "scene with depth but no colour");
    for (int k = 0; k < 16; ++k)
      if (!std::isfinite(c2w[16 * i + k]))
        return fail(b, VH_ERR_NOT_FINITE, "camera pose has a non-finite entry");
  }
  // the upload block of this step (host copy reused only after its upload
  // ran; device copy only after every group's step that read it)
  const int k = b->ring_pos;
  unsigned char *blk = b->h_block + b->block_bytes * k;
  if (cudaEventSynchronize(b->ring_ev[k]) != cudaSuccess)
    return fail(b, VH_ERR_CUDA, "upload ring wait failed");
  for (BatchGroup &g : b->groups)
    if (g.used[k] && cudaStreamWaitEvent(b->stream, g.done[k], 0) != cudaSuccess)
      return fail(b, VH_ERR_CUDA, "upload ring wait failed");
  SceneDesc *hd = reinterpret_cast<SceneDesc *>(blk);
  float *hp = reinterpret_cast<float *>(blk + b->desc_bytes);
  uint8_t *ha = blk + b->desc_bytes + b->pose_bytes;
  for (int i = 0; i < b->n; ++i) {
    vh_handle *h = b->scenes[i];
    const FrameBuffers fb = handle_frame_buffers(h);
    SceneDesc &sd = hd[i];
    std::memset(&sd, 0, sizeof(sd));
    sd.V = handle_view(h);
    sd.C = handle_cam(h);
    sd.depth = fb.depth;
    sd.rgb = fb.rgb;
    sd.pose = b->pose(k, i);
    sd.pix = fb.pix;
    sd.tris = fb.tris;
    sd.tri_cap = (uint32_t)std::min<int64_t>(fb.tri_cap, 0xFFFFFFFFll);
    ha[i] = depth[i] ? 1 : 0;
    std::memcpy(hp + 16 * (size_t)i, c2w + 16 * (size_t)i, 16 * sizeof(float));
    if (!depth[i]) continue;
    if (mem == VH_MEM_DEVICE) {  // read in place: no staging copy
      sd.depth = depth[i];
      sd.rgb = rgb[i];
      continue;
    }
  }
  if (cudaMemcpyAsync(b->block(k), blk, b->block_bytes, cudaMemcpyHostToDevice, b->stream) !=
          cudaSuccess ||
      cudaEventRecord(b->ring_ev[k], b->stream) != cudaSuccess)
    return fail(b, VH_ERR_CUDA, "descriptor upload failed");
  b->ring_pos = (k + 1) % kRing;
  const bool graphs_ok = !(handle_params(b->scenes[0]).flags & VH_FLAG_NO_GRAPH);
  int shape[3];
  batch_shape(b, shape);
  if (std::memcmp(shape, b->graph_shape, sizeof(shape)) != 0) {  // tuning changed
    drop_step_graphs(b);
    std::memcpy(b->graph_shape, shape, sizeof(shape));
  }
  for (BatchGroup &g : b->groups) {
    // the descriptors of this step have arrived; host frames are staged on
    // the group's stream, after its previous step has read the staging
    if (cudaStreamWaitEvent(g.stream, b->ring_ev[k], 0) != cudaSuccess)
      return fail(b, VH_ERR_CUDA, "step wait failed");
    bool any = false;
    for (int j = g.s0; j < g.s0 + g.n; ++j) {
      if (!depth[j]) continue;
      any = true;
      if (mem == VH_MEM_DEVICE) continue;
      const FrameBuffers fb = handle_frame_buffers(b->scenes[j]);
      const vh_params &p = handle_params(b->scenes[j]);
      const size_t npx = (size_t)p.width * p.height;
      const size_t dbytes = npx * (depth_fmt == VH_DEPTH_U16_MM ? 2 : 4);
      if (cudaMemcpyAsync(fb.depth, depth[j], dbytes, cudaMemcpyHostToDevice, g.stream) !=
              cudaSuccess ||
          cudaMemcpyAsync(fb.rgb, rgb[j], 3 * npx, cudaMemcpyHostToDevice, g.stream) != cudaSuccess)
        return fail(b, VH_ERR_CUDA, "frame staging failed");
    }
    if (!any) continue;  // no scene of this group has a frame this step
    if (graphs_ok) {
      cudaGraphExec_t &x = g.graphs[depth_fmt][with_mesh ? 1 : 0][k];
      if (!x) {
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
          return fail(b, VH_ERR_CUDA, "capture failed");
        enqueue_group_step(b, g, k, depth_fmt, with_mesh != 0, shape);
        cudaError_t e = cudaStreamEndCapture(g.stream, &graph);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&x, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
          x = nullptr;
          return fail(b, VH_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
        }
      }
      if (cudaGraphLaunch(x, g.stream) != cudaSuccess) return fail(b, VH_ERR_CUDA, "graph launch");
    } else {
      enqueue_group_step(b, g, k, depth_fmt, with_mesh != 0, shape);
      if (cudaGetLastError() != cudaSuccess) return fail(b, VH_ERR_CUDA, "batch launch failed");
    }
    if (cudaEventRecord(g.done[k], g.stream) != cudaSuccess ||
        cudaEventRecord(g.last, g.stream) != cudaSuccess)
      return fail(b, VH_ERR_CUDA, "step record failed");
    g.used[k] = true;
  }
  for (int i = 0; i < b->n; ++i)
    if (depth[i]) handle_note_frame(b->scenes[i]);
  if (handle_params(b->scenes[0]).flags & VH_FLAG_SYNC) return check_batch(b, nullptr, nullptr, false);
  return VH_OK;
}

vh_status vh_batch_sync(vh_batch *b, vh_status *status, vh_stats *stats) {
  VH_NVTX("vh_batch_sync");
  DeviceScope on_device(b ? b->device : -1);
  if (!on_device.ok()) return VH_ERR_CUDA;
  if (!b) return VH_ERR_INVALID_ARG;
  return check_batch(b, status, stats, true);
}

}  // extern "C"

namespace {

// Waits for the batch and maps every scene's sticky error bits to a status;
// `clear` resets them afterwards.
vh_status check_batch(vh_batch *b, vh_status *status, vh_stats *stats, bool clear) {
  for (BatchGroup &g : b->groups)  // every group's latest work, including its scenes' calls
    if (cudaEventRecord(g.last, g.stream) != cudaSuccess ||
        cudaStreamWaitEvent(b->stream, g.last, 0) != cudaSuccess)
      return fail(b, VH_ERR_CUDA, "batch join failed");
  launch_batch_gather_state(b->d_static, b->n, b->d_states, b->stream);
  if (cudaMemcpyAsync(b->h_states, b->d_states, sizeof(DevState) * b->n, cudaMemcpyDeviceToHost,
                      b->stream) != cudaSuccess ||
      cudaStreamSynchronize(b->stream) != cudaSuccess)
    return fail(b, VH_ERR_CUDA, std::string("batch sync: ") + cudaGetErrorString(cudaGetLastError()));
  vh_status first = VH_OK;
  bool any_error = false;
  for (int i = 0; i < b->n; ++i) {
    const DevState &st = b->h_states[i];
    vh_handle *h = b->scenes[i];
    const vh_status s = handle_status_of_bits(h, st.error);
    any_error = any_error || st.error;
    if (status) status[i] = s;
    if (s != VH_OK && first == VH_OK) first = s;
    if (stats) {
      const vh_params &p = handle_params(h);
      vh_stats &o = stats[i];
      std::memset(&o, 0, sizeof(o));
      o.frames = handle_frames(h);
      o.blocks_allocated = (int64_t)st.pool_top - (int64_t)st.free_count;
      o.frame_blocks = std::min<int64_t>(st.frame_count, p.max_frame_blocks);
      o.new_blocks = st.new_blocks;
      o.voxels_updated = (int64_t)st.voxels_updated;
      o.triangles = st.tri_count;
      o.pool_capacity = p.pool_blocks;
      o.table_slots = (int64_t)1 << p.table_log2;
      o.tombstones = st.tombstones;
      o.device_error = st.error;
    }
  }
  if (any_error && clear) {
    launch_batch_clear_errors(b->d_static, b->n, b->stream);
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return fail(b, VH_ERR_CUDA, "clear failed");
  }
  return first;
}

}  // namespace
