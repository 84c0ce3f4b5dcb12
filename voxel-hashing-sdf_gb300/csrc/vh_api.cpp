// vh_api.cpp - host orchestration behind the C ABI (include/vhsdf.h).
//
// The reference's processFrame (src/tsdf.cu:1484-1598) rebuilds two hash
// tables, streams host chunks in, runs three kernels with blocking copies in
// between and streams everything back out every frame.  Here the volume stays
// resident in HBM; a frame is one CUDA graph
//     frame_begin -> allocate -> resolve -> integrate [-> mc]
// whose first kernel carries the frame's descriptor (pose, image addresses)
// as a parameter updated per launch.  Device images are read in place; host
// images are uploaded on a copy stream into one of two staging slots,
// overlapping the previous frame.  All counts stay on the device; the host
// reads the state block only when a call has to report something
// (VH_FLAG_SYNC, stats, mesh copies), and without VH_FLAG_SYNC the frame's
// last kernel writes it to mapped host memory at the end of every frame.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/vhsdf.h"
#include "vh_common.cuh"
#include "vh_internal.h"
#include "vh_mc_tables.h"
#include "vh_mesh.h"

using namespace vh;

namespace {
constexpr int kNumEvents = 5;
// Marching-cubes mode of a frame graph: none, into the handle's triangle
// buffer (vh_process_frame, vh_extract), into mesh slot 0 / 1 of
// vh_process_frame_mesh, or as an indexed mesh into slot 0 / 1 of
// vh_process_frame_indexed.
enum { kMcNone = 0, kMcMain = 1, kMcSlot0 = 2, kMcSlot1 = 3, kMcIdx0 = 4, kMcIdx1 = 5,
       kMcModes = 6 };
}  // namespace

struct vh_handle {
  vh_params p{};
  int sm_count = 0;
  int integrate_per_sm = 1;  // resident CTAs per SM in use
  int mc_per_sm = 1;
  vh_tuning tuning{};        // requested configuration (0 = occupancy max)
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  VolumeView V{};
  CamParams C{};
  void *d_depth = nullptr;      // staging of single images (refinement, batches)
  float *d_depth_f = nullptr;  // filtered depth (VH_FLAG_DEPTH_FILTER)
  uint8_t *d_rgb = nullptr;
  FrameIn *d_fin = nullptr;    // the current frame's pose and image pointers
  FrameIn fin{};               // the next frame's, passed to k_frame_begin
  uint2 *d_pix = nullptr;
  float *d_rcp = nullptr;  // correctly rounded 1 / w for the integration update
  float4 *d_tris = nullptr;
  int64_t tri_cap = 0;
  // Host frames: two device slots filled on copy_stream, so the upload of a
  // frame overlaps the kernels of the one before.  in_copied[k] follows the
  // upload into slot k, in_consumed[k] the kernels of the frame that read it.
  cudaStream_t copy_stream = nullptr;
  void *d_in_depth[2] = {nullptr, nullptr};
  uint8_t *d_in_rgb[2] = {nullptr, nullptr};
  cudaEvent_t in_copied[2] = {}, in_consumed[2] = {};
  int in_pos = 0;
  int in_used = -1;  // slot read by the frame being enqueued (-1: device inputs)
  DevState *h_state = nullptr;    // pinned, mapped
  DevState *h_state_dev = nullptr;  // its device address (k_state_out)
  // Frame graphs per depth format and marching-cubes mode (kMc*).
  cudaGraphExec_t graphs[2][kMcModes] = {};
  cudaGraph_t graph_src[2][kMcModes] = {};
  cudaGraphNode_t graph_fb[2][kMcModes] = {};  // k_frame_begin
  int frame_kernels = 0;  // kernels one frame launches (counted when enqueued)
  // Per-frame meshes to host (vh_process_frame_mesh): two device triangle
  // buffers and two mapped counter mirrors, used by alternate frames, so that
  // one frame's copy-out overlaps the next frame's kernels.
  float4 *d_mtris[2] = {nullptr, nullptr};
  int64_t mtri_cap = 0;
  // Indexed per-frame meshes (vh_process_frame_indexed): vertices and faces
  // of the two slots (the slots' mirrors, events and stream are shared).
  float4 *d_mverts[2] = {nullptr, nullptr};
  int32_t *d_mfaces[2] = {nullptr, nullptr};
  int64_t midx_cap = 0;  // vertices and faces each slot holds
  int mcidx_per_sm = 1;
  DevState *h_mstate = nullptr;      // 2 entries, pinned and mapped
  DevState *h_mstate_dev = nullptr;  // their device address
  cudaStream_t mesh_stream = nullptr;
  cudaEvent_t mesh_done[2] = {}, mesh_copied[2] = {};
  bool mesh_copy_issued[2] = {false, false};
  int mesh_slot = 0;
  struct PendingMesh {
    bool valid = false;
    bool indexed = false;  // faces in tris/capacity/count, vertices below
    int slot = 0;
    float *tris = nullptr;
    int64_t capacity = 0;
    int64_t *count = nullptr;
    float *verts = nullptr;
    int64_t vcapacity = 0;
    int64_t *vcount = nullptr;
  } pending;
  bool mesh_overflow = false;  // a frame had more triangles than its host buffer
  cudaEvent_t ev[kNumEvents] = {};
  bool ev_pending = false;
  bool ev_has_mc = false;
  void *d_work = nullptr;  // workspace of the gradient calls
  size_t work_bytes = 0;
  RefineCtx *refine = nullptr;  // device state of pose refinement (vh_adjoint.cu)
  StreamStore *stream_store = nullptr;  // streamed-out blocks (vh_stream.cu)
  int64_t frames = 0;
  bool nb_valid = false;  // frame_nb matches the current block list
  std::string last_error;
  vh_stats stage{};
};

namespace vh {
namespace {
std::mutex g_log_mu;
vh_log_fn g_log_fn = nullptr;
void *g_log_user = nullptr;
}  // namespace

void log_error(const std::string &msg) {
  vh_log_fn fn;
  void *user;
  {
    std::lock_guard<std::mutex> lock(g_log_mu);
    fn = g_log_fn;
    user = g_log_user;
  }
  if (fn) fn(VH_LOG_ERROR, msg.c_str(), user);  // outside the lock
}

void set_log(vh_log_fn fn, void *user) {
  std::lock_guard<std::mutex> lock(g_log_mu);
  g_log_fn = fn;
  g_log_user = user;
}
}  // namespace vh

namespace {

vh_status fail(vh_handle *h, vh_status s, const std::string &msg) {
  if (h) h->last_error = msg;
  vh::log_error(msg);
  return s;
}

vh_status cuda_fail(vh_handle *h, cudaError_t e, const char *what) {
  return fail(h, VH_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define VH_CUDA(h, expr)                                   \
  do {                                                     \
    cudaError_t e__ = (expr);                              \
    if (e__ != cudaSuccess) return cuda_fail(h, e__, #expr); \
  } while (0)

// 1 / b correctly rounded to float: the double quotient rounded once, then
// the float neighbours checked in case that double rounding missed.
float rn_reciprocal(float b) {
  const double ex = 1.0 / (double)b;
  float y = (float)ex;
  const float up = std::nextafter(y, INFINITY), down = std::nextafter(y, -INFINITY);
  if (std::fabs((double)up - ex) < std::fabs((double)y - ex)) y = up;
  if (std::fabs((double)down - ex) < std::fabs((double)y - ex)) y = down;
  return y;
}

bool finite_pose(const float *c2w) {
  for (int i = 0; i < 16; ++i)
    if (!std::isfinite(c2w[i])) return false;
  return true;
}

// Maps sticky device error bits to a status (most severe first).
vh_status status_of_bits(uint32_t bits, std::string &msg) {
  if (bits & kErrTableFull) {
    msg = "hash table full: a probe sequence reached max_probe";
    return VH_ERR_TABLE_FULL;
  }
  if (bits & kErrPoolFull) {
    msg = "voxel-block pool exhausted (raise pool_blocks)";
    return VH_ERR_POOL_FULL;
  }
  if (bits & kErrRange) {
    msg = "a block coordinate left the key range [-2^20, 2^20)";
    return VH_ERR_OUT_OF_RANGE;
  }
  if (bits & kErrFrameCap) {
    msg = "frame block list overflowed max_frame_blocks";
    return VH_ERR_CAPACITY;
  }
  if (bits & kErrTriCap) {
    msg = "triangle buffer overflowed max_triangles";
    return VH_ERR_CAPACITY;
  }
  if (bits & kErrRetry) {
    msg = "a bounded device wait gave up";
    return VH_ERR_RETRY_EXHAUSTED;
  }
  if (bits & kErrCheck) {
    msg = "an index check of the checked build failed (access skipped)";
    return VH_ERR_CHECK;
  }
  return VH_OK;
}

// Copies the device state into h->h_state and waits for the stream.
vh_status pull_state(vh_handle *h) {
  VH_CUDA(h, cudaMemcpyAsync(h->h_state, h->V.st, sizeof(DevState), cudaMemcpyDeviceToHost,
                             h->stream));
  VH_CUDA(h, cudaStreamSynchronize(h->stream));
  VH_CUDA(h, cudaGetLastError());
  return VH_OK;
}

// Synchronises, then reports (and clears) sticky device errors.
vh_status sync_and_check(vh_handle *h) {
  vh_status s = pull_state(h);
  if (s != VH_OK) return s;
  if (h->ev_pending && (h->p.flags & VH_FLAG_PROFILE)) {
    float a = 0, b = 0, c = 0;
    cudaEventElapsedTime(&a, h->ev[0], h->ev[1]);
    cudaEventElapsedTime(&b, h->ev[1], h->ev[2]);
    h->stage.ms_allocate = a;
    h->stage.ms_integrate = b;
    if (h->ev_has_mc) {
      cudaEventElapsedTime(&c, h->ev[2], h->ev[3]);
      h->stage.ms_extract = c;
      cudaEventElapsedTime(&a, h->ev[0], h->ev[3]);
    } else {
      h->stage.ms_extract = 0;
      cudaEventElapsedTime(&a, h->ev[0], h->ev[2]);
    }
    h->stage.ms_frame = a;
    h->ev_pending = false;
  }
  const uint32_t bits = h->h_state->error;
  if (!bits) return VH_OK;
  std::string msg;
  vh_status st = status_of_bits(bits, msg);
  VH_CUDA(h, cudaMemsetAsync(&h->V.st->error, 0, sizeof(uint32_t), h->stream));
  VH_CUDA(h, cudaStreamSynchronize(h->stream));
  return fail(h, st, msg);
}

// Persistent grids: exactly the CTAs that are resident at once (no tail wave).
int integrate_grid(const vh_handle *h) { return h->sm_count * h->integrate_per_sm; }
int mc_grid(const vh_handle *h) { return h->sm_count * h->mc_per_sm; }

// Records a stage event; inside a stream capture it must become a real
// event-record node of the graph (cudaEventRecordExternal).
void stage_event(cudaEvent_t ev, cudaStream_t s, bool capturing) {
  if (capturing)
    cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal);
  else
    cudaEventRecord(ev, s);
}

// Enqueues one frame's kernels (optionally with per-stage events); mc is a
// kMc* mode.  Counts the kernels it launches into h->frame_kernels.
void enqueue_frame(vh_handle *h, int fmt, int mc, bool events, bool capturing) {
  cudaStream_t s = h->stream;
  int kernels = 0;
  if (events) stage_event(h->ev[0], s, capturing);
  launch_frame_begin(h->V, &h->fin, h->d_fin, s);
  ++kernels;
  // the frame's own image, found through d_fin; the depth pre-filter runs
  // inside the allocation kernel, whose pixel records integration reads
  launch_allocate(h->V, h->C, h->d_fin, nullptr, fmt, (h->p.flags & VH_FLAG_DEPTH_FILTER) != 0,
                  h->d_pix, s);
  launch_frame_resolve(h->V, h->sm_count * 8, mc != kMcNone, s);  // probes in flight: many CTAs
  kernels += 2;
  if (events) stage_event(h->ev[1], s, capturing);
  launch_integrate(h->V, h->C, h->d_pix, h->d_fin->pose, integrate_grid(h),
                   h->tuning.integrate_variant, s);
  ++kernels;
  if (events) stage_event(h->ev[2], s, capturing);
  // Without VH_FLAG_SYNC every frame still brings its counters to the host
  // mirror (a 64-byte in-stream write to mapped memory, no copy on the
  // stream): by the last MC CTA, or by k_state_out after an integration.
  // Frames of vh_process_frame_mesh use their slot's own mirror and buffer.
  DevState *mirror = (h->p.flags & VH_FLAG_SYNC) ? nullptr : h->h_state_dev;
  if (mc != kMcNone) {
    float4 *tris = h->d_tris;
    int64_t cap = h->tri_cap;
    if (mc == kMcSlot0 || mc == kMcSlot1) {
      const int k = mc - kMcSlot0;
      tris = h->d_mtris[k];
      cap = h->mtri_cap;
      mirror = h->h_mstate_dev + k;
    }
    if (mc == kMcIdx0 || mc == kMcIdx1) {
      const int k = mc - kMcIdx0;
      launch_mc_indexed(h->V, h->C.mc_min_weight, h->d_mverts[k], (uint32_t)h->midx_cap,
                        h->d_mfaces[k], (uint32_t)h->midx_cap, h->sm_count * h->mcidx_per_sm,
                        h->h_mstate_dev + k, s);
    } else {
      launch_mc(h->V, 0, h->C.mc_min_weight, tris, (uint32_t)cap, mc_grid(h),
                h->tuning.mc_variant, mirror, s);
    }
    ++kernels;
    if (events) stage_event(h->ev[3], s, capturing);
  } else if (mirror) {
    launch_state_out(h->V, mirror, s);
    ++kernels;
  }
  h->frame_kernels = kernels;
}

void drop_graphs(vh_handle *h) {
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < kMcModes; ++b) {
      if (h->graphs[a][b]) cudaGraphExecDestroy(h->graphs[a][b]);
      if (h->graph_src[a][b]) cudaGraphDestroy(h->graph_src[a][b]);
      h->graphs[a][b] = nullptr;
      h->graph_src[a][b] = nullptr;
      h->graph_fb[a][b] = nullptr;
    }
}

// Resolves a requested configuration against the occupancy limits.
void apply_tuning(vh_handle *h, const vh_tuning &t) {
  h->tuning = t;
  h->tuning.integrate_variant =
      t.integrate_variant > 0 && t.integrate_variant < integrate_variants() ? t.integrate_variant : 0;
  h->tuning.mc_variant = t.mc_variant > 0 && t.mc_variant < mc_variants() ? t.mc_variant : 0;
  const int imax = integrate_ctas_per_sm(h->tuning.integrate_variant);
  const int mmax = mc_ctas_per_sm(h->tuning.mc_variant);
  h->integrate_per_sm =
      t.integrate_ctas_per_sm > 0 && t.integrate_ctas_per_sm < imax ? t.integrate_ctas_per_sm : imax;
  h->mc_per_sm = t.mc_ctas_per_sm > 0 && t.mc_ctas_per_sm < mmax ? t.mc_ctas_per_sm : mmax;
  h->tuning.integrate_ctas_per_sm = h->integrate_per_sm;
  h->tuning.mc_ctas_per_sm = h->mc_per_sm;
  drop_graphs(h);  // graphs hold the grid sizes
}

// Runs the frame chain as a CUDA graph (captured on first use) or directly.
vh_status inputs_consumed(vh_handle *h);

vh_status run_frame(vh_handle *h, int fmt, int mc) {
  const bool events = (h->p.flags & VH_FLAG_PROFILE) != 0;
  const bool graphs_ok = !(h->p.flags & VH_FLAG_NO_GRAPH) && h->stream != nullptr;
  if (graphs_ok) {
    const int m = mc;
    cudaGraphExec_t &g = h->graphs[fmt][m];
    if (!g) {  // captured with this frame's descriptor
      cudaGraph_t graph = nullptr;
      VH_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
      enqueue_frame(h, fmt, mc, events, true);
      cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
      if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
      e = cudaGraphInstantiate(&g, graph, 0);
      if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        g = nullptr;
        return cuda_fail(h, e, "cudaGraphInstantiate");
      }
      h->graph_src[fmt][m] = graph;  // its nodes address the parameter updates
      h->graph_fb[fmt][m] = find_frame_begin_node(graph);
      if (!h->graph_fb[fmt][m]) {
        drop_graphs(h);
        return fail(h, VH_ERR_CUDA, "frame graph without its begin node");
      }
    } else {
      const cudaError_t e = update_frame_begin(g, h->graph_fb[fmt][m], h->V, h->fin, h->d_fin);
      if (e != cudaSuccess) return cuda_fail(h, e, "cudaGraphExecKernelNodeSetParams");
    }
    VH_CUDA(h, cudaGraphLaunch(g, h->stream));
  } else {
    enqueue_frame(h, fmt, mc, events, false);
    VH_CUDA(h, cudaGetLastError());
  }
  h->ev_pending = events;
  h->ev_has_mc = mc != kMcNone;
  return inputs_consumed(h);
}

// Prepares one frame's descriptor (h->fin, written to d_fin by the frame's
// first kernel): device images are read in place (the caller keeps them
// unchanged until the frame's work on the handle's stream has run), host
// images are uploaded into a staging slot on the copy stream, which the
// handle's stream waits for.  run_frame records inputs_consumed() after the
// frame's kernels.
vh_status stage_inputs(vh_handle *h, const void *depth, int32_t fmt, const uint8_t *rgb,
                       const float *c2w, int32_t mem) {
  if (!depth || !rgb || !c2w) return fail(h, VH_ERR_INVALID_ARG, "null input pointer");
  if (fmt != VH_DEPTH_U16_MM && fmt != VH_DEPTH_F32_M)
    return fail(h, VH_ERR_INVALID_ARG, "unknown depth format");
  if (mem != VH_MEM_HOST && mem != VH_MEM_DEVICE)
    return fail(h, VH_ERR_INVALID_ARG, "unknown memory kind");
  if (!finite_pose(c2w)) return fail(h, VH_ERR_NOT_FINITE, "camera pose has a non-finite entry");
  const size_t npx = (size_t)h->p.width * h->p.height;
  FrameIn *slot = &h->fin;
  std::memcpy(slot->pose, c2w, 16 * sizeof(float));
  h->in_used = -1;
  if (mem == VH_MEM_DEVICE) {
    slot->depth = depth;
    slot->rgb = rgb;
  } else {
    const int k = h->in_pos;  // last read by the frame two host frames back
    const size_t dbytes = npx * (fmt == VH_DEPTH_U16_MM ? 2 : 4);
    VH_CUDA(h, cudaStreamWaitEvent(h->copy_stream, h->in_consumed[k], 0));
    VH_CUDA(h, cudaMemcpyAsync(h->d_in_depth[k], depth, dbytes, cudaMemcpyHostToDevice,
                               h->copy_stream));
    VH_CUDA(h, cudaMemcpyAsync(h->d_in_rgb[k], rgb, 3 * npx, cudaMemcpyHostToDevice,
                               h->copy_stream));
    VH_CUDA(h, cudaEventRecord(h->in_copied[k], h->copy_stream));
    VH_CUDA(h, cudaStreamWaitEvent(h->stream, h->in_copied[k], 0));
    slot->depth = h->d_in_depth[k];
    slot->rgb = h->d_in_rgb[k];
    h->in_used = k;
    h->in_pos ^= 1;
  }
  return VH_OK;
}

// After the frame's kernels: its host staging slot may be refilled.
vh_status inputs_consumed(vh_handle *h) {
  if (h->in_used >= 0) VH_CUDA(h, cudaEventRecord(h->in_consumed[h->in_used], h->stream));
  h->in_used = -1;
  return VH_OK;
}

void free_all(vh_handle *h) {
  if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
  if (h->mesh_stream) cudaStreamSynchronize(h->mesh_stream);
  for (int k = 0; k < 2; ++k) {
    cudaFree(h->d_mtris[k]);
    cudaFree(h->d_mverts[k]);
    cudaFree(h->d_mfaces[k]);
    if (h->mesh_done[k]) cudaEventDestroy(h->mesh_done[k]);
    if (h->mesh_copied[k]) cudaEventDestroy(h->mesh_copied[k]);
  }
  if (h->h_mstate) cudaFreeHost(h->h_mstate);
  if (h->mesh_stream) cudaStreamDestroy(h->mesh_stream);
  drop_graphs(h);
  refine_ctx_free(h->refine);
  h->refine = nullptr;
  stream_store_free(h->stream_store);
  h->stream_store = nullptr;
  cudaFree(h->V.slots);
  cudaFree(h->V.pool);
  cudaFree(h->V.block_keys);
  cudaFree(h->V.free_list);
  cudaFree(h->V.frame_list);
  cudaFree(h->V.frame_nb);
  cudaFree(h->V.frame_res);
  cudaFree(h->V.st);
  cudaFree(h->d_depth);
  cudaFree(h->d_depth_f);
  cudaFree(h->d_rgb);
  cudaFree(h->d_fin);
  for (int k = 0; k < 2; ++k) {
    cudaFree(h->d_in_depth[k]);
    cudaFree(h->d_in_rgb[k]);
    if (h->in_copied[k]) cudaEventDestroy(h->in_copied[k]);
    if (h->in_consumed[k]) cudaEventDestroy(h->in_consumed[k]);
  }
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  cudaFree(h->d_pix);
  cudaFree(h->d_rcp);
  cudaFree(h->d_tris);
  cudaFree(h->d_work);
  if (h->h_state) cudaFreeHost(h->h_state);
  for (auto &e : h->ev)
    if (e) cudaEventDestroy(e);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
}

// Clears table, pool blocks in use, key list and counters.
vh_status clear_volume(vh_handle *h, bool zero_pool_prefix) {
  cudaStream_t s = h->stream;
  uint32_t used = (uint32_t)h->p.pool_blocks;
  if (zero_pool_prefix) {
    vh_status st = pull_state(h);
    if (st != VH_OK) return st;
    used = h->h_state->pool_top;
  }
  VH_CUDA(h, cudaMemsetAsync(h->V.slots, 0xFF, sizeof(Slot) * ((size_t)h->V.slot_mask + 1), s));
  VH_CUDA(h, cudaMemsetAsync(h->V.block_keys, 0xFF, sizeof(unsigned long long) * h->p.pool_blocks, s));
  if (used)
    VH_CUDA(h, cudaMemsetAsync(h->V.pool, 0, sizeof(float) * kBlockWords * (size_t)used, s));
  VH_CUDA(h, cudaMemsetAsync(h->V.st, 0, sizeof(DevState), s));
  VH_CUDA(h, cudaStreamSynchronize(s));
  h->frames = 0;
  h->nb_valid = false;
  return VH_OK;
}

template <typename T>
struct DevBuf {
  T *ptr = nullptr;
  ~DevBuf() {
    if (ptr) cudaFree(ptr);
  }
};

// Makes `n` elements available on the device: returns `src` itself for
// device memory, else a temporary copy.
template <typename T>
vh_status device_view(vh_handle *h, const T *src, size_t n, int32_t mem, DevBuf<T> &tmp,
                      const T **out) {
  if (mem == VH_MEM_DEVICE) {
    *out = src;
    return VH_OK;
  }
  if (mem != VH_MEM_HOST) return fail(h, VH_ERR_INVALID_ARG, "unknown memory kind");
  VH_CUDA(h, cudaMalloc(&tmp.ptr, sizeof(T) * (n ? n : 1)));
  VH_CUDA(h, cudaMemcpyAsync(tmp.ptr, src, sizeof(T) * n, cudaMemcpyHostToDevice, h->stream));
  *out = tmp.ptr;
  return VH_OK;
}

vh_status grow_tris(vh_handle *h, int64_t need) {
  int64_t cap = need + need / 4 + 1024;
  if (cap > 0x7FFFFFFF / 3) cap = 0x7FFFFFFF / 3;
  if (cap <= h->tri_cap) return VH_OK;
  VH_CUDA(h, cudaStreamSynchronize(h->stream));
  cudaFree(h->d_tris);
  h->d_tris = nullptr;
  h->tri_cap = 0;
  drop_graphs(h);  // captured graphs hold the old pointer
  VH_CUDA(h, cudaMalloc(&h->d_tris, sizeof(float4) * 3 * (size_t)cap));
  h->tri_cap = cap;
  return VH_OK;
}

// First use of vh_process_frame_mesh / vh_process_frame_indexed: the two
// slots' mapped counter mirrors, the copy-out stream and its events, then
// the slots' buffers of the kind asked for (triangle soup, or vertices and
// faces), each of max_triangles entries.
vh_status mesh_setup(vh_handle *h, bool indexed) {
  const int64_t cap = h->tri_cap ? h->tri_cap : 1;
  if (!h->mesh_stream) {
    bool ok =
        cudaHostAlloc(&h->h_mstate, 2 * sizeof(DevState), cudaHostAllocMapped) == cudaSuccess &&
        cudaHostGetDevicePointer(&h->h_mstate_dev, h->h_mstate, 0) == cudaSuccess;
    for (int k = 0; ok && k < 2; ++k)
      ok = cudaEventCreateWithFlags(&h->mesh_done[k], cudaEventDisableTiming) == cudaSuccess &&
           cudaEventCreateWithFlags(&h->mesh_copied[k], cudaEventDisableTiming) == cudaSuccess;
    if (ok) ok = cudaStreamCreateWithFlags(&h->mesh_stream, cudaStreamNonBlocking) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      for (int k = 0; k < 2; ++k) {
        if (h->mesh_done[k]) cudaEventDestroy(h->mesh_done[k]);
        if (h->mesh_copied[k]) cudaEventDestroy(h->mesh_copied[k]);
        h->mesh_done[k] = h->mesh_copied[k] = nullptr;
      }
      if (h->h_mstate) cudaFreeHost(h->h_mstate);
      h->h_mstate = h->h_mstate_dev = nullptr;
      return fail(h, VH_ERR_CUDA, "per-frame mesh buffers: allocation failed");
    }
    std::memset(h->h_mstate, 0, 2 * sizeof(DevState));
  }
  if (!indexed && !h->d_mtris[0]) {
    const bool ok =
        cudaMalloc(&h->d_mtris[0], sizeof(float4) * 3 * (size_t)cap) == cudaSuccess &&
        cudaMalloc(&h->d_mtris[1], sizeof(float4) * 3 * (size_t)cap) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      for (int k = 0; k < 2; ++k) {
        cudaFree(h->d_mtris[k]);
        h->d_mtris[k] = nullptr;
      }
      return fail(h, VH_ERR_CUDA, "per-frame mesh buffers: allocation failed");
    }
    h->mtri_cap = cap;
  }
  if (indexed && !h->d_mverts[0]) {
    bool ok = true;
    for (int k = 0; ok && k < 2; ++k)
      ok = cudaMalloc(&h->d_mverts[k], sizeof(float4) * (size_t)cap) == cudaSuccess &&
           cudaMalloc(&h->d_mfaces[k], 3 * sizeof(int32_t) * (size_t)cap) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      for (int k = 0; k < 2; ++k) {
        cudaFree(h->d_mverts[k]);
        cudaFree(h->d_mfaces[k]);
        h->d_mverts[k] = nullptr;
        h->d_mfaces[k] = nullptr;
      }
      return fail(h, VH_ERR_CUDA, "per-frame indexed mesh buffers: allocation failed");
    }
    h->midx_cap = cap;
    h->mcidx_per_sm = mc_indexed_ctas_per_sm();
  }
  return VH_OK;
}

// Issues the copy-out of the pending mesh frame: waits (host) for that
// frame's kernels, reads its triangle count from its slot's mirror and
// copies the triangles into the caller's buffer on the mesh stream.
vh_status mesh_flush(vh_handle *h) {
  if (!h->pending.valid) return VH_OK;
  vh_handle::PendingMesh p = h->pending;
  h->pending.valid = false;
  VH_CUDA(h, cudaEventSynchronize(h->mesh_done[p.slot]));
  const int64_t n = h->h_mstate[p.slot].tri_count;
  if (p.indexed) {  // faces, then the vertices they number
    const int64_t nv = h->h_mstate[p.slot].vert_count;
    const int64_t mf = std::min(std::min(n, p.capacity), h->midx_cap);
    const int64_t mv = std::min(std::min(nv, p.vcapacity), h->midx_cap);
    if (mv > 0)
      VH_CUDA(h, cudaMemcpyAsync(p.verts, h->d_mverts[p.slot], sizeof(float4) * (size_t)mv,
                                 cudaMemcpyDeviceToHost, h->mesh_stream));
    if (mf > 0)
      VH_CUDA(h, cudaMemcpyAsync(p.tris, h->d_mfaces[p.slot], 3 * sizeof(int32_t) * (size_t)mf,
                                 cudaMemcpyDeviceToHost, h->mesh_stream));
    if (p.vcount) *p.vcount = nv;
    if (nv > p.vcapacity) h->mesh_overflow = true;
  } else {
    const int64_t m = std::min(std::min(n, p.capacity), h->mtri_cap);
    if (m > 0)
      VH_CUDA(h, cudaMemcpyAsync(p.tris, h->d_mtris[p.slot], sizeof(float4) * 3 * (size_t)m,
                                 cudaMemcpyDeviceToHost, h->mesh_stream));
  }
  VH_CUDA(h, cudaEventRecord(h->mesh_copied[p.slot], h->mesh_stream));
  h->mesh_copy_issued[p.slot] = true;
  if (p.count) *p.count = n;
  if (n > p.capacity) h->mesh_overflow = true;
  // the copy issued by the previous flush (the frame before) is complete
  // when this returns: a caller may reuse that frame's buffer
  const int q = p.slot ^ 1;
  if (h->mesh_copy_issued[q]) VH_CUDA(h, cudaEventSynchronize(h->mesh_copied[q]));
  return VH_OK;
}

// Every pending mesh copied out; a mesh larger than its host buffer is
// reported (once) as VH_ERR_CAPACITY.
vh_status mesh_drain(vh_handle *h) {
  if (!h->mesh_stream) return VH_OK;
  vh_status s = mesh_flush(h);
  if (s != VH_OK) return s;
  VH_CUDA(h, cudaStreamSynchronize(h->mesh_stream));
  if (h->mesh_overflow) {
    h->mesh_overflow = false;
    return fail(h, VH_ERR_CAPACITY, "a frame's mesh was larger than its host buffer");
  }
  return VH_OK;
}

}  // namespace

namespace vh {
VolumeView handle_view(const vh_handle *h) { return h->V; }
cudaStream_t handle_stream(const vh_handle *h) { return h->stream; }
int handle_device(const vh_handle *h) { return h->p.device; }
vh_status handle_fail(vh_handle *h, vh_status s, const char *msg) { return fail(h, s, msg); }
vh_status handle_sync(vh_handle *h) { return sync_and_check(h); }
CamParams handle_cam(const vh_handle *h) { return h->C; }
int handle_sm_count(const vh_handle *h) { return h->sm_count; }
vh_status handle_stage_depth(vh_handle *h, const void *depth, int fmt, int mem, const void **dev) {
  if (!depth || (fmt != VH_DEPTH_U16_MM && fmt != VH_DEPTH_F32_M) ||
      (mem != VH_MEM_HOST && mem != VH_MEM_DEVICE))
    return fail(h, VH_ERR_INVALID_ARG, "bad depth argument");
  const size_t bytes = (size_t)h->p.width * h->p.height * (fmt == VH_DEPTH_U16_MM ? 2 : 4);
  VH_CUDA(h, cudaMemcpyAsync(h->d_depth, depth, bytes,
                             mem == VH_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                             h->stream));
  *dev = h->d_depth;
  return VH_OK;
}
RefineCtx *&handle_refine(vh_handle *h) { return h->refine; }
StreamStore *&handle_stream_store(vh_handle *h) { return h->stream_store; }
const DevState &handle_state(const vh_handle *h) { return *h->h_state; }
void handle_invalidate_nb(vh_handle *h) { h->nb_valid = false; }

FrameBuffers handle_frame_buffers(const vh_handle *h) {
  return FrameBuffers{h->d_depth, h->d_rgb, h->d_pix, h->d_tris, h->tri_cap,
                      h->integrate_per_sm, h->mc_per_sm, h->tuning.mc_variant};
}

const vh_params &handle_params(const vh_handle *h) { return h->p; }

int64_t handle_frames(const vh_handle *h) { return h->frames; }

void handle_note_frame(vh_handle *h) {
  h->frames++;
  h->nb_valid = true;
  h->ev_pending = false;
}

vh_status handle_status_of_bits(vh_handle *h, uint32_t bits) {
  if (!bits) return VH_OK;
  std::string msg;
  const vh_status st = status_of_bits(bits, msg);
  return fail(h, st, msg);
}

vh_status handle_workspace(vh_handle *h, size_t bytes, void **ptr) {
  if (bytes > h->work_bytes) {
    VH_CUDA(h, cudaStreamSynchronize(h->stream));
    cudaFree(h->d_work);
    h->d_work = nullptr;
    h->work_bytes = 0;
    VH_CUDA(h, cudaMalloc(&h->d_work, bytes));
    h->work_bytes = bytes;
  }
  *ptr = h->d_work;
  return VH_OK;
}
}  // namespace vh

extern "C" {

const char *vh_status_string(vh_status s) {
  switch (s) {
    case VH_OK: return "ok";
    case VH_ERR_INVALID_ARG: return "invalid argument";
    case VH_ERR_CUDA: return "CUDA error";
    case VH_ERR_TABLE_FULL: return "hash table full";
    case VH_ERR_POOL_FULL: return "block pool full";
    case VH_ERR_RETRY_EXHAUSTED: return "retry limit reached";
    case VH_ERR_NOT_FINITE: return "non-finite input";
    case VH_ERR_UNSUPPORTED: return "unsupported";
    case VH_ERR_OUT_OF_RANGE: return "coordinate out of range";
    case VH_ERR_CAPACITY: return "capacity exceeded";
    case VH_ERR_IO: return "I/O error";
    case VH_ERR_NO_DEVICE: return "no CUDA device";
    case VH_ERR_CHECK: return "bounds check failed";
  }
  return "unknown status";
}

vh_status vh_params_default(vh_params *p) {
  if (!p) return VH_ERR_INVALID_ARG;
  std::memset(p, 0, sizeof(*p));
  p->width = 640;
  p->height = 480;
  p->fx = 577.0f;
  p->fy = 577.0f;
  p->cx = 320.0f;
  p->cy = 240.0f;
  p->min_depth = 0.1f;
  p->max_depth = 10.0f;
  p->depth_scale = 0.001f;
  p->voxel_size = 0.036f;
  p->trunc = 0.18f;
  p->mc_min_weight = 1.0f;
  p->table_log2 = 20;
  p->max_probe = 256;
  p->pool_blocks = 1 << 18;
  p->max_frame_blocks = 1 << 18;
  p->max_triangles = 1 << 22;
  p->flags = VH_FLAG_SYNC;
  p->device = 0;
  return VH_OK;
}

vh_status vh_params_validate(const vh_params *p) {
  if (!p) return VH_ERR_INVALID_ARG;
  if (p->width < 1 || p->height < 1 || p->width > 16384 || p->height > 16384)
    return VH_ERR_INVALID_ARG;
  const float fs[] = {p->fx, p->fy, p->cx, p->cy, p->min_depth, p->max_depth,
                      p->depth_scale, p->voxel_size, p->trunc, p->mc_min_weight};
  for (float f : fs)
    if (!std::isfinite(f)) return VH_ERR_NOT_FINITE;
  if (!(p->fx > 0) || !(p->fy > 0)) return VH_ERR_INVALID_ARG;
  if (!(p->min_depth >= 0) || !(p->max_depth > p->min_depth)) return VH_ERR_INVALID_ARG;
  if (!(p->depth_scale > 0) || !(p->voxel_size > 0) || !(p->trunc > 0)) return VH_ERR_INVALID_ARG;
  if (p->table_log2 < 8 || p->table_log2 > 31) return VH_ERR_INVALID_ARG;
  if (p->max_probe < 1 || (int64_t)p->max_probe > (1ll << p->table_log2)) return VH_ERR_INVALID_ARG;
  if (p->pool_blocks < 1 || p->pool_blocks > 0x7FFFFFFF) return VH_ERR_INVALID_ARG;
  if (p->max_frame_blocks < 1 || p->max_frame_blocks > 0x7FFFFFFF) return VH_ERR_INVALID_ARG;
  if (p->max_triangles < 0 || p->max_triangles > 0x7FFFFFFF / 3) return VH_ERR_INVALID_ARG;
  if (p->device < 0) return VH_ERR_INVALID_ARG;
  if (p->flags &
      ~(uint32_t)(VH_FLAG_SYNC | VH_FLAG_NO_GRAPH | VH_FLAG_PROFILE | VH_FLAG_DEPTH_FILTER |
                  VH_FLAG_BATCH_FUSED))
    return VH_ERR_INVALID_ARG;
  return VH_OK;
}

vh_status vh_create(const vh_params *p, vh_handle **out) {
  if (!out) return VH_ERR_INVALID_ARG;
  *out = nullptr;
  vh_status vs = vh_params_validate(p);
  if (vs != VH_OK) {
    vh::log_error(std::string("vh_create: invalid parameters (") + vh_status_string(vs) + ")");
    return vs;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    vh::log_error("vh_create: no CUDA device");
    return VH_ERR_NO_DEVICE;
  }
  if (p->device >= ndev) {
    vh::log_error("vh_create: device index " + std::to_string(p->device) + " out of range (" +
              std::to_string(ndev) + " devices)");
    return VH_ERR_INVALID_ARG;
  }
  DeviceScope on_device(p->device);  // the caller's current device is restored
  if (!on_device.ok()) return VH_ERR_CUDA;
  vh_handle *h = new vh_handle();
  h->p = *p;
  auto bail = [&](vh_status s) {
    free_all(h);
    delete h;
    return s;
  };
  if (cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess)
    return bail(VH_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(VH_ERR_CUDA);
  h->stream = h->own_stream;
  apply_tuning(h, vh_tuning{});
  const size_t slots = (size_t)1 << p->table_log2;
  const size_t npx = (size_t)p->width * p->height;
  h->tri_cap = p->max_triangles;
  bool ok = cudaMalloc(&h->V.slots, sizeof(Slot) * slots) == cudaSuccess &&
            cudaMalloc(&h->V.pool, sizeof(float) * kBlockWords * (size_t)p->pool_blocks) == cudaSuccess &&
            cudaMalloc(&h->V.block_keys, sizeof(unsigned long long) * p->pool_blocks) == cudaSuccess &&
            cudaMalloc(&h->V.free_list, sizeof(uint32_t) * p->pool_blocks) == cudaSuccess &&
            cudaMalloc(&h->V.frame_list, sizeof(uint32_t) * p->max_frame_blocks) == cudaSuccess &&
            cudaMalloc(&h->V.frame_nb, 8 * sizeof(uint32_t) * p->max_frame_blocks) == cudaSuccess &&
            cudaMalloc(&h->V.frame_res, sizeof(ulonglong2) * p->max_frame_blocks) == cudaSuccess &&
            cudaMalloc(&h->V.st, sizeof(DevState)) == cudaSuccess &&
            cudaMalloc(&h->d_depth, 4 * npx) == cudaSuccess &&
            cudaMalloc(&h->d_depth_f, 4 * npx) == cudaSuccess &&
            cudaMalloc(&h->d_rgb, 3 * npx) == cudaSuccess &&
            cudaMalloc(&h->d_fin, sizeof(FrameIn)) == cudaSuccess &&
            cudaMalloc(&h->d_in_depth[0], 4 * npx) == cudaSuccess &&
            cudaMalloc(&h->d_in_depth[1], 4 * npx) == cudaSuccess &&
            cudaMalloc(&h->d_in_rgb[0], 3 * npx) == cudaSuccess &&
            cudaMalloc(&h->d_in_rgb[1], 3 * npx) == cudaSuccess &&
            cudaMalloc(&h->d_pix, sizeof(uint2) * npx) == cudaSuccess &&
            cudaMalloc(&h->d_rcp, sizeof(float) * (kRcpMax + 1)) == cudaSuccess &&
            cudaMalloc(&h->d_tris, sizeof(float4) * 3 * (size_t)(h->tri_cap ? h->tri_cap : 1)) == cudaSuccess &&
            cudaHostAlloc(&h->h_state, sizeof(DevState), cudaHostAllocMapped) == cudaSuccess &&
            cudaHostGetDevicePointer(&h->h_state_dev, h->h_state, 0) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    vh::log_error("vh_create: device allocation failed");
    return bail(VH_ERR_CUDA);
  }
  for (int k = 0; k < 2; ++k)
    if (cudaEventCreateWithFlags(&h->in_copied[k], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->in_consumed[k], cudaEventDisableTiming) != cudaSuccess)
      return bail(VH_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(VH_ERR_CUDA);
  for (auto &e : h->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return bail(VH_ERR_CUDA);
  h->V.slot_mask = (uint32_t)(slots - 1);
  h->V.max_probe = p->max_probe;
  h->V.frame_cap = (uint32_t)p->max_frame_blocks;
  h->V.pool_cap = (uint32_t)p->pool_blocks;
  h->C.width = p->width;
  h->C.height = p->height;
  h->C.wf = (float)p->width;
  h->C.hf = (float)p->height;
  h->C.fx = p->fx;
  h->C.fy = p->fy;
  h->C.cx = p->cx;
  h->C.cy = p->cy;
  h->C.min_depth = p->min_depth;
  h->C.max_depth = p->max_depth;
  h->C.depth_scale = p->depth_scale;
  h->C.voxel = p->voxel_size;
  h->C.trunc = p->trunc;
  h->C.mc_min_weight = p->mc_min_weight;
  h->C.rtrunc = rn_reciprocal(p->trunc);
  launch_rcp_table(h->d_rcp, h->stream);
  h->C.rcp_w = h->d_rcp;
  vs = clear_volume(h, false);
  if (vs != VH_OK) return bail(vs);
  *out = h;
  return VH_OK;
}

vh_status vh_destroy(vh_handle *h) {
  VH_HANDLE_DEVICE(h);
  if (!h) return VH_ERR_INVALID_ARG;
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_all(h);
  delete h;
  return VH_OK;
}

vh_status vh_reset(vh_handle *h) {
  VH_HANDLE_DEVICE(h);
  if (!h) return VH_ERR_INVALID_ARG;
  return clear_volume(h, true);
}

vh_status vh_set_stream(vh_handle *h, void *stream) {
  VH_HANDLE_DEVICE(h);
  if (!h) return VH_ERR_INVALID_ARG;
  VH_CUDA(h, cudaStreamSynchronize(h->stream));
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return VH_OK;
}

vh_status vh_sync(vh_handle *h) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_sync");
  if (!h) return VH_ERR_INVALID_ARG;
  vh_status s = mesh_drain(h);
  vh_status t = sync_and_check(h);
  vh_status e = stream_store_settle(h);
  return s != VH_OK ? s : (t != VH_OK ? t : e);
}

const char *vh_last_error(const vh_handle *h) { return h ? h->last_error.c_str() : "null handle"; }

vh_status vh_integrate(vh_handle *h, const void *depth, int32_t depth_fmt, const uint8_t *rgb,
                       const float *c2w, int32_t mem) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_integrate");
  if (!h) return VH_ERR_INVALID_ARG;
  vh_status s = stage_inputs(h, depth, depth_fmt, rgb, c2w, mem);
  if (s != VH_OK) return s;
  s = run_frame(h, depth_fmt, kMcNone);
  if (s != VH_OK) return s;
  h->frames++;
  h->nb_valid = true;
  return (h->p.flags & VH_FLAG_SYNC) ? sync_and_check(h) : VH_OK;
}

vh_status vh_extract(vh_handle *h, int32_t scope, vh_mesh_view *out) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_extract");
  if (!h) return VH_ERR_INVALID_ARG;
  if (scope != VH_SCOPE_FRAME && scope != VH_SCOPE_ALL)
    return fail(h, VH_ERR_INVALID_ARG, "unknown extraction scope");
  if (scope == VH_SCOPE_FRAME && !h->nb_valid) {
    launch_frame_nb(h->V, h->stream);
    h->nb_valid = true;
  }
  for (int attempt = 0; attempt < 2; ++attempt) {
    launch_mc_begin(h->V, h->stream);
    launch_mc(h->V, scope == VH_SCOPE_ALL, h->C.mc_min_weight, h->d_tris, (uint32_t)h->tri_cap,
              mc_grid(h), h->tuning.mc_variant, nullptr, h->stream);
    VH_CUDA(h, cudaGetLastError());
    h->ev_pending = false;
    if (scope == VH_SCOPE_FRAME && !out && !(h->p.flags & VH_FLAG_SYNC)) return VH_OK;
    vh_status s = pull_state(h);
    if (s != VH_OK) return s;
    const int64_t need = h->h_state->tri_count;
    if (need > h->tri_cap && attempt == 0) {
      // too many triangles: clear the overflow bit, grow and extract again
      VH_CUDA(h, cudaMemsetAsync(&h->V.st->error, 0, sizeof(uint32_t), h->stream));
      s = grow_tris(h, need);
      if (s != VH_OK) return s;
      continue;
    }
    break;
  }
  vh_status s = sync_and_check(h);
  if (out) {
    out->vertices = (const float *)h->d_tris;
    out->num_triangles = std::min<int64_t>(h->h_state->tri_count, h->tri_cap);
    out->voxel_size = h->p.voxel_size;
  }
  return s;
}

vh_status vh_process_frame(vh_handle *h, const void *depth, int32_t depth_fmt, const uint8_t *rgb,
                           const float *c2w, int32_t mem, vh_mesh_view *out) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_process_frame");
  if (!h) return VH_ERR_INVALID_ARG;
  vh_status s = stage_inputs(h, depth, depth_fmt, rgb, c2w, mem);
  if (s != VH_OK) return s;
  s = run_frame(h, depth_fmt, kMcMain);
  if (s != VH_OK) return s;
  h->frames++;
  h->nb_valid = true;
  if (!(h->p.flags & VH_FLAG_SYNC) && !out) return VH_OK;
  s = sync_and_check(h);
  if (out) {
    out->vertices = (const float *)h->d_tris;
    out->num_triangles = std::min<int64_t>(h->h_state->tri_count, h->tri_cap);
    out->voxel_size = h->p.voxel_size;
  }
  return s;
}

vh_status vh_process_frame_mesh(vh_handle *h, const void *depth, int32_t depth_fmt,
                                const uint8_t *rgb, const float *c2w, int32_t mem, float *tris,
                                int64_t capacity, int64_t *num_triangles) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_process_frame_mesh");
  if (!h) return VH_ERR_INVALID_ARG;
  if (capacity < 0 || (capacity > 0 && !tris) || !num_triangles)
    return fail(h, VH_ERR_INVALID_ARG, "mesh output: null buffer or negative capacity");
  vh_status s = stage_inputs(h, depth, depth_fmt, rgb, c2w, mem);
  if (s != VH_OK) return s;
  if (h->p.flags & VH_FLAG_SYNC) {  // the reference's blocking order
    s = run_frame(h, depth_fmt, kMcMain);
    if (s != VH_OK) return s;
    h->frames++;
    h->nb_valid = true;
    s = sync_and_check(h);
    const int64_t n = std::min<int64_t>(h->h_state->tri_count, h->tri_cap);
    *num_triangles = h->h_state->tri_count;
    const int64_t m = std::min(n, capacity);
    if (m > 0)
      VH_CUDA(h, cudaMemcpy(tris, h->d_tris, sizeof(float4) * 3 * (size_t)m,
                            cudaMemcpyDeviceToHost));
    if (s != VH_OK) return s;
    if (n > capacity) return fail(h, VH_ERR_CAPACITY, "the frame's mesh is larger than its buffer");
    return VH_OK;
  }
  s = mesh_setup(h, false);
  if (s != VH_OK) return s;
  const int k = h->mesh_slot;
  // slot k's buffer was last read by the copy-out of the frame two back
  if (h->mesh_copy_issued[k]) VH_CUDA(h, cudaStreamWaitEvent(h->stream, h->mesh_copied[k], 0));
  s = run_frame(h, depth_fmt, kMcSlot0 + k);
  if (s != VH_OK) return s;
  h->frames++;
  h->nb_valid = true;
  VH_CUDA(h, cudaEventRecord(h->mesh_done[k], h->stream));
  // this frame is queued behind the pending one: copy that one out now
  s = mesh_flush(h);
  h->pending = vh_handle::PendingMesh{};
  h->pending.valid = true;
  h->pending.slot = k;
  h->pending.tris = tris;
  h->pending.capacity = capacity;
  h->pending.count = num_triangles;
  h->mesh_slot = k ^ 1;
  return s;
}

vh_status vh_process_frame_indexed(vh_handle *h, const void *depth, int32_t depth_fmt,
                                   const uint8_t *rgb, const float *c2w, int32_t mem,
                                   float *vertices, int64_t vertex_capacity, int32_t *faces,
                                   int64_t face_capacity, int64_t *num_vertices,
                                   int64_t *num_faces) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_process_frame_indexed");
  if (!h) return VH_ERR_INVALID_ARG;
  if (vertex_capacity < 0 || face_capacity < 0 || (vertex_capacity > 0 && !vertices) ||
      (face_capacity > 0 && !faces) || !num_vertices || !num_faces)
    return fail(h, VH_ERR_INVALID_ARG, "indexed mesh output: null buffer or negative capacity");
  vh_status s = stage_inputs(h, depth, depth_fmt, rgb, c2w, mem);
  if (s != VH_OK) return s;
  s = mesh_setup(h, true);
  if (s != VH_OK) return s;
  if (h->p.flags & VH_FLAG_SYNC) {  // the reference's blocking order, slot 0
    if (h->mesh_copy_issued[0]) VH_CUDA(h, cudaStreamWaitEvent(h->stream, h->mesh_copied[0], 0));
    s = run_frame(h, depth_fmt, kMcIdx0);
    if (s != VH_OK) return s;
    h->frames++;
    h->nb_valid = true;
    s = sync_and_check(h);
    const int64_t nf = h->h_state->tri_count, nv = h->h_state->vert_count;
    *num_faces = nf;
    *num_vertices = nv;
    const int64_t mf = std::min(std::min(nf, face_capacity), h->midx_cap);
    const int64_t mv = std::min(std::min(nv, vertex_capacity), h->midx_cap);
    if (mv > 0)
      VH_CUDA(h, cudaMemcpy(vertices, h->d_mverts[0], sizeof(float4) * (size_t)mv,
                            cudaMemcpyDeviceToHost));
    if (mf > 0)
      VH_CUDA(h, cudaMemcpy(faces, h->d_mfaces[0], 3 * sizeof(int32_t) * (size_t)mf,
                            cudaMemcpyDeviceToHost));
    if (s != VH_OK) return s;
    if (nf > face_capacity || nv > vertex_capacity)
      return fail(h, VH_ERR_CAPACITY, "the frame's mesh is larger than its buffers");
    return VH_OK;
  }
  const int k = h->mesh_slot;
  // slot k's buffers were last read by the copy-out of the frame two back
  if (h->mesh_copy_issued[k]) VH_CUDA(h, cudaStreamWaitEvent(h->stream, h->mesh_copied[k], 0));
  s = run_frame(h, depth_fmt, kMcIdx0 + k);
  if (s != VH_OK) return s;
  h->frames++;
  h->nb_valid = true;
  VH_CUDA(h, cudaEventRecord(h->mesh_done[k], h->stream));
  s = mesh_flush(h);  // this frame is queued behind the pending one
  h->pending = vh_handle::PendingMesh{};
  h->pending.valid = true;
  h->pending.indexed = true;
  h->pending.slot = k;
  h->pending.tris = reinterpret_cast<float *>(faces);
  h->pending.capacity = face_capacity;
  h->pending.count = num_faces;
  h->pending.verts = vertices;
  h->pending.vcapacity = vertex_capacity;
  h->pending.vcount = num_vertices;
  h->mesh_slot = k ^ 1;
  return s;
}

vh_status vh_copy_mesh(vh_handle *h, float *xyz, uint8_t *rgb, int64_t capacity,
                       int64_t *num_triangles) {
  VH_HANDLE_DEVICE(h);
  if (!h || capacity < 0) return VH_ERR_INVALID_ARG;
  vh_status s = pull_state(h);
  if (s != VH_OK) return s;
  const int64_t n = std::min<int64_t>(h->h_state->tri_count, h->tri_cap);
  if (num_triangles) *num_triangles = n;
  const int64_t m = std::min(n, capacity);
  if (m > 0 && (xyz || rgb)) {
    std::vector<float> buf((size_t)m * 12);
    VH_CUDA(h, cudaMemcpy(buf.data(), h->d_tris, sizeof(float) * 12 * (size_t)m, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < 3 * m; ++i) {
      const float *v = &buf[4 * (size_t)i];
      if (xyz) {
        xyz[3 * i] = v[0];
        xyz[3 * i + 1] = v[1];
        xyz[3 * i + 2] = v[2];
      }
      if (rgb) {
        uint32_t c;
        std::memcpy(&c, &v[3], 4);
        rgb[3 * i] = (uint8_t)(c & 0xFF);
        rgb[3 * i + 1] = (uint8_t)((c >> 8) & 0xFF);
        rgb[3 * i + 2] = (uint8_t)((c >> 16) & 0xFF);
      }
    }
  }
  if (m < n && (xyz || rgb)) return fail(h, VH_ERR_CAPACITY, "mesh larger than the output capacity");
  return VH_OK;
}

// Full-volume extraction, then the GPU indexing of its triangle soup.
static vh_status indexed_mesh(vh_handle *h, std::vector<float> &vert, std::vector<uint8_t> &col,
                              std::vector<int32_t> &faces) {
  vh_status s = vh_extract(h, VH_SCOPE_ALL, nullptr);
  if (s != VH_OK) return s;
  const int64_t n = std::min<int64_t>(h->h_state->tri_count, h->tri_cap);
  return index_mesh(h, h->d_tris, n, h->p.voxel_size, vert, col, faces);
}

vh_status vh_save_ply(vh_handle *h, const char *path, int32_t binary) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_save_ply");
  if (!h || !path) return VH_ERR_INVALID_ARG;
  std::vector<float> vert;
  std::vector<uint8_t> col;
  std::vector<int32_t> faces;
  vh_status s = indexed_mesh(h, vert, col, faces);
  if (s != VH_OK) return s;
  if (!write_ply(path, vert, col, faces, binary != 0))
    return fail(h, VH_ERR_IO, std::string("cannot write ") + path);
  return VH_OK;
}

vh_status vh_mesh_indexed(vh_handle *h, float *vertices, uint8_t *colors, int64_t vertex_capacity,
                          int32_t *faces, int64_t face_capacity, int64_t *num_vertices,
                          int64_t *num_faces) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_mesh_indexed");
  if (!h || vertex_capacity < 0 || face_capacity < 0) return VH_ERR_INVALID_ARG;
  std::vector<float> vert;
  std::vector<uint8_t> col;
  std::vector<int32_t> fc;
  vh_status s = indexed_mesh(h, vert, col, fc);
  if (s != VH_OK) return s;
  const int64_t nv = (int64_t)(vert.size() / 3), nf = (int64_t)(fc.size() / 3);
  if (num_vertices) *num_vertices = nv;
  if (num_faces) *num_faces = nf;
  const bool want = vertices || colors || faces;
  if (!want) return VH_OK;
  if (nv > vertex_capacity || nf > face_capacity)
    return fail(h, VH_ERR_CAPACITY, "mesh larger than the output capacity");
  if (vertices && nv) std::memcpy(vertices, vert.data(), sizeof(float) * 3 * (size_t)nv);
  if (colors && nv) std::memcpy(colors, col.data(), 3 * (size_t)nv);
  if (faces && nf) std::memcpy(faces, fc.data(), sizeof(int32_t) * 3 * (size_t)nf);
  return VH_OK;
}

vh_status vh_filter_depth(vh_handle *h, const void *depth, int32_t depth_fmt, float *out,
                          int32_t mem) {
  VH_HANDLE_DEVICE(h);
  if (!h || !out) return VH_ERR_INVALID_ARG;
  const void *d = nullptr;
  vh_status s = handle_stage_depth(h, depth, depth_fmt, mem, &d);
  if (s != VH_OK) return s;
  float *dst = mem == VH_MEM_DEVICE ? out : h->d_depth_f;
  launch_depth_filter(h->C, d, nullptr, depth_fmt, dst, h->stream);
  VH_CUDA(h, cudaGetLastError());
  if (mem == VH_MEM_HOST)
    VH_CUDA(h, cudaMemcpyAsync(out, dst, sizeof(float) * (size_t)h->p.width * h->p.height,
                               cudaMemcpyDeviceToHost, h->stream));
  return sync_and_check(h);
}

vh_status vh_render(vh_handle *h) {
  return fail(h, VH_ERR_UNSUPPORTED, "render() needs OpenGL, which is not available");
}

vh_status vh_alloc_keys(vh_handle *h, const int32_t *xyz, int64_t n, int32_t mem) {
  VH_HANDLE_DEVICE(h);
  if (h) h->nb_valid = false;
  if (!h || n < 0 || (n && !xyz) || n > 0x7FFFFFFF / 3) return VH_ERR_INVALID_ARG;
  if (!n) return VH_OK;
  DevBuf<int32_t> tmp;
  const int32_t *d = nullptr;
  vh_status s = device_view(h, xyz, 3 * (size_t)n, mem, tmp, &d);
  if (s != VH_OK) return s;
  launch_epoch_end(h->V, h->stream);
  launch_alloc_keys(h->V, d, (uint32_t)n, h->stream);
  launch_epoch_end(h->V, h->stream);
  VH_CUDA(h, cudaGetLastError());
  return sync_and_check(h);
}

vh_status vh_find_keys(vh_handle *h, const int32_t *xyz, int64_t n, int32_t *out_block,
                       int32_t mem) {
  VH_HANDLE_DEVICE(h);
  if (!h || n < 0 || (n && (!xyz || !out_block)) || n > 0x7FFFFFFF / 3) return VH_ERR_INVALID_ARG;
  if (!n) return VH_OK;
  DevBuf<int32_t> tmp, res;
  const int32_t *d = nullptr;
  vh_status s = device_view(h, xyz, 3 * (size_t)n, mem, tmp, &d);
  if (s != VH_OK) return s;
  int32_t *dout = out_block;
  if (mem == VH_MEM_HOST) {
    VH_CUDA(h, cudaMalloc(&res.ptr, sizeof(int32_t) * n));
    dout = res.ptr;
  }
  launch_find_keys(h->V, d, (uint32_t)n, dout, h->stream);
  VH_CUDA(h, cudaGetLastError());
  if (mem == VH_MEM_HOST)
    VH_CUDA(h, cudaMemcpyAsync(out_block, dout, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, h->stream));
  return sync_and_check(h);
}

vh_status vh_erase_keys(vh_handle *h, const int32_t *xyz, int64_t n, int64_t *num_erased,
                        int32_t mem) {
  VH_HANDLE_DEVICE(h);
  if (h) h->nb_valid = false;
  if (!h || n < 0 || (n && !xyz) || n > 0x7FFFFFFF / 3) return VH_ERR_INVALID_ARG;
  if (num_erased) *num_erased = 0;
  if (!n) return VH_OK;
  DevBuf<int32_t> tmp;
  const int32_t *d = nullptr;
  vh_status s = device_view(h, xyz, 3 * (size_t)n, mem, tmp, &d);
  if (s != VH_OK) return s;
  launch_epoch_end(h->V, h->stream);
  VH_CUDA(h, cudaMemsetAsync(&h->V.st->erased, 0, sizeof(uint32_t), h->stream));
  launch_erase_keys(h->V, d, (uint32_t)n, h->stream);
  VH_CUDA(h, cudaGetLastError());
  s = sync_and_check(h);
  if (num_erased) *num_erased = h->h_state->erased;
  return s;
}

vh_status vh_clear_block_list(vh_handle *h) {
  VH_HANDLE_DEVICE(h);
  if (h) h->nb_valid = false;
  if (!h) return VH_ERR_INVALID_ARG;
  launch_clear_list(h->V, h->stream);
  VH_CUDA(h, cudaGetLastError());
  return (h->p.flags & VH_FLAG_SYNC) ? sync_and_check(h) : VH_OK;
}

vh_status vh_block_list(vh_handle *h, int32_t *xyz, int64_t capacity, int64_t *n) {
  VH_HANDLE_DEVICE(h);
  if (!h || capacity < 0) return VH_ERR_INVALID_ARG;
  vh_status s = pull_state(h);
  if (s != VH_OK) return s;
  const int64_t cnt = std::min<int64_t>(h->h_state->frame_count, h->p.max_frame_blocks);
  if (n) *n = cnt;
  const int64_t m = std::min(cnt, capacity);
  if (m > 0 && xyz) {
    DevBuf<int32_t> tmp;
    VH_CUDA(h, cudaMalloc(&tmp.ptr, sizeof(int32_t) * 3 * m));
    launch_list_keys(h->V, tmp.ptr, (uint32_t)m, h->stream);
    VH_CUDA(h, cudaGetLastError());
    VH_CUDA(h, cudaMemcpyAsync(xyz, tmp.ptr, sizeof(int32_t) * 3 * m, cudaMemcpyDeviceToHost, h->stream));
    VH_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  if (m < cnt && xyz) return fail(h, VH_ERR_CAPACITY, "block list larger than the output capacity");
  return VH_OK;
}

uint64_t vh_block_hash_ref(int32_t x, int32_t y, int32_t z) { return ref_block_hash(x, y, z); }

vh_status vh_get_device_table(vh_handle *h, vh_device_table *out) {
  if (!h || !out) return VH_ERR_INVALID_ARG;
  static_assert(sizeof(Slot) == 16 && kBlockWords == 3 * VH_BLOCK_VOXELS, "published layout");
  std::memset(out, 0, sizeof(*out));
  out->layout = VH_DEVICE_TABLE_LAYOUT;
  out->slot_mask = h->V.slot_mask;
  out->max_probe = h->V.max_probe;
  out->key_bias = kKeyBias;
  out->slots = h->V.slots;
  out->pool = h->V.pool;
  out->block_keys = reinterpret_cast<const uint64_t *>(h->V.block_keys);
  out->pool_top = &h->V.st->pool_top;
  out->pool_capacity = h->V.pool_cap;
  out->voxel_size = h->p.voxel_size;
  out->device = h->p.device;
  out->stream = h->stream;
  return VH_OK;
}

vh_status vh_mc_tables(int32_t *corner, int32_t *edge_mask, int32_t *tri) {
  for (int k = 0; corner && k < 8; ++k)
    for (int a = 0; a < 3; ++a) corner[3 * k + a] = kMcCorner[k][a];
  for (int i = 0; edge_mask && i < 256; ++i) edge_mask[i] = kMcEdgeMask[i];
  for (int i = 0; tri && i < 256; ++i)
    for (int j = 0; j < 16; ++j) tri[16 * i + j] = kMcTri[i][j];
  return VH_OK;
}

vh_status vh_export_blocks(vh_handle *h, int32_t *xyz, float *sdf, float *weight, uint8_t *rgb,
                           int64_t capacity, int64_t *n) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_export_blocks");
  if (!h || capacity < 0) return VH_ERR_INVALID_ARG;
  launch_epoch_end(h->V, h->stream);
  vh_status s = pull_state(h);
  if (s != VH_OK) return s;
  const uint32_t top = h->h_state->pool_top;
  std::vector<unsigned long long> keys(top);
  if (top)
    VH_CUDA(h, cudaMemcpy(keys.data(), h->V.block_keys, sizeof(unsigned long long) * top,
                          cudaMemcpyDeviceToHost));
  int64_t live = 0;
  for (uint32_t b = 0; b < top; ++b) live += keys[b] < kTombKey;
  if (n) *n = live;
  const bool want_data = sdf || weight || rgb;
  const uint32_t chunk = 8192;
  std::vector<float> buf;
  int64_t o = 0;
  for (uint32_t b0 = 0; b0 < top && o < capacity; b0 += chunk) {
    const uint32_t cnt = std::min(chunk, top - b0);
    if (want_data) {
      buf.resize((size_t)cnt * kBlockWords);
      VH_CUDA(h, cudaMemcpy(buf.data(), h->V.pool + (size_t)b0 * kBlockWords,
                            sizeof(float) * kBlockWords * cnt, cudaMemcpyDeviceToHost));
    }
    for (uint32_t j = 0; j < cnt && o < capacity; ++j) {
      const unsigned long long k = keys[b0 + j];
      if (k >= kTombKey) continue;
      int x, y, z;
      unpack_key(k, x, y, z);
      if (xyz) {
        xyz[3 * o] = x;
        xyz[3 * o + 1] = y;
        xyz[3 * o + 2] = z;
      }
      const float *blk = want_data ? &buf[(size_t)j * kBlockWords] : nullptr;
      if (sdf) std::memcpy(sdf + (size_t)o * kB3, blk, sizeof(float) * kB3);
      if (weight) std::memcpy(weight + (size_t)o * kB3, blk + kB3, sizeof(float) * kB3);
      if (rgb) {
        const uint32_t *c = reinterpret_cast<const uint32_t *>(blk + 2 * kB3);
        uint8_t *dst = rgb + (size_t)o * kB3 * 3;
        for (int v = 0; v < kB3; ++v) {
          dst[3 * v] = (uint8_t)(c[v] & 0xFF);
          dst[3 * v + 1] = (uint8_t)((c[v] >> 8) & 0xFF);
          dst[3 * v + 2] = (uint8_t)((c[v] >> 16) & 0xFF);
        }
      }
      ++o;
    }
  }
  if (o < live && (xyz || want_data))
    return fail(h, VH_ERR_CAPACITY, "volume larger than the output capacity");
  return VH_OK;
}

// Host-side checks of a block set before anything on the device changes.
// Weights are observation counts: integration adds 1 per update, and its
// exact colour average relies on whole weights.  Keys must lie in the key
// range; `replace`: the set will replace the volume, so it must fit the pool.
static vh_status check_blocks(vh_handle *h, const int32_t *xyz, const float *weight, int64_t n,
                              bool replace) {
  for (size_t i = 0, m = (size_t)n * kB3; i < m; ++i)
    if (!(weight[i] >= 0.0f && weight[i] <= 16777216.0f && weight[i] == std::floor(weight[i])))
      return fail(h, VH_ERR_INVALID_ARG, "block weights must be whole numbers in [0, 2^24]");
  for (int64_t i = 0; i < n; ++i)
    if (!key_in_range(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]))
      return fail(h, VH_ERR_OUT_OF_RANGE, "a block coordinate lies outside [-2^20, 2^20)");
  if (replace && n > h->p.pool_blocks)
    return fail(h, VH_ERR_POOL_FULL, "more blocks than the pool holds (raise pool_blocks)");
  return VH_OK;
}

vh_status vh_import_blocks(vh_handle *h, const int32_t *xyz, const float *sdf, const float *weight,
                           const uint8_t *rgb, int64_t n) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_import_blocks");
  if (h) h->nb_valid = false;
  if (!h || n < 0 || (n && (!xyz || !sdf || !weight || !rgb)) || n > (1ll << 24))
    return VH_ERR_INVALID_ARG;
  if (!n) return VH_OK;
  vh_status cs = check_blocks(h, xyz, weight, n, false);
  if (cs != VH_OK) return cs;
  DevBuf<int32_t> dk;
  DevBuf<float> ds, dw;
  DevBuf<uint8_t> dc;
  const int32_t *k = nullptr;
  const float *s_ = nullptr, *w_ = nullptr;
  const uint8_t *c_ = nullptr;
  vh_status s;
  if ((s = device_view(h, xyz, 3 * (size_t)n, VH_MEM_HOST, dk, &k)) != VH_OK) return s;
  if ((s = device_view(h, sdf, (size_t)n * kB3, VH_MEM_HOST, ds, &s_)) != VH_OK) return s;
  if ((s = device_view(h, weight, (size_t)n * kB3, VH_MEM_HOST, dw, &w_)) != VH_OK) return s;
  if ((s = device_view(h, rgb, (size_t)n * kB3 * 3, VH_MEM_HOST, dc, &c_)) != VH_OK) return s;
  launch_epoch_end(h->V, h->stream);
  launch_alloc_keys(h->V, k, (uint32_t)n, h->stream);
  launch_epoch_end(h->V, h->stream);
  launch_scatter_blocks(h->V, k, s_, w_, c_, (uint32_t)n, h->stream);
  VH_CUDA(h, cudaGetLastError());
  return sync_and_check(h);
}

vh_status vh_save(vh_handle *h, const char *path) {
  VH_HANDLE_DEVICE(h);
  if (!h || !path) return VH_ERR_INVALID_ARG;
  int64_t n = 0;
  vh_status s = vh_export_blocks(h, nullptr, nullptr, nullptr, nullptr, 0, &n);
  if (s != VH_OK && s != VH_ERR_CAPACITY) return s;
  std::vector<int32_t> xyz(3 * (size_t)n);
  std::vector<float> sdf((size_t)n * kB3), w((size_t)n * kB3);
  std::vector<uint8_t> rgb((size_t)n * kB3 * 3);
  s = vh_export_blocks(h, xyz.data(), sdf.data(), w.data(), rgb.data(), n, &n);
  if (s != VH_OK) return s;
  if (!write_snapshot(path, h->p.voxel_size, h->p.trunc, xyz.data(), sdf.data(), w.data(),
                      rgb.data(), n))
    return fail(h, VH_ERR_IO, std::string("cannot write ") + path);
  return VH_OK;
}

vh_status vh_load(vh_handle *h, const char *path) {
  VH_HANDLE_DEVICE(h);
  if (!h || !path) return VH_ERR_INVALID_ARG;
  std::vector<int32_t> xyz;
  std::vector<float> sdf, w;
  std::vector<uint8_t> rgb;
  float voxel = 0, trunc = 0;
  if (!read_snapshot(path, &voxel, &trunc, xyz, sdf, w, rgb))
    return fail(h, VH_ERR_IO, std::string("cannot read snapshot ") + path);
  if (voxel != h->p.voxel_size)
    return fail(h, VH_ERR_INVALID_ARG, "snapshot voxel size differs from the handle's");
  const int64_t n = (int64_t)xyz.size() / 3;
  // Everything the import would reject is rejected before the volume is
  // cleared, so a bad snapshot leaves the caller's volume unchanged.
  if (n > (1ll << 24)) return fail(h, VH_ERR_INVALID_ARG, "snapshot holds more than 2^24 blocks");
  vh_status s = check_blocks(h, xyz.data(), w.data(), n, true);
  if (s != VH_OK) return s;
  s = clear_volume(h, true);
  if (s != VH_OK) return s;
  s = vh_import_blocks(h, xyz.data(), sdf.data(), w.data(), rgb.data(), n);
  if (s != VH_OK) return s;
  return vh_clear_block_list(h);
}

vh_status vh_get_stats(vh_handle *h, vh_stats *out) {
  VH_HANDLE_DEVICE(h);
  if (!h || !out) return VH_ERR_INVALID_ARG;
  launch_epoch_end(h->V, h->stream);
  vh_status s = sync_and_check(h);
  const DevState &d = *h->h_state;
  std::memset(out, 0, sizeof(*out));
  out->frames = h->frames;
  out->blocks_allocated = (int64_t)d.pool_top - (int64_t)d.free_count;
  out->frame_blocks = std::min<int64_t>(d.frame_count, h->p.max_frame_blocks);
  out->new_blocks = d.new_blocks;
  out->voxels_updated = (int64_t)d.voxels_updated;
  out->triangles = d.tri_count;
  out->pool_capacity = h->p.pool_blocks;
  out->table_slots = (int64_t)h->V.slot_mask + 1;
  out->tombstones = d.tombstones;
  out->device_error = d.error;
  out->frame_kernels = (uint32_t)h->frame_kernels;
  out->ms_allocate = h->stage.ms_allocate;
  out->ms_integrate = h->stage.ms_integrate;
  out->ms_extract = h->stage.ms_extract;
  out->ms_frame = h->stage.ms_frame;
  return s;
}

void vh_set_log_callback(vh_log_fn fn, void *user) { vh::set_log(fn, user); }

void vh_tuning_variants(int32_t *integrate, int32_t *mc) {
  if (integrate) *integrate = integrate_variants();
  if (mc) *mc = mc_variants();
}

vh_status vh_get_tuning(vh_handle *h, vh_tuning *out) {
  if (!h || !out) return VH_ERR_INVALID_ARG;
  *out = h->tuning;
  return VH_OK;
}

vh_status vh_set_tuning(vh_handle *h, const vh_tuning *t) {
  VH_HANDLE_DEVICE(h);
  if (!h || !t || t->integrate_variant < 0 || t->integrate_variant >= integrate_variants() ||
      t->mc_variant < 0 || t->mc_variant >= mc_variants() || t->integrate_ctas_per_sm < 0 ||
      t->mc_ctas_per_sm < 0)
    return VH_ERR_INVALID_ARG;
  VH_CUDA(h, cudaStreamSynchronize(h->stream));
  apply_tuning(h, *t);
  return VH_OK;
}

}  // extern "C"

namespace {

std::mutex g_tune_mu;
std::map<std::string, vh_tuning> g_tune_cache;

std::string tune_key(const vh_handle *h) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, h->p.device) != cudaSuccess) std::strcpy(prop.name, "?");
  std::ostringstream k;
  k << prop.name << "|sm" << h->sm_count << "|" << h->p.width << "x" << h->p.height << "|v"
    << h->p.voxel_size << "|t" << h->p.trunc << "|d" << h->p.min_depth << "-" << h->p.max_depth
    << "|f" << h->p.fx << "|w" << h->p.mc_min_weight;
  std::string s = k.str();
  for (char &c : s)
    if (c == ' ' || c == '\t' || c == '\n') c = '_';
  return s;
}

bool cache_lookup(const std::string &key, vh_tuning *t) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tune_cache.find(key);
  if (it != g_tune_cache.end()) {
    *t = it->second;
    return true;
  }
  const char *path = std::getenv("VHSDF_TUNING_CACHE");
  if (!path) return false;
  std::ifstream f(path);
  std::string k;
  vh_tuning v{};
  while (f >> k >> v.integrate_variant >> v.integrate_ctas_per_sm >> v.mc_ctas_per_sm >>
         v.mc_variant) {
    if (k == key) {
      g_tune_cache[key] = v;
      *t = v;
      return true;
    }
  }
  return false;
}

void cache_store(const std::string &key, const vh_tuning &t) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune_cache[key] = t;
  const char *path = std::getenv("VHSDF_TUNING_CACHE");
  if (!path) return;
  std::ofstream f(path, std::ios::app);
  f << key << " " << t.integrate_variant << " " << t.integrate_ctas_per_sm << " "
    << t.mc_ctas_per_sm << " " << t.mc_variant << "\n";
}

float median(std::vector<float> v) {
  std::sort(v.begin(), v.end());
  return v.empty() ? 0.0f : v[v.size() / 2];
}

}  // namespace

extern "C" vh_status vh_autotune(vh_handle *h, const void *depth, int32_t depth_fmt,
                                 const uint8_t *rgb, const float *c2w, int32_t mem,
                                 vh_tuning *chosen) {
  VH_HANDLE_DEVICE(h);
  if (!h) return VH_ERR_INVALID_ARG;
  const std::string key = tune_key(h);
  vh_tuning best{};
  if (cache_lookup(key, &best)) {
    vh_status s = vh_set_tuning(h, &best);
    if (chosen) *chosen = h->tuning;
    return s;
  }
  vh_params sp = h->p;
  sp.flags = VH_FLAG_SYNC | VH_FLAG_PROFILE | VH_FLAG_NO_GRAPH;
  sp.pool_blocks = std::min<int64_t>(h->p.pool_blocks, h->p.max_frame_blocks + 4096);
  vh_handle *sc = nullptr;
  vh_status s = vh_create(&sp, &sc);
  if (s != VH_OK) return fail(h, s, "autotune: cannot create the scratch volume");
  // Medians of 9 frames; a shape replaces the best so far only when it is
  // more than 2 % faster, so timing noise leaves the default (tried first).
  const int reps = 9;
  const float margin = 0.98f;
  auto run = [&](const vh_tuning &t, float *ms_int, float *ms_mc) -> vh_status {
    apply_tuning(sc, t);
    std::vector<float> a, b;
    for (int r = 0; r < reps; ++r) {
      vh_status st = vh_process_frame(sc, depth, depth_fmt, rgb, c2w, mem, nullptr);
      if (st != VH_OK) return st;
      a.push_back(sc->stage.ms_integrate);
      b.push_back(sc->stage.ms_extract);
    }
    *ms_int = median(a);
    *ms_mc = median(b);
    return VH_OK;
  };
  float mi = 0, mm = 0;
  s = run(vh_tuning{}, &mi, &mm);  // also allocates the frame's blocks
  float best_int = 1e30f, best_mc = 1e30f;
  for (int variant = 0; variant < integrate_variants() && s == VH_OK; ++variant) {
    const int occ = integrate_ctas_per_sm(variant);
    const int opts[3] = {occ, std::max(1, occ * 3 / 4), std::max(1, occ / 2)};
    for (int o = 0; o < 3 && s == VH_OK; ++o) {
      if (o > 0 && opts[o] == opts[o - 1]) continue;
      vh_tuning t{};
      t.integrate_variant = variant;
      t.integrate_ctas_per_sm = opts[o];
      s = run(t, &mi, &mm);
      if (s == VH_OK && mi < best_int * margin) {
        best_int = mi;
        best.integrate_variant = variant;
        best.integrate_ctas_per_sm = opts[o];
      }
    }
  }
  for (int variant = 0; variant < mc_variants() && s == VH_OK; ++variant) {
    const int mocc = mc_ctas_per_sm(variant);
    const int mopts[3] = {mocc, std::max(1, mocc * 2 / 3), std::max(1, mocc / 2)};
    for (int o = 0; o < 3 && s == VH_OK; ++o) {
      if (o > 0 && mopts[o] == mopts[o - 1]) continue;
      vh_tuning t = best;
      t.mc_variant = variant;
      t.mc_ctas_per_sm = mopts[o];
      s = run(t, &mi, &mm);
      if (s == VH_OK && mm < best_mc * margin) {
        best_mc = mm;
        best.mc_variant = variant;
        best.mc_ctas_per_sm = mopts[o];
      }
    }
  }
  vh_destroy(sc);
  if (s != VH_OK) return fail(h, s, "autotune: a trial frame failed");
  cache_store(key, best);
  s = vh_set_tuning(h, &best);
  if (chosen) *chosen = h->tuning;
  return s;
}
