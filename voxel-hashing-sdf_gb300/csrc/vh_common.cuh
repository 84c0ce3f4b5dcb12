// vh_common.cuh - data layout and device helpers shared by the kernels and
// the host orchestration.
//
// HBM layout of one volume:
//   slots       2^k x 16 B  open-addressed hash: {u64 key, u32 block, u32 stamp}
//   pool        N x 6 KiB   voxel blocks; block b is sdf[512] | weight[512] |
//                           rgba8[512] (x-fastest voxel order x + 8y + 64z)
//   block_keys  N x 8 B     packed key of every pool block (EMPTY if free)
//   free_list   N x 4 B     recycled (already zeroed) block ids
//   frame_list  M x 4 B     slot ids touched by the current frame
//   frame_res   M x 16 B    {key, pool id} of each listed slot (one load instead
//                           of list -> slot)
//   frame_nb    M x 32 B    pool ids of each listed block and of its +x/+y/+z
//                           neighbours (written by integration, read by MC)
//   state       one DevState of counters and sticky error bits
//
// The reference keeps a bucketed, lock-protected table with overflow chains
// (include/vhashing.h:149-239,394-484) and rebuilds it every frame
// (src/tsdf.cu:1488,1492).  Here the table is resident and lock-free: a key
// is claimed with one 64-bit atomicCAS and probes are linear and bounded.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vh {

constexpr int kB = 8;          // voxels per block edge
constexpr int kB3 = 512;       // voxels per block
constexpr int kBlockWords = 3 * kB3;  // sdf, weight, rgba
constexpr int kKeyBias = 1 << 20;     // block coords in [-2^20, 2^20)
constexpr unsigned long long kEmptyKey = 0xFFFFFFFFFFFFFFFFull;
constexpr unsigned long long kTombKey = 0xFFFFFFFFFFFFFFFEull;
constexpr uint32_t kNoBlock = 0xFFFFFFFFu;
// |continuous block coordinate| bound that keeps every walked key in range
constexpr float kGridLimit = 1048000.0f;

// Device error bits (sticky until reported).
enum : uint32_t {
  kErrTableFull = 1u,
  kErrPoolFull = 2u,
  kErrRange = 4u,
  kErrFrameCap = 8u,
  kErrTriCap = 16u,
  kErrRetry = 32u,
  kErrCheck = 64u,  // a bounds check of the checked build failed
};

// Bounds checks of the checked build (compiled with -DVH_CHECKED): a failed
// check sets kErrCheck in the volume's error word and evaluates to false, so
// the caller skips the access instead of faulting.  In the normal build the
// condition is not evaluated and the macro is `true`.
#ifdef VH_CHECKED
#define VH_CHECK(st, cond) ((cond) || (atomicOr(&(st)->error, kErrCheck), false))
#else
#define VH_CHECK(st, cond) true
#endif

struct __align__(16) Slot {
  unsigned long long key;
  uint32_t block;
  uint32_t stamp;
};

struct DevState {
  uint32_t frame;        // stamp of the current block list (never 0 after begin)
  uint32_t frame_count;  // entries appended to frame_list (may exceed capacity)
  uint32_t pool_top;     // ids [0, pool_top) have been handed out at least once
  uint32_t free_count;   // recycled ids in free_list[0, free_count)
  uint32_t ticket;       // ids taken in the open allocation epoch
  uint32_t new_blocks;   // blocks created by the last allocation epoch(s)
  uint32_t tri_count;    // triangles produced by the last extraction
  uint32_t error;        // sticky kErr* bits
  unsigned long long voxels_updated;  // by the last integration
  uint32_t tombstones;   // erased slots
  uint32_t erased;       // keys erased by the last erase call
  uint32_t mc_next;      // marching cubes: blocks handed out past the first grid
  uint32_t mc_done;      // marching cubes: CTAs finished (state copy-out)
  uint32_t vert_count;   // vertices of the last indexed per-frame mesh
  uint32_t pad;
};

// Everything a kernel needs to reach the volume; passed by value.
struct VolumeView {
  Slot *slots;
  uint32_t slot_mask;
  int32_t max_probe;
  float *pool;
  unsigned long long *block_keys;
  uint32_t *free_list;
  uint32_t *frame_list;
  uint32_t *frame_nb;  // per frame-list entry: the block and its 7 +x/+y/+z neighbours
  ulonglong2 *frame_res;  // per frame-list entry: {key, pool block} (resolved slot)
  uint32_t frame_cap;
  uint32_t pool_cap;
  DevState *st;
};

// Camera and integration constants of a handle.
struct CamParams {
  int32_t width, height;
  float wf, hf;  // width, height as floats
  float fx, fy, cx, cy;
  float min_depth, max_depth, depth_scale;
  float voxel, trunc, mc_min_weight;
  float rtrunc;         // 1 / trunc correctly rounded (host-computed)
  const float *rcp_w;   // device table: rcp_w[w] = 1 / w correctly rounded, w <= kRcpMax
};

// Weights up to this have a correctly rounded reciprocal in CamParams::rcp_w.
constexpr int kRcpMax = 2048;

__host__ __device__ inline bool key_in_range(int x, int y, int z) {
  return (uint32_t)(x + kKeyBias) < (1u << 21) && (uint32_t)(y + kKeyBias) < (1u << 21) &&
         (uint32_t)(z + kKeyBias) < (1u << 21);
}

__host__ __device__ inline unsigned long long pack_key(int x, int y, int z) {
  return (unsigned long long)(uint32_t)(x + kKeyBias) |
         ((unsigned long long)(uint32_t)(y + kKeyBias) << 21) |
         ((unsigned long long)(uint32_t)(z + kKeyBias) << 42);
}

__host__ __device__ inline void unpack_key(unsigned long long k, int &x, int &y, int &z) {
  x = (int)(k & 0x1FFFFFull) - kKeyBias;
  y = (int)((k >> 21) & 0x1FFFFFull) - kKeyBias;
  z = (int)((k >> 42) & 0x1FFFFFull) - kKeyBias;
}

// 64-bit finaliser (splitmix64 / Stafford mix 13) for the slot index.
__host__ __device__ inline unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// The reference's BlockHasher (include/tsdf.cuh:144-156): each int component
// is converted to size_t (sign-extended), multiplied and XORed.
__host__ __device__ inline unsigned long long ref_block_hash(int x, int y, int z) {
  return ((unsigned long long)(long long)x * 73856093ull) ^
         ((unsigned long long)(long long)y * 19349669ull) ^
         ((unsigned long long)(long long)z * 83492791ull);
}

// One scene of a batch: everything the batched kernels need to reach the
// scene's volume and its staged frame (device array built by vh_batch.cpp).
struct SceneDesc {
  VolumeView V;
  CamParams C;
  const void *depth;  // staged depth (format shared by the batch)
  const uint8_t *rgb;
  const float *pose;  // row-major camera-to-world, rows 0-2 used
  uint2 *pix;
  float4 *tris;
  uint32_t tri_cap;
  uint32_t pad;
};

constexpr int kMaxBatchScenes = 1024;
constexpr int kBatchPixelThreads = 256;  // threads of a batched allocation CTA

// Work hand-out of a batched step run as one persistent launch
// (k_batch_step): per scene, the stage it is in and the next ticket of that
// stage in one 64-bit word, so that taking a ticket and learning which stage
// it belongs to is one atomic.  Stages: 0 allocation, 1 frame-list resolve,
// 2 integration, 3 marching cubes, 4 (kStepDone) finished or no frame.
constexpr uint32_t kStepDone = 4;
struct StepSched {
  unsigned long long word;  // stage << 32 | next ticket of that stage
  uint32_t total[4];        // items of each stage (written before it opens)
  uint32_t done[4];         // finished items of each stage
  uint32_t count;           // frame-list length after allocation
  uint32_t pad[3];
};
struct StepGlobal {
  uint32_t remaining;  // scenes of the step not finished yet
  uint32_t gave_up;    // CTAs that stopped waiting for work (a bug: never expected)
  uint32_t pad[2];
};

// The inputs of one frame as the kernels find them on the device: the
// camera pose and where the depth and colour images live (the caller's own
// device buffers, or the handle's staging copy of host images).  Written per
// frame by k_frame_begin from its parameters, so a captured frame graph
// serves every frame.
struct FrameIn {
  float pose[16];  // row-major camera-to-world; the kernels read rows 0-2
  const void *depth;
  const uint8_t *rgb;
};

// ---- host-side launchers (vh_kernels.cu) ----------------------------------
// fin (optional): the frame's descriptor, written to d_fin by the kernel.
void launch_frame_begin(const VolumeView &V, const FrameIn *fin, FrameIn *d_fin, cudaStream_t s);
// Copies the device counters to `host` (mapped pinned memory) in-stream.
void launch_state_out(const VolumeView &V, DevState *host, cudaStream_t s);
// The k_frame_begin node of a captured frame graph (nullptr if it has none),
// and the per-launch update of its descriptor parameter.
cudaGraphNode_t find_frame_begin_node(cudaGraph_t g);
cudaError_t update_frame_begin(cudaGraphExec_t e, cudaGraphNode_t n, const VolumeView &V,
                               const FrameIn &fin, FrameIn *d_fin);
void launch_epoch_end(const VolumeView &V, cudaStream_t s);
void launch_clear_list(const VolumeView &V, cudaStream_t s);
void launch_mc_begin(const VolumeView &V, cudaStream_t s);

// fmt: 0 = uint16 scaled by depth_scale, 1 = float metres.  depth (when not
// null) replaces fin->depth.  filter: each pixel's depth goes through the
// bilateral pre-filter (VH_FLAG_DEPTH_FILTER) inside the allocation kernel.
void launch_allocate(const VolumeView &V, const CamParams &C, const FrameIn *fin,
                     const void *depth, int fmt, bool filter, uint2 *pix, cudaStream_t s);
// variant 0: one block in flight per CTA; 1: next block prefetched
void launch_integrate(const VolumeView &V, const CamParams &C, const uint2 *pix,
                      const float *pose, int grid, int variant, cudaStream_t s);
// host_state (optional, mapped host memory): the last CTA copies the device
// counters there, as launch_state_out would after the kernel.
void launch_mc(const VolumeView &V, int scope_all, float min_weight, float4 *tris,
               uint32_t tri_cap, int grid, int variant, DevState *host_state, cudaStream_t s);
// Marching cubes of the frame's blocks into an indexed mesh: vertices
// (float4 {x, y, z, rgb bits}, global voxel units) and faces (3 vertex
// numbers each), counts in the state's vert_count and tri_count; the last
// CTA copies the counters to host_state (mapped host memory) if given.
void launch_mc_indexed(const VolumeView &V, float min_weight, float4 *verts, uint32_t vcap,
                       int32_t *faces, uint32_t fcap, int grid, DevState *host_state,
                       cudaStream_t s);
int mc_indexed_ctas_per_sm();
// Resident CTAs per SM of the persistent kernels (for grid sizing), and the
// number of launch shapes of each (variants 0 .. n - 1).
int integrate_ctas_per_sm(int variant);
int mc_ctas_per_sm(int variant);
int integrate_variants();
int mc_variants();
void launch_alloc_keys(const VolumeView &V, const int32_t *xyz, uint32_t n, cudaStream_t s);
void launch_find_keys(const VolumeView &V, const int32_t *xyz, uint32_t n, int32_t *out,
                      cudaStream_t s);
void launch_erase_keys(const VolumeView &V, const int32_t *xyz, uint32_t n, cudaStream_t s);
void launch_frame_nb(const VolumeView &V, cudaStream_t s);
// Writes frame_res and frame_nb for the current block list (after
// allocation); also closes the allocation epoch and, with mc_follows, resets
// the marching-cubes counters (what launch_mc_begin does).
void launch_frame_resolve(const VolumeView &V, int grid, bool mc_follows, cudaStream_t s);
void launch_list_keys(const VolumeView &V, int32_t *xyz, uint32_t n, cudaStream_t s);
void launch_scatter_blocks(const VolumeView &V, const int32_t *xyz, const float *sdf,
                           const float *w, const uint8_t *rgb, uint32_t n, cudaStream_t s);

// Bilateral pre-filter of one depth image into float metres; depth ==
// nullptr reads the image of fin.
// rcp[w] = 1 / w correctly rounded for w in [1, kRcpMax] (rcp[0] = 0).
void launch_rcp_table(float *rcp, cudaStream_t s);

void launch_depth_filter(const CamParams &C, const void *depth, const FrameIn *fin, int fmt,
                         float *out, cudaStream_t s);

// Batched stages: one launch covers the work of every active scene.
// active[i] != 0: scene i has a frame this step.  px_start: first global
// pixel of each scene (multiples of kBatchPixelThreads; n + 1 entries).  prefix: per-scene
// work prefix (n + 1 entries) written by launch_batch_resolve (frame
// lists) and read by the later stages.
void launch_batch_frame_begin(const SceneDesc *d, const uint8_t *active, int n, cudaStream_t s);
void launch_batch_allocate(const SceneDesc *d, const uint8_t *active, const uint32_t *px_start,
                           uint32_t total_px, int n, int fmt, cudaStream_t s);
// Closes every active scene's allocation epoch, writes prefix and resolves
// the frame lists (one launch); with_mesh: also resets every active
// scene's marching-cubes counters.
void launch_batch_resolve(const SceneDesc *d, const uint8_t *active, int n, uint32_t *prefix,
                          bool with_mesh, int grid, cudaStream_t s);
void launch_batch_integrate(const SceneDesc *d, const uint32_t *prefix, int n, int grid,
                            cudaStream_t s);
void launch_batch_mc(const SceneDesc *d, uint32_t *prefix, int n, int grid, int variant,
                     cudaStream_t s);
void launch_batch_gather_state(const SceneDesc *d, int n, DevState *out, cudaStream_t s);
// Resident CTAs per SM of the batched persistent kernels.
int batch_integrate_ctas_per_sm();
int batch_mc_ctas_per_sm(int variant);
void launch_batch_clear_errors(const SceneDesc *d, int n, cudaStream_t s);
// A whole batched step as one persistent launch (after a one-CTA begin
// kernel that opens every active scene's frame and resets the hand-out):
// allocation, resolve, integration and, with with_mesh, marching cubes of
// every active scene, CTAs taking work items of whichever scene has some.
// sched: n entries; glob: one.  n <= kMaxBatchScenes.  grid: persistent
// CTAs (SMs x batch_step_ctas_per_sm; progress does not depend on it).
void launch_batch_step(const SceneDesc *d, const uint8_t *active, int n, StepSched *sched,
                       StepGlobal *glob, int fmt, bool with_mesh, int grid, cudaStream_t s);
int batch_step_ctas_per_sm(bool with_mesh);

}  // namespace vh
