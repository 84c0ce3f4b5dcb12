// vh_stream.cu - out-of-core blocks: moving parts of the volume between HBM
// and a host store.
//
// The reference keeps its volume on the host in 128^3-voxel chunks and every
// frame streams the chunks near the camera in and everything back out
// (src/tsdf.cu:118-596, GpuTsdfGenerator::processFrame :1484-1598).  Here
// the volume stays resident and streaming is explicit and selective: blocks
// whose centre is farther than a radius from a point (typically the camera)
// leave HBM for a host store in the handle, and come back when the caller
// asks for a region.  Blocks travel in their pool layout (sdf | weight |
// rgba, 6 KiB), so a block that goes out and comes back is bit-identical.
//   out: one kernel lists the far blocks (key, pool id) of the pool; the
//        blocks are gathered into a contiguous buffer, copied to the host
//        store, and erased (slot tombstoned, block zeroed and freed);
//   in:  the store's blocks within the radius are copied up, their keys
//        inserted (joining the current block list, as vh_alloc_keys does)
//        and their voxels written into the new pool blocks.

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>

#include <stdlib.h>
#include <sys/mman.h>
#include <unordered_map>
#include <vector>

#include "vh_device.cuh"
#include "vh_internal.h"

namespace vh {

// Asynchronous eviction (vh_evict_async): one in-flight eviction per slot.
// Device staging holds the gathered blocks once they have left the volume;
// a copy kernel on the evictor's own stream writes them into mapped pinned
// host memory while the handle's stream runs later frames.
constexpr uint32_t kEvictCap = 1u << 15;  // blocks per call (192 MiB per slot)

struct EvictSlot {
  float *d_data = nullptr;              // kEvictCap blocks, device
  unsigned long long *d_keys = nullptr;
  uint32_t *d_ids = nullptr;
  uint32_t *d_count = nullptr;          // selected blocks (may exceed kEvictCap)
  float *h_data = nullptr;              // pinned and mapped: the copy's target
  unsigned long long *h_keys = nullptr;
  uint32_t *h_count = nullptr;
  float *h_data_dev = nullptr;          // their device addresses
  unsigned long long *h_keys_dev = nullptr;
  uint32_t *h_count_dev = nullptr;
  cudaEvent_t done = nullptr;           // the copy kernel has finished
  bool busy = false;
  uint64_t seq = 0;
};

struct StreamStore;
void store_put(StreamStore &S, unsigned long long key, const float *blk);
void store_reserve(StreamStore &S, size_t more);
int64_t store_size(const StreamStore &S);

// A host thread moves each finished eviction into the store, so the calling
// thread only enqueues GPU work.  mu guards the store, the queue and the
// slots' busy flags while the thread runs.
struct Evictor {
  cudaStream_t stream = nullptr;
  EvictSlot slot[2];
  uint64_t seq = 0;
  uint64_t evicted_since_compaction = 0;
  int device = 0;
  StreamStore *store = nullptr;
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<int> queue;  // slots whose copy is awaited, oldest first
  bool stop = false;
  bool failed = false;
  int64_t stored = 0;  // blocks in the store after the last finished eviction

  void run() {
    cudaSetDevice(device);
    for (;;) {
      int k;
      {
        std::unique_lock<std::mutex> lock(mu);
        cv.wait(lock, [&] { return stop || !queue.empty(); });
        if (queue.empty()) return;
        k = queue.front();
      }
      EvictSlot &e = slot[k];
      const cudaError_t q = cudaEventSynchronize(e.done);
      // the store is this thread's while the queue is not empty (the API
      // calls that use it wait for an empty queue first), so it is filled
      // without holding mu and vh_evict_async never waits for it
      uint32_t n = 0;
      bool stored_ok = q == cudaSuccess;
      if (stored_ok) {
        n = *e.h_count;
        try {
          store_reserve(*store, n);
          for (uint32_t j = 0; j < n; ++j)
            store_put(*store, e.h_keys[j], e.h_data + (size_t)j * kBlockWords);
        } catch (const std::bad_alloc &) {
          stored_ok = false;
        }
      }
      {
        std::lock_guard<std::mutex> lock(mu);
        if (!stored_ok) failed = true;
        evicted_since_compaction += n;
        stored = store_size(*store);
        e.busy = false;
        queue.pop_front();
      }
      cv.notify_all();
    }
  }

  ~Evictor() {
    {
      std::lock_guard<std::mutex> lock(mu);
      stop = true;
    }
    cv.notify_all();
    if (worker.joinable()) worker.join();
    if (stream) cudaStreamSynchronize(stream);
    for (auto &e : slot) {
      cudaFree(e.d_data);
      cudaFree(e.d_keys);
      cudaFree(e.d_ids);
      cudaFree(e.d_count);
      if (e.h_data) cudaFreeHost(e.h_data);
      if (e.h_keys) cudaFreeHost(e.h_keys);
      if (e.h_count) cudaFreeHost(e.h_count);
      if (e.done) cudaEventDestroy(e.done);
    }
    if (stream) cudaStreamDestroy(stream);
  }
};

// Host memory of the stored blocks: chunks of kChunkBlocks blocks, allocated
// without zero fill (on huge pages where the OS grants them) and faulted in
// when a chunk is added, so filing a block later costs one memcpy.
class BlockArena {
 public:
  static constexpr size_t kChunkBlocks = 8192;  // 48 MiB per chunk
  BlockArena() = default;
  BlockArena(const BlockArena &) = delete;
  BlockArena &operator=(const BlockArena &) = delete;
  ~BlockArena() {
    for (void *c : chunks_) std::free(c);
  }
  float *block(size_t e) const {
    return static_cast<float *>(chunks_[e / kChunkBlocks]) + (e % kChunkBlocks) * kBlockWords;
  }
  // entries [0, n) addressable
  bool reserve(size_t n) {
    while (chunks_.size() * kChunkBlocks < n)
      if (!add_chunk()) return false;
    return true;
  }
  void swap(BlockArena &o) { chunks_.swap(o.chunks_); }

 private:
  bool add_chunk() {
    const size_t bytes = kChunkBlocks * kBlockWords * sizeof(float);
    void *p = nullptr;
    if (posix_memalign(&p, (size_t)1 << 21, bytes) != 0) return false;
    madvise(p, bytes, MADV_HUGEPAGE);  // a hint: fewer page faults if granted
    for (size_t o = 0; o < bytes; o += 4096) static_cast<volatile char *>(p)[o] = 0;
    chunks_.push_back(p);
    return true;
  }
  std::vector<void *> chunks_;
};

struct StreamStore {
  std::unordered_map<unsigned long long, size_t> index;  // key -> entry
  std::vector<unsigned long long> keys;                   // per entry (kEmptyKey: free)
  BlockArena arena;                                       // kBlockWords per entry
  std::vector<size_t> free_entries;
  Evictor *evict = nullptr;                               // created on first use
  ~StreamStore() { delete evict; }
};

void stream_store_free(StreamStore *s) { delete s; }

namespace {

constexpr uint32_t kChunk = 1u << 16;  // blocks per transfer (384 MiB)

// Far blocks of the pool: key and pool id of every live block whose centre
// is farther than sqrt(r2) from (cx, cy, cz).
__global__ void __launch_bounds__(256) k_select_far(VolumeView V, float voxel, float cx, float cy,
                                                    float cz, float r2,
                                                    uint32_t *__restrict__ count,
                                                    unsigned long long *__restrict__ keys,
                                                    uint32_t *__restrict__ ids, uint32_t cap) {
  const uint32_t top = min(V.st->pool_top, V.pool_cap);
  for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < top; b += gridDim.x * blockDim.x) {
    const unsigned long long key = V.block_keys[b];
    if (key >= kTombKey) continue;
    int bx, by, bz;
    unpack_key(key, bx, by, bz);
    const float x = ((float)(bx * kB) + 3.5f) * voxel - cx;
    const float y = ((float)(by * kB) + 3.5f) * voxel - cy;
    const float z = ((float)(bz * kB) + 3.5f) * voxel - cz;
    if (x * x + y * y + z * z <= r2) continue;
    const uint32_t slot = atomicAdd(count, 1u);
    if (slot < cap) {
      keys[slot] = key;
      ids[slot] = b;
    }
  }
}

// One CTA per block: out[i] = pool block ids[i] (16-byte copies).
__global__ void __launch_bounds__(128) k_gather_blocks(const float *__restrict__ pool,
                                                       const uint32_t *__restrict__ ids,
                                                       uint32_t n, float *__restrict__ out) {
  const uint32_t i = blockIdx.x;
  if (i >= n) return;
  const float4 *src = reinterpret_cast<const float4 *>(pool + (size_t)ids[i] * kBlockWords);
  float4 *dst = reinterpret_cast<float4 *>(out + (size_t)i * kBlockWords);
  for (int k = threadIdx.x; k < kBlockWords / 4; k += blockDim.x) dst[k] = src[k];
}

__global__ void k_keys_to_xyz(const unsigned long long *__restrict__ keys, uint32_t n,
                              int32_t *__restrict__ xyz) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int x, y, z;
  unpack_key(keys[i], x, y, z);
  xyz[3 * i] = x;
  xyz[3 * i + 1] = y;
  xyz[3 * i + 2] = z;
}

// Weighted average of two partial averages of one voxel: a copy observed
// w_a times with value a and one observed w_b times with value b combine to
// (a w_a + b w_b) / (w_a + w_b) with weight w_a + w_b.  Explicit roundings
// (no contraction), stored copy first.
__device__ __forceinline__ void merge_voxel(float &sdf, float &w, uint32_t &rgb, float s_sdf,
                                            float s_w, uint32_t s_rgb) {
  if (s_w == 0.0f) return;  // the stored copy never saw this voxel
  if (w == 0.0f) {          // only the stored copy did: exact copy
    sdf = s_sdf;
    w = s_w;
    rgb = s_rgb;
    return;
  }
  const float wn = __fadd_rn(s_w, w);
  sdf = __fdiv_rn(__fadd_rn(__fmul_rn(s_sdf, s_w), __fmul_rn(sdf, w)), wn);
  // colour: exact integer floor of the weighted sum (weights are whole
  // numbers below 2^24, so every product fits in 64 bits)
  const unsigned long long ws = (unsigned long long)s_w, wr = (unsigned long long)w,
                           wt = ws + wr;
  uint32_t out = 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const unsigned long long n =
        ((s_rgb >> (8 * c)) & 0xFFu) * ws + ((rgb >> (8 * c)) & 0xFFu) * wr;
    out |= (uint32_t)(n / wt) << (8 * c);
  }
  rgb = out;
  w = wn;
}

// One CTA per block: brings data[i] (pool layout) into the block of key
// xyz[i].  A block created by this stream-in is zero, so it receives an
// exact copy; a block that a frame re-created after the key was moved out
// holds the observations made since, and the two copies are merged voxel by
// voxel (merge_voxel) so that neither set of observations is lost.
__global__ void __launch_bounds__(128) k_scatter_raw(VolumeView V, const int32_t *__restrict__ xyz,
                                                     const float *__restrict__ data, uint32_t n) {
  const uint32_t i = blockIdx.x;
  if (i >= n) return;
  const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  if (!key_in_range(x, y, z)) return;
  const uint32_t b = block_of(V, pack_key(x, y, z));
  if (b == kNoBlock) return;  // the insert failed (pool or table full): reported by the state
  const float *src = data + (size_t)i * kBlockWords;
  float *dst = V.pool + (size_t)b * kBlockWords;
  const int t = threadIdx.x;  // voxels 4t .. 4t+3
  const float4 ss = reinterpret_cast<const float4 *>(src)[t];
  const float4 sw = reinterpret_cast<const float4 *>(src + kB3)[t];
  const uint4 sc = reinterpret_cast<const uint4 *>(src + 2 * kB3)[t];
  float4 ds = reinterpret_cast<const float4 *>(dst)[t];
  float4 dw = reinterpret_cast<const float4 *>(dst + kB3)[t];
  uint4 dc = reinterpret_cast<const uint4 *>(dst + 2 * kB3)[t];
  merge_voxel(ds.x, dw.x, dc.x, ss.x, sw.x, sc.x);
  merge_voxel(ds.y, dw.y, dc.y, ss.y, sw.y, sc.y);
  merge_voxel(ds.z, dw.z, dc.z, ss.z, sw.z, sc.z);
  merge_voxel(ds.w, dw.w, dc.w, ss.w, sw.w, sc.w);
  reinterpret_cast<float4 *>(dst)[t] = ds;
  reinterpret_cast<float4 *>(dst + kB3)[t] = dw;
  reinterpret_cast<uint4 *>(dst + 2 * kB3)[t] = dc;
}

// Eviction, on the handle's stream: every selected block (keys[i], pool id
// ids[i], i < min(*count, cap)) is copied into the device staging buffer,
// then its slot becomes a tombstone and the block is zeroed and returned to
// the free list, so that work enqueued after it no longer sees the block.
// One CTA of 128 threads per block, grid-stride.
__global__ void __launch_bounds__(128) k_evict(VolumeView V, const unsigned long long *__restrict__ keys,
                                               const uint32_t *__restrict__ ids,
                                               const uint32_t *__restrict__ count, uint32_t cap,
                                               float *__restrict__ out) {
  const uint32_t n = min(*count, cap);
  const int t = threadIdx.x;
  for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
    const uint32_t b = ids[i];
    float4 *blk = reinterpret_cast<float4 *>(V.pool + (size_t)b * kBlockWords);
    float4 *dst = reinterpret_cast<float4 *>(out + (size_t)i * kBlockWords);
    for (int k = t; k < kBlockWords / 4; k += blockDim.x) dst[k] = blk[k];
    __syncthreads();  // the block is in the staging buffer before it is cleared
    for (int k = t; k < kBlockWords / 4; k += blockDim.x) blk[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    if (t == 0) {
      const unsigned long long key = keys[i];
      const uint32_t h = (uint32_t)mix64(key) & V.slot_mask;
      for (int p = 0; p < V.max_probe; ++p) {
        const uint32_t s = (h + (uint32_t)p) & V.slot_mask;
        const unsigned long long k = V.slots[s].key;
        if (k == kEmptyKey) break;
        if (k != key) continue;
        V.slots[s].key = kTombKey;
        V.slots[s].block = kNoBlock;
        atomicAdd(&V.st->tombstones, 1u);
        V.block_keys[b] = kEmptyKey;
        __threadfence();
        const uint32_t f = atomicAdd(&V.st->free_count, 1u);
        V.free_list[f] = b;
        break;
      }
    }
  }
}

// Opens an eviction: the allocation epoch closed (as k_epoch_end) and the
// selection counter cleared.
__global__ void k_evict_begin(VolumeView V, uint32_t *__restrict__ count) {
  if (threadIdx.x != 0) return;
  reconcile_epoch(V);
  *count = 0u;
}

// The evicted blocks and their keys from device staging into mapped host
// memory (on the evictor's stream, beside later frames); count last.
__global__ void __launch_bounds__(256) k_evict_copy(const float *__restrict__ data,
                                                    const unsigned long long *__restrict__ keys,
                                                    const uint32_t *__restrict__ count, uint32_t cap,
                                                    float *__restrict__ h_data,
                                                    unsigned long long *__restrict__ h_keys,
                                                    uint32_t *__restrict__ h_count) {
  const uint32_t n = min(*count, cap);
  const size_t words4 = (size_t)n * (kBlockWords / 4);
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const float4 *src = reinterpret_cast<const float4 *>(data);
  float4 *dst = reinterpret_cast<float4 *>(h_data);
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < words4; k += stride)
    dst[k] = src[k];
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride)
    h_keys[k] = keys[k];
  if (blockIdx.x == 0 && threadIdx.x == 0) *h_count = n;
}

// Table rebuild: every slot emptied, then the key of every live pool block
// inserted again with its block id (keys are unique, so plain CAS claims).
__global__ void __launch_bounds__(256) k_clear_slots(Slot *__restrict__ slots, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    slots[i].key = kEmptyKey;
    slots[i].block = kNoBlock;
    slots[i].stamp = 0xFFFFFFFFu;  // never stamped
  }
}

__global__ void __launch_bounds__(256) k_reinsert(VolumeView V) {
  const uint32_t top = min(V.st->pool_top, V.pool_cap);
  for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < top; b += gridDim.x * blockDim.x) {
    const unsigned long long key = V.block_keys[b];
    if (key >= kTombKey) continue;
    const uint32_t h = (uint32_t)mix64(key) & V.slot_mask;
    bool placed = false;
    for (int i = 0; i < V.max_probe && !placed; ++i) {
      const uint32_t s = (h + (uint32_t)i) & V.slot_mask;
      if (atomicCAS(&V.slots[s].key, kEmptyKey, key) == kEmptyKey) {
        V.slots[s].block = b;
        placed = true;
      }
    }
    if (!placed) atomicOr(&V.st->error, kErrTableFull);
  }
}

// Device scratch freed on scope exit.
struct Scratch {
  std::vector<void *> ptrs;
  ~Scratch() {
    for (void *p : ptrs) cudaFree(p);
  }
  template <typename T>
  bool alloc(T **p, size_t count) {
    void *q = nullptr;
    if (cudaMalloc(&q, sizeof(T) * (count ? count : 1)) != cudaSuccess) return false;
    ptrs.push_back(q);
    *p = static_cast<T *>(q);
    return true;
  }
};

StreamStore &store_of(vh_handle *h) {
  StreamStore *&s = handle_stream_store(h);
  if (!s) s = new StreamStore();
  return *s;
}

// merge_voxel on the host: `blk` (the newer copy) absorbs `old`, voxel by
// voxel, with the same single roundings (volatile temporaries keep the
// compiler from contracting or reordering them).
void merge_block_host(float *blk, const float *old) {
  float *sdf = blk, *w = blk + kB3;
  uint32_t *rgb = reinterpret_cast<uint32_t *>(blk + 2 * kB3);
  const float *o_sdf = old, *o_w = old + kB3;
  const uint32_t *o_rgb = reinterpret_cast<const uint32_t *>(old + 2 * kB3);
  for (int v = 0; v < kB3; ++v) {
    if (o_w[v] == 0.0f) continue;
    if (w[v] == 0.0f) {
      sdf[v] = o_sdf[v];
      w[v] = o_w[v];
      rgb[v] = o_rgb[v];
      continue;
    }
    volatile float wn = o_w[v] + w[v];
    volatile float a = o_sdf[v] * o_w[v];
    volatile float b = sdf[v] * w[v];
    volatile float num = a + b;
    sdf[v] = num / wn;
    const unsigned long long ws = (unsigned long long)o_w[v], wr = (unsigned long long)w[v],
                             wt = ws + wr;
    uint32_t out = 0;
    for (int c = 0; c < 3; ++c) {
      const unsigned long long n =
          ((o_rgb[v] >> (8 * c)) & 0xFFu) * ws + ((rgb[v] >> (8 * c)) & 0xFFu) * wr;
      out |= (uint32_t)(n / wt) << (8 * c);
    }
    rgb[v] = out;
    w[v] = wn;
  }
}

bool far_enough(unsigned long long key, float voxel, const float c[3], double r2) {
  int bx, by, bz;
  unpack_key(key, bx, by, bz);
  const double x = ((double)bx * kB + 3.5) * voxel - c[0];
  const double y = ((double)by * kB + 3.5) * voxel - c[1];
  const double z = ((double)bz * kB + 3.5) * voxel - c[2];
  return x * x + y * y + z * z > r2;
}

}  // namespace

// Adds block `blk` of `key` to the host store; an older stored copy of the
// same key is merged into it (merge_block_host) and dropped.
int64_t store_size(const StreamStore &S) { return (int64_t)S.index.size(); }

// Room for `more` new entries, so that a batch of insertions reallocates
// at most once (geometric growth).
void store_reserve(StreamStore &S, size_t more) {
  const size_t want = S.keys.size() + more;
  if (want > S.keys.capacity()) S.keys.reserve(std::max(want, 2 * S.keys.capacity()));
  S.arena.reserve(want);
  S.index.reserve(S.index.size() + more);
}

void store_put(StreamStore &S, unsigned long long key, const float *blk) {
  size_t e;
  if (!S.free_entries.empty()) {
    e = S.free_entries.back();
    S.free_entries.pop_back();
  } else {
    e = S.keys.size();
    if (!S.arena.reserve(e + 1)) throw std::bad_alloc();
    S.keys.push_back(kEmptyKey);
  }
  std::memcpy(S.arena.block(e), blk, sizeof(float) * kBlockWords);
  S.keys[e] = key;
  auto it = S.index.find(key);
  if (it != S.index.end()) {
    merge_block_host(S.arena.block(e), S.arena.block(it->second));
    S.keys[it->second] = kEmptyKey;
    S.free_entries.push_back(it->second);
    it->second = e;
  } else {
    S.index.emplace(key, e);
  }
}

namespace {

// Waits until the eviction thread has moved every pending eviction into the
// host store (the store is then the calling thread's until the next
// vh_evict_async).
vh_status evict_settle(vh_handle *h) {
  StreamStore *Sp = handle_stream_store(h);
  if (!Sp || !Sp->evict) return VH_OK;
  Evictor &E = *Sp->evict;
  std::unique_lock<std::mutex> lock(E.mu);
  E.cv.wait(lock, [&] { return E.queue.empty(); });
  if (E.failed) {
    E.failed = false;
    return handle_fail(h, VH_ERR_CUDA, "eviction copy failed");
  }
  return VH_OK;
}

vh_status evictor_setup(vh_handle *h, Evictor **out) {
  StreamStore &S = store_of(h);
  if (S.evict) {
    *out = S.evict;
    return VH_OK;
  }
  Evictor *E = new Evictor();
  bool ok = cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking) == cudaSuccess;
  for (auto &e : E->slot) {
    ok = ok && cudaMalloc(&e.d_data, sizeof(float) * kBlockWords * (size_t)kEvictCap) == cudaSuccess &&
         cudaMalloc(&e.d_keys, sizeof(unsigned long long) * kEvictCap) == cudaSuccess &&
         cudaMalloc(&e.d_ids, sizeof(uint32_t) * kEvictCap) == cudaSuccess &&
         cudaMalloc(&e.d_count, sizeof(uint32_t)) == cudaSuccess &&
         cudaHostAlloc(&e.h_data, sizeof(float) * kBlockWords * (size_t)kEvictCap,
                       cudaHostAllocMapped) == cudaSuccess &&
         cudaHostAlloc(&e.h_keys, sizeof(unsigned long long) * kEvictCap, cudaHostAllocMapped) ==
             cudaSuccess &&
         cudaHostAlloc(&e.h_count, sizeof(uint32_t), cudaHostAllocMapped) == cudaSuccess &&
         cudaHostGetDevicePointer(&e.h_data_dev, e.h_data, 0) == cudaSuccess &&
         cudaHostGetDevicePointer(&e.h_keys_dev, e.h_keys, 0) == cudaSuccess &&
         cudaHostGetDevicePointer(&e.h_count_dev, e.h_count, 0) == cudaSuccess &&
         cudaEventCreateWithFlags(&e.done, cudaEventDisableTiming | cudaEventBlockingSync) ==
             cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    delete E;
    return handle_fail(h, VH_ERR_CUDA, "asynchronous eviction: buffer allocation failed");
  }
  E->device = handle_device(h);
  E->store = &S;
  E->worker = std::thread([E] { E->run(); });
  S.evict = E;
  *out = E;
  return VH_OK;
}

}  // namespace
}  // namespace vh

using namespace vh;

extern "C" vh_status vh_evict_async(vh_handle *h, const float *centre, float radius) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_evict_async");
  if (!h || !centre || !(radius >= 0.0f)) return VH_ERR_INVALID_ARG;
  for (int a = 0; a < 3; ++a)
    if (!std::isfinite(centre[a])) return VH_ERR_NOT_FINITE;
  Evictor *E = nullptr;
  vh_status s = evictor_setup(h, &E);
  if (s != VH_OK) return s;
  const VolumeView V = handle_view(h);
  uint64_t evicted = 0;
  {
    std::lock_guard<std::mutex> lock(E->mu);
    evicted = E->evicted_since_compaction;
  }
  // erased slots stay tombstones: rebuild the table (synchronously, rare)
  // once the evictions since the last rebuild could fill an eighth of it
  if (evicted + handle_state(h).tombstones > (V.slot_mask + 1u) / 8u) {
    if ((s = evict_settle(h)) != VH_OK || (s = vh_compact_table(h)) != VH_OK) return s;
    std::lock_guard<std::mutex> lock(E->mu);
    E->evicted_since_compaction = 0;
  }
  EvictSlot *slot = nullptr;
  int k = 0;
  {  // a free slot (both in flight: wait for the older one to be stored)
    std::unique_lock<std::mutex> lock(E->mu);
    E->cv.wait(lock, [&] { return !E->slot[0].busy || !E->slot[1].busy; });
    k = E->slot[0].busy ? 1 : 0;
    slot = &E->slot[k];
    if (E->failed) {
      E->failed = false;
      return handle_fail(h, VH_ERR_CUDA, "eviction copy failed");
    }
  }
  const CamParams C = handle_cam(h);
  const cudaStream_t st = handle_stream(h);
  const float r2 = radius * radius;
  // allocation tickets settled before blocks are freed; selection count 0
  k_evict_begin<<<1, 32, 0, st>>>(V, slot->d_count);
  k_select_far<<<std::min<uint32_t>((V.pool_cap + 255) / 256, 4096), 256, 0, st>>>(
      V, C.voxel, centre[0], centre[1], centre[2], std::isfinite(r2) ? r2 : 3.0e38f, slot->d_count,
      slot->d_keys, slot->d_ids, kEvictCap);
  k_evict<<<2048, 128, 0, st>>>(V, slot->d_keys, slot->d_ids, slot->d_count, kEvictCap,
                                slot->d_data);
  cudaEvent_t gathered = slot->done;  // reused: recorded on st, then waited by the copy
  if (cudaGetLastError() != cudaSuccess || cudaEventRecord(gathered, st) != cudaSuccess ||
      cudaStreamWaitEvent(E->stream, gathered, 0) != cudaSuccess)
    return handle_fail(h, VH_ERR_CUDA, "eviction failed");
  k_evict_copy<<<64, 256, 0, E->stream>>>(slot->d_data, slot->d_keys, slot->d_count, kEvictCap,
                                          slot->h_data_dev, slot->h_keys_dev, slot->h_count_dev);
  if (cudaGetLastError() != cudaSuccess || cudaEventRecord(slot->done, E->stream) != cudaSuccess)
    return handle_fail(h, VH_ERR_CUDA, "eviction copy failed");
  {
    std::lock_guard<std::mutex> lock(E->mu);
    slot->busy = true;
    slot->seq = ++E->seq;
    E->queue.push_back(k);
  }
  E->cv.notify_all();
  handle_invalidate_nb(h);
  return VH_OK;
}

namespace vh {
vh_status stream_store_settle(vh_handle *h) { return evict_settle(h); }
}  // namespace vh

extern "C" vh_status vh_compact_table(vh_handle *h) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_compact_table");
  if (!h) return VH_ERR_INVALID_ARG;
  const VolumeView V = handle_view(h);
  const cudaStream_t st = handle_stream(h);
  const uint32_t slots = V.slot_mask + 1u;
  launch_epoch_end(V, st);
  k_clear_slots<<<std::min<uint32_t>((slots + 255) / 256, 8192), 256, 0, st>>>(V.slots, slots);
  k_reinsert<<<std::min<uint32_t>((V.pool_cap + 255) / 256, 8192), 256, 0, st>>>(V);
  // the block list held slot ids: start an empty one
  launch_clear_list(V, st);
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemsetAsync(&V.st->tombstones, 0, sizeof(uint32_t), st) != cudaSuccess)
    return handle_fail(h, VH_ERR_CUDA, "table rebuild failed");
  handle_invalidate_nb(h);
  return handle_sync(h);
}

extern "C" vh_status vh_stream_out(vh_handle *h, const float *centre, float radius,
                                   int64_t *moved) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_stream_out");
  if (moved) *moved = 0;
  if (!h || !centre || !(radius >= 0.0f)) return VH_ERR_INVALID_ARG;
  for (int a = 0; a < 3; ++a)
    if (!std::isfinite(centre[a])) return VH_ERR_NOT_FINITE;
  vh_status es = evict_settle(h);  // keeps the order of earlier evictions
  if (es != VH_OK) return es;
  const VolumeView V = handle_view(h);
  const CamParams C = handle_cam(h);
  const cudaStream_t st = handle_stream(h);
  launch_epoch_end(V, st);
  vh_status s = handle_sync(h);
  if (s != VH_OK) return s;
  const uint32_t top = handle_state(h).pool_top;
  if (!top) return VH_OK;
  Scratch sc;
  uint32_t *d_count, *d_ids;
  unsigned long long *d_keys;
  if (!sc.alloc(&d_count, 1) || !sc.alloc(&d_keys, top) || !sc.alloc(&d_ids, top))
    return handle_fail(h, VH_ERR_CUDA, "stream out: device allocation failed");
  uint32_t n = 0;
  const float r2 = radius * radius;
  if (cudaMemsetAsync(d_count, 0, sizeof(uint32_t), st) != cudaSuccess)
    return handle_fail(h, VH_ERR_CUDA, "stream out failed");
  k_select_far<<<std::min<uint32_t>((top + 255) / 256, 4096), 256, 0, st>>>(
      V, C.voxel, centre[0], centre[1], centre[2], std::isfinite(r2) ? r2 : 3.0e38f, d_count,
      d_keys, d_ids, top);
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(&n, d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return handle_fail(h, VH_ERR_CUDA, "stream out: selection failed");
  n = std::min(n, top);
  if (!n) return VH_OK;
  StreamStore &S = store_of(h);
  float *d_data;
  int32_t *d_xyz;
  if (!sc.alloc(&d_data, (size_t)std::min(n, kChunk) * kBlockWords) || !sc.alloc(&d_xyz, 3 * (size_t)n))
    return handle_fail(h, VH_ERR_CUDA, "stream out: device allocation failed");
  std::vector<unsigned long long> keys(n);
  if (cudaMemcpyAsync(keys.data(), d_keys, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost,
                      st) != cudaSuccess)
    return handle_fail(h, VH_ERR_CUDA, "stream out: key copy failed");
  std::vector<float> buf;
  for (uint32_t c0 = 0; c0 < n; c0 += kChunk) {
    const uint32_t cnt = std::min(kChunk, n - c0);
    k_gather_blocks<<<cnt, 128, 0, st>>>(V.pool, d_ids + c0, cnt, d_data);
    buf.resize((size_t)cnt * kBlockWords);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(buf.data(), d_data, sizeof(float) * kBlockWords * cnt,
                        cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return handle_fail(h, VH_ERR_CUDA, "stream out: block copy failed");
    // an older stored copy of a key (moved out before a frame re-created the
    // block) is merged into the outgoing one and dropped
    try {
      store_reserve(S, cnt);
      for (uint32_t j = 0; j < cnt; ++j) store_put(S, keys[c0 + j], &buf[(size_t)j * kBlockWords]);
    } catch (const std::bad_alloc &) {
      return handle_fail(h, VH_ERR_CUDA, "stream out: host store allocation failed");
    }
  }
  k_keys_to_xyz<<<(n + 255) / 256, 256, 0, st>>>(d_keys, n, d_xyz);
  int64_t erased = 0;
  if (cudaGetLastError() != cudaSuccess) return handle_fail(h, VH_ERR_CUDA, "stream out failed");
  s = vh_erase_keys(h, d_xyz, n, &erased, VH_MEM_DEVICE);
  if (s != VH_OK) return s;
  if (moved) *moved = erased;
  // erased slots stay tombstones (inserts do not reuse them): rebuild the
  // table once they fill an eighth of it
  if (handle_state(h).tombstones > (V.slot_mask + 1u) / 8u) return vh_compact_table(h);
  return VH_OK;
}

extern "C" vh_status vh_stream_in(vh_handle *h, const float *centre, float radius, int64_t *moved) {
  VH_HANDLE_DEVICE(h);
  VH_NVTX("vh_stream_in");
  if (moved) *moved = 0;
  if (!h || !centre || !(radius >= 0.0f)) return VH_ERR_INVALID_ARG;
  for (int a = 0; a < 3; ++a)
    if (!std::isfinite(centre[a])) return VH_ERR_NOT_FINITE;
  vh_status es = evict_settle(h);  // pending evictions reach the store first
  if (es != VH_OK) return es;
  StreamStore *Sp = handle_stream_store(h);
  if (!Sp || Sp->index.empty()) return VH_OK;
  StreamStore &S = *Sp;
  const CamParams C = handle_cam(h);
  const double r2 = std::isfinite(radius) ? (double)radius * radius : 1e300;
  std::vector<size_t> pick;
  for (const auto &kv : S.index)
    if (!far_enough(kv.first, C.voxel, centre, r2)) pick.push_back(kv.second);
  if (pick.empty()) return VH_OK;
  std::sort(pick.begin(), pick.end());
  const VolumeView V = handle_view(h);
  const cudaStream_t st = handle_stream(h);
  Scratch sc;
  const uint32_t total = (uint32_t)pick.size();
  int32_t *d_xyz;
  float *d_data;
  if (!sc.alloc(&d_xyz, 3 * (size_t)std::min(total, kChunk)) ||
      !sc.alloc(&d_data, (size_t)std::min(total, kChunk) * kBlockWords))
    return handle_fail(h, VH_ERR_CUDA, "stream in: device allocation failed");
  std::vector<int32_t> xyz;
  std::vector<float> buf;
  int64_t done = 0;
  for (uint32_t c0 = 0; c0 < total; c0 += kChunk) {
    const uint32_t cnt = std::min(kChunk, total - c0);
    xyz.resize(3 * (size_t)cnt);
    buf.resize((size_t)cnt * kBlockWords);
    for (uint32_t j = 0; j < cnt; ++j) {
      const size_t e = pick[c0 + j];
      int x, y, z;
      unpack_key(S.keys[e], x, y, z);
      xyz[3 * j] = x;
      xyz[3 * j + 1] = y;
      xyz[3 * j + 2] = z;
      std::memcpy(&buf[(size_t)j * kBlockWords], S.arena.block(e), sizeof(float) * kBlockWords);
    }
    if (cudaMemcpyAsync(d_xyz, xyz.data(), sizeof(int32_t) * 3 * cnt, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(d_data, buf.data(), sizeof(float) * kBlockWords * cnt,
                        cudaMemcpyHostToDevice, st) != cudaSuccess)
      return handle_fail(h, VH_ERR_CUDA, "stream in: copy failed");
    launch_epoch_end(V, st);
    launch_alloc_keys(V, d_xyz, cnt, st);
    launch_epoch_end(V, st);
    k_scatter_raw<<<cnt, 128, 0, st>>>(V, d_xyz, d_data, cnt);
    if (cudaGetLastError() != cudaSuccess) return handle_fail(h, VH_ERR_CUDA, "stream in failed");
    handle_invalidate_nb(h);
    vh_status s = handle_sync(h);  // pool / table full surface here; the store keeps the blocks
    if (s != VH_OK) return s;
    for (uint32_t j = 0; j < cnt; ++j) {
      const size_t e = pick[c0 + j];
      S.index.erase(S.keys[e]);
      S.keys[e] = kEmptyKey;
      S.free_entries.push_back(e);
    }
    done += cnt;
  }
  // compact the store when most of it is free
  if (S.free_entries.size() > 1024 && S.free_entries.size() * 2 > S.keys.size()) {
    StreamStore T;  // the live entries, packed (the evictor stays with S)
    try {
      store_reserve(T, S.index.size());
      for (const auto &kv : S.index) store_put(T, kv.first, S.arena.block(kv.second));
    } catch (const std::bad_alloc &) {
      return handle_fail(h, VH_ERR_CUDA, "stream in: host store allocation failed");
    }
    S.index.swap(T.index);
    S.keys.swap(T.keys);
    S.free_entries.swap(T.free_entries);
    S.arena.swap(T.arena);
  }
  if (moved) *moved = done;
  return VH_OK;
}

extern "C" int64_t vh_host_blocks(const vh_handle *h) {
  if (!h) return 0;
  StreamStore *Sp = handle_stream_store(const_cast<vh_handle *>(h));
  if (Sp && Sp->evict) {  // finished evictions count; pending ones are not waited for
    std::lock_guard<std::mutex> lock(Sp->evict->mu);
    return Sp->evict->queue.empty() ? (int64_t)Sp->index.size() : Sp->evict->stored;
  }
  StreamStore *s = handle_stream_store(const_cast<vh_handle *>(h));
  return s ? (int64_t)s->index.size() : 0;
}
