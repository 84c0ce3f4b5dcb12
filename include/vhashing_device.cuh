/*
 * vhashing_device.cuh - device-side access to a volume's block hash from
 * kernels that the caller writes, in the shape of the device members of
 * vhashing::HashTable (include/vhashing.h of E-BAO/Voxel-Hashing-SDF):
 *
 *   table.find(key), table[key]  HashTable::find and operator[]
 *                                (include/vhashing.h:122-135, probe
 *                                tryfind :149-194)
 *   Apply(table, op)             HashTable::Apply (include/vhashing.h:818-825)
 *   Filter(table, pred, ...)     HashTable::Filter (include/vhashing.h:790-805)
 *   ApplyVoxels(table, op)       (no counterpart: one thread per voxel)
 *
 * Header-only CUDA C++ for .cu files compiled by nvcc.  The addresses come
 * from vh_get_device_table (vhsdf.h) or BlockHashTable::device_table().
 *
 * Differences from the reference, all forced by its layout or by safety:
 *  - a block's value is the pool's structure-of-arrays record (BlockRef:
 *    512 sdf, 512 weights, 512 packed colours) instead of a VoxelBlock of
 *    125 {sdf, colour, weight} structs;
 *  - operator[] of an absent key returns an invalid BlockRef (id -1, null
 *    pointers) where the reference asserts and dereferences null;
 *  - Filter and Apply walk the pool's live blocks (ids below *pool_top
 *    whose key is set), not the hash slots; Filter writes into buffers the
 *    caller passes (the reference allocates with thrust::malloc) in no
 *    particular order;
 *  - inserting and erasing stay with the library's calls (vh_alloc_keys,
 *    vh_erase_keys): device code here reads slots and keys and may rewrite
 *    voxel values of live blocks, nothing else.
 *
 * Launches go to the table's GPU (made current for the launch, the caller's
 * current device restored) on `stream`, or on the handle's stream when
 * stream is NULL, so they run after the work the handle has enqueued.
 */
#ifndef VHASHING_DEVICE_CUH
#define VHASHING_DEVICE_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "vhashing_table.h"

namespace vhashing {

/* One block's voxels (index x + 8y + 64z), or none (id < 0). */
struct BlockRef {
  float *sdf;      /* 512 signed distances, units of the truncation distance */
  float *weight;   /* 512 observation counts                                */
  uint32_t *rgba;  /* 512 colours r | g << 8 | b << 16                        */
  int32_t id;      /* pool index, -1 when the key is absent                  */
  __host__ __device__ bool valid() const { return id >= 0; }
};

class DeviceBlockTable {
 public:
  DeviceBlockTable() = default;
  __host__ explicit DeviceBlockTable(const vh_device_table &t) : t_(t) {}

  __host__ __device__ const vh_device_table &raw() const { return t_; }
  /* false when the library publishes a layout this header does not know */
  __host__ bool compatible() const { return t_.layout == VH_DEVICE_TABLE_LAYOUT; }

  /* Pool index of block `k`, or -1 if absent or outside the key range. */
  __device__ int32_t find(BlockKey k) const {
    const long long bias = t_.key_bias;
    if (!in_range(k.x, bias) || !in_range(k.y, bias) || !in_range(k.z, bias)) return -1;
    const unsigned long long key = (unsigned long long)(k.x + bias) |
                                   ((unsigned long long)(k.y + bias) << 21) |
                                   ((unsigned long long)(k.z + bias) << 42);
    const ulonglong2 *slots = static_cast<const ulonglong2 *>(t_.slots);
    const uint32_t h = (uint32_t)mix(key) & t_.slot_mask;
    for (int i = 0; i < t_.max_probe; ++i) {
      const ulonglong2 e = slots[(h + (uint32_t)i) & t_.slot_mask];  // {key, id | stamp << 32}
      if (e.x == key) return (int32_t)(uint32_t)e.y;  /* an id of all ones reads as -1 */
      if (e.x == kEmpty) return -1;
    }
    return -1;
  }

  /* The block of key `k` (HashTable::operator[]); invalid when absent. */
  __device__ BlockRef operator[](BlockKey k) const { return block(find(k)); }

  /* The block with pool index `id`; invalid when id is out of range. */
  __device__ BlockRef block(int32_t id) const {
    if (id < 0 || (int64_t)id >= t_.pool_capacity) return BlockRef{nullptr, nullptr, nullptr, -1};
    float *b = t_.pool + (size_t)id * (3 * VH_BLOCK_VOXELS);
    return BlockRef{b, b + VH_BLOCK_VOXELS, reinterpret_cast<uint32_t *>(b + 2 * VH_BLOCK_VOXELS),
                    id};
  }

  /* Pool ids [0, pool_top()) have been handed out; live ones have a key. */
  __device__ uint32_t pool_top() const { return *t_.pool_top; }

  /* true and the key of pool block `id` when it is live. */
  __device__ bool key_of(uint32_t id, BlockKey *k) const {
    if ((int64_t)id >= t_.pool_capacity) return false;
    const unsigned long long key = t_.block_keys[id];
    if (key >= kTomb) return false;
    const int bias = t_.key_bias;
    k->x = (int)(key & 0x1FFFFFull) - bias;
    k->y = (int)((key >> 21) & 0x1FFFFFull) - bias;
    k->z = (int)((key >> 42) & 0x1FFFFFull) - bias;
    return true;
  }

 private:
  static constexpr unsigned long long kEmpty = 0xFFFFFFFFFFFFFFFFull;
  static constexpr unsigned long long kTomb = 0xFFFFFFFFFFFFFFFEull;

  __device__ static bool in_range(int c, long long bias) {
    return (unsigned long long)(c + bias) < (unsigned long long)(2 * bias);
  }
  /* The slot hash of the library's table: the splitmix64 finaliser of the
   * packed key (the table's own choice; the reference buckets with
   * BlockHasher, vh_block_hash_ref). */
  __device__ static unsigned long long mix(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }

  vh_device_table t_{};
};

namespace detail {

template <class Op>
__global__ void apply_blocks(DeviceBlockTable t, Op op) {
  const uint32_t top = t.pool_top();
  for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < top; b += gridDim.x * blockDim.x) {
    BlockKey k;
    if (t.key_of(b, &k)) op(k, t.block((int32_t)b));
  }
}

template <class Op>
__global__ void apply_voxels(DeviceBlockTable t, Op op) {
  const uint32_t top = t.pool_top();
  for (uint32_t b = blockIdx.x; b < top; b += gridDim.x) {
    BlockKey k;
    if (!t.key_of(b, &k)) continue;  // the same for the whole CTA
    const BlockRef r = t.block((int32_t)b);
    for (int v = threadIdx.x; v < VH_BLOCK_VOXELS; v += blockDim.x) op(k, v, r);
  }
}

// Every warp walks the same ids (the loop bound is uniform per CTA), so the
// kept blocks of a warp take one atomic.
template <class Pred>
__global__ void filter_blocks(DeviceBlockTable t, Pred pred, int32_t *xyz, int32_t *ids,
                              unsigned long long cap, unsigned long long *count) {
  const uint32_t top = t.pool_top();
  const int lane = threadIdx.x & 31;
  for (uint32_t b0 = blockIdx.x * blockDim.x; b0 < top; b0 += gridDim.x * blockDim.x) {
    const uint32_t b = b0 + threadIdx.x;
    BlockKey k{0, 0, 0};
    const bool keep = b < top && t.key_of(b, &k) && pred(k, t.block((int32_t)b));
    const unsigned m = __ballot_sync(0xFFFFFFFFu, keep);
    if (!m) continue;
    const int first = __ffs(m) - 1;
    unsigned long long base = 0;
    if (lane == first) base = atomicAdd(count, (unsigned long long)__popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, first);
    if (keep) {
      const unsigned long long i = base + (unsigned long long)__popc(m & ((1u << lane) - 1u));
      if (i < cap) {
        if (xyz) {
          xyz[3 * i] = k.x;
          xyz[3 * i + 1] = k.y;
          xyz[3 * i + 2] = k.z;
        }
        if (ids) ids[i] = (int32_t)b;
      }
    }
  }
}

// Makes the table's GPU current for one launch and restores the caller's.
class OnDevice {
 public:
  explicit OnDevice(int device) {
    ok_ = cudaGetDevice(&prev_) == cudaSuccess && cudaSetDevice(device) == cudaSuccess;
  }
  ~OnDevice() {
    if (ok_) cudaSetDevice(prev_);
  }
  bool ok() const { return ok_; }

 private:
  int prev_ = 0;
  bool ok_ = false;
};

inline int resident_grid(int device, int ctas_per_sm) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms < 1)
    sms = 1;
  return sms * ctas_per_sm;
}

inline cudaStream_t stream_or_handle(const DeviceBlockTable &t, cudaStream_t s) {
  return s ? s : static_cast<cudaStream_t>(t.raw().stream);
}

inline vh_status launched() {
  return cudaGetLastError() == cudaSuccess ? VH_OK : VH_ERR_CUDA;
}

}  // namespace detail

/* HashTable::Apply: op(BlockKey key, BlockRef block) once for every live
 * block, one thread each, in no particular order.  Asynchronous. */
template <class Op>
vh_status Apply(const DeviceBlockTable &t, Op op, cudaStream_t stream = nullptr) {
  if (!t.compatible()) return VH_ERR_UNSUPPORTED;
  detail::OnDevice on(t.raw().device);
  if (!on.ok()) return VH_ERR_CUDA;
  detail::apply_blocks<Op><<<detail::resident_grid(t.raw().device, 8), 256, 0,
                             detail::stream_or_handle(t, stream)>>>(t, op);
  return detail::launched();
}

/* op(BlockKey key, int voxel, BlockRef block) once for every voxel of
 * every live block (voxel = x + 8y + 64z; one CTA per block at a time, one
 * thread per voxel).  Asynchronous. */
template <class Op>
vh_status ApplyVoxels(const DeviceBlockTable &t, Op op, cudaStream_t stream = nullptr) {
  if (!t.compatible()) return VH_ERR_UNSUPPORTED;
  detail::OnDevice on(t.raw().device);
  if (!on.ok()) return VH_ERR_CUDA;
  detail::apply_voxels<Op><<<detail::resident_grid(t.raw().device, 8), 128, 0,
                             detail::stream_or_handle(t, stream)>>>(t, op);
  return detail::launched();
}

/* HashTable::Filter: the live blocks with pred(BlockKey, BlockRef) true.
 * Device outputs: xyz (3 ints per block, may be NULL), ids (pool index,
 * may be NULL), at most `capacity` of them, in no particular order;
 * *count (device) receives the number of blocks kept, which may exceed
 * capacity.  Asynchronous: *count is cleared on the stream first. */
template <class Pred>
vh_status Filter(const DeviceBlockTable &t, Pred pred, int32_t *xyz, int32_t *ids,
                 int64_t capacity, unsigned long long *count, cudaStream_t stream = nullptr) {
  if (!t.compatible()) return VH_ERR_UNSUPPORTED;
  if (!count || capacity < 0) return VH_ERR_INVALID_ARG;
  detail::OnDevice on(t.raw().device);
  if (!on.ok()) return VH_ERR_CUDA;
  const cudaStream_t s = detail::stream_or_handle(t, stream);
  if (cudaMemsetAsync(count, 0, sizeof(*count), s) != cudaSuccess) return VH_ERR_CUDA;
  detail::filter_blocks<Pred><<<detail::resident_grid(t.raw().device, 8), 256, 0, s>>>(
      t, pred, xyz, ids, (unsigned long long)capacity, count);
  return detail::launched();
}

}  // namespace vhashing

#endif  // VHASHING_DEVICE_CUH
