// vh_device.cuh - read-only hash lookups shared by the device code.
#pragma once
#include "vh_common.cuh"

namespace vh {

// Slot of `key` or kNoBlock.  Only valid between kernels that insert: a
// lookup never races with a concurrent insertion of the same key.
__device__ __forceinline__ uint32_t slot_find(const VolumeView &V, unsigned long long key) {
  const uint32_t h = (uint32_t)mix64(key) & V.slot_mask;
  for (int i = 0; i < V.max_probe; ++i) {
    const uint32_t s = (h + (uint32_t)i) & V.slot_mask;
    const unsigned long long k = __ldg(&V.slots[s].key);
    if (k == key) return s;
    if (k == kEmptyKey) return kNoBlock;
  }
  return kNoBlock;
}

// Pool block of `key` or kNoBlock.  One 16-byte load per probe: the key and
// the block id of a slot arrive together (same validity rule as slot_find).
__device__ __forceinline__ uint32_t block_of(const VolumeView &V, unsigned long long key) {
  const uint32_t h = (uint32_t)mix64(key) & V.slot_mask;
  for (int i = 0; i < V.max_probe; ++i) {
    const ulonglong2 e =
        __ldg(reinterpret_cast<const ulonglong2 *>(V.slots + ((h + (uint32_t)i) & V.slot_mask)));
    if (e.x == key) return (uint32_t)e.y;
    if (e.x == kEmptyKey) return kNoBlock;
  }
  return kNoBlock;
}

}  // namespace vh
