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

// L2 policy for hash-slot reads: evict-last, so that the table (64 MB at
// 2^22 slots) keeps its L2 lines against the voxel and triangle traffic that
// streams through L2 every frame (allocation 25.4 -> 24.8 us per frame on the
// long stream).
__device__ __forceinline__ unsigned long long l2_keep_policy() {
  unsigned long long pol;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

// One 16-byte slot {key, block | stamp << 32} through the read-only path,
// with the table's L2 policy (for kernels that do not insert).
__device__ __forceinline__ ulonglong2 ld_slot_ro(const Slot *p) {
  ulonglong2 r;
  asm volatile("ld.global.nc.L2::cache_hint.v2.u64 {%0, %1}, [%2], %3;"
               : "=l"(r.x), "=l"(r.y)
               : "l"(p), "l"(l2_keep_policy()));
  return r;
}

// Pool block of `key` or kNoBlock.  One 16-byte load per probe: the key and
// the block id of a slot arrive together (same validity rule as slot_find).
__device__ __forceinline__ uint32_t block_of(const VolumeView &V, unsigned long long key) {
  const uint32_t h = (uint32_t)mix64(key) & V.slot_mask;
  for (int i = 0; i < V.max_probe; ++i) {
    const ulonglong2 e = ld_slot_ro(V.slots + ((h + (uint32_t)i) & V.slot_mask));
    if (e.x == key) return (uint32_t)e.y;
    if (e.x == kEmptyKey) return kNoBlock;
  }
  return kNoBlock;
}

// Trilinear TSDF sample at a world point with its gradient (shared by the
// sampling adjoint, pose refinement and ray casting).
struct Sample {
  bool ok;
  float phi, gx, gy, gz;  // sdf (units of T) and d sdf / d world (per metre)
};

__device__ __forceinline__ uint32_t nb_block(const VolumeView &V, int bx, int by, int bz) {
  return key_in_range(bx, by, bz) ? block_of(V, pack_key(bx, by, bz)) : kNoBlock;
}

// Trilinear interpolation of the TSDF at world point (x, y, z) and its
// gradient.  Fails when any of the 8 corner voxels is unallocated or has a
// weight below min_w.  The corner blocks are resolved first (one hash lookup,
// more only where the cell crosses a block face); then all 16 loads are
// issued together, without a branch between them (a missing block reads
// block 0, which always exists, and fails the sample afterwards).
__device__ __forceinline__ Sample sample_tsdf(const VolumeView &V, float inv_voxel, float min_w,
                                              float x, float y, float z) {
  Sample s;
  s.ok = false;
  const float qx = x * inv_voxel, qy = y * inv_voxel, qz = z * inv_voxel;
  if (!(fabsf(qx) < 8.0e6f && fabsf(qy) < 8.0e6f && fabsf(qz) < 8.0e6f)) return s;
  const float fxb = floorf(qx), fyb = floorf(qy), fzb = floorf(qz);
  const int ix = (int)fxb, iy = (int)fyb, iz = (int)fzb;
  const float fx = qx - fxb, fy = qy - fyb, fz = qz - fzb;
  const int bx = ix >> 3, by = iy >> 3, bz = iz >> 3;  // floor division
  const int lx = ix & 7, ly = iy & 7, lz = iz & 7;
  const bool cx = lx == 7, cy = ly == 7, cz = lz == 7;  // corners cross into +1 blocks
  uint32_t b[8];
  b[0] = nb_block(V, bx, by, bz);
  b[1] = cx ? nb_block(V, bx + 1, by, bz) : b[0];
  b[2] = cy ? nb_block(V, bx, by + 1, bz) : b[0];
  b[3] = cx && cy ? nb_block(V, bx + 1, by + 1, bz) : (cx ? b[1] : b[2]);
  b[4] = cz ? nb_block(V, bx, by, bz + 1) : b[0];
  b[5] = cz ? (cx ? nb_block(V, bx + 1, by, bz + 1) : b[4]) : b[1];
  b[6] = cz ? (cy ? nb_block(V, bx, by + 1, bz + 1) : b[4]) : b[2];
  b[7] = cz ? ((cx || cy) ? nb_block(V, bx + cx, by + cy, bz + 1) : b[4]) : b[3];
  float val[8], w[8];
  bool found = true;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int dx = c & 1, dy = (c >> 1) & 1, dz = c >> 2;
    found = found && b[c] != kNoBlock;
    const int li = ((lx + dx) & 7) + 8 * ((ly + dy) & 7) + 64 * ((lz + dz) & 7);
    const float *base = V.pool + (size_t)(b[c] == kNoBlock ? 0u : b[c]) * kBlockWords;
    w[c] = __ldg(base + kB3 + li);
    val[c] = __ldg(base + li);
  }
  bool observed = true;
#pragma unroll
  for (int c = 0; c < 8; ++c) observed = observed && !(w[c] < min_w);
  if (!found || !observed) return s;
  const float gx0 = 1.0f - fx, gy0 = 1.0f - fy, gz0 = 1.0f - fz;
  // phi = sum_c w_c val_c, w_c = (dx ? fx : 1-fx)(dy ? fy : 1-fy)(dz ? fz : 1-fz)
  const float c00 = val[0] * gx0 + val[1] * fx, c10 = val[2] * gx0 + val[3] * fx;
  const float c01 = val[4] * gx0 + val[5] * fx, c11 = val[6] * gx0 + val[7] * fx;
  const float c0 = c00 * gy0 + c10 * fy, c1 = c01 * gy0 + c11 * fy;
  s.phi = c0 * gz0 + c1 * fz;
  const float d00 = val[1] - val[0], d10 = val[3] - val[2];
  const float d01 = val[5] - val[4], d11 = val[7] - val[6];
  const float dphidx = (d00 * gy0 + d10 * fy) * gz0 + (d01 * gy0 + d11 * fy) * fz;
  const float dphidy = (c10 - c00) * gz0 + (c11 - c01) * fz;
  const float dphidz = c1 - c0;
  s.gx = dphidx * inv_voxel;
  s.gy = dphidy * inv_voxel;
  s.gz = dphidz * inv_voxel;
  s.ok = true;
  return s;
}

// Closes the open allocation epoch (one thread): the tickets handed out
// since the last close become blocks taken from the free list first, then
// from the bump pointer (capped at the pool's capacity).
__device__ __forceinline__ void reconcile_epoch(const VolumeView &V) {
  DevState *st = V.st;
  const uint32_t t = st->ticket;
  if (!t) return;
  const uint32_t from_free = min(t, st->free_count);
  st->free_count -= from_free;
  const unsigned long long top = (unsigned long long)st->pool_top + (t - from_free);
  const uint32_t new_top = (uint32_t)min(top, (unsigned long long)V.pool_cap);
  st->new_blocks += from_free + (new_top - st->pool_top);
  st->pool_top = new_top;
  st->ticket = 0;
}

}  // namespace vh
