// vh_kernels.cu - the per-frame hot path on sm_103a.
//
//   k_allocate   one thread per pixel: walks the blocks of the pixel's
//                truncation band, de-duplicates keys across the warp with
//                __match_any_sync, collects the warp's keys in shared memory
//                and resolves them in rounds of 32: claims new keys with one
//                atomicCAS, hands out pool blocks with one warp-aggregated
//                atomic, stamps each touched slot once per frame and appends
//                it to the frame list (replaces HashAssignKernel,
//                src/tsdf.cu:2088-2238, and the locked insert of
//                include/vhashing.h:205-239,394-484).
//   k_frame_resolve  the frame list's slots and +x/+y/+z neighbours, 8 threads
//                per entry; also closes the allocation epoch.
//   k_integrate  persistent CTAs of 128 threads, one voxel block per CTA
//                iteration, four voxels per thread with 16-byte loads and
//                stores of sdf, weight and colour (replaces
//                IntegrateHashKernel, src/tsdf.cu:599-751).
//   k_mc         persistent CTAs, blocks handed out by a counter: one block
//                plus its +x/+y/+z halo staged in shared memory (no hash
//                probe per voxel), cube cases counted, CTA-wide scans compact
//                the triangles into one output range per round (replaces
//                marchingCubeHashKernel, src/tsdf.cu:884-1110).
//
// This file is compiled with -fmad=false: every fp32 operation that decides a
// pixel, a block, a cube case or a stored value is a single IEEE rounding in
// the reference's operation order, so the CPU oracle (built with
// -ffp-contract=off) reproduces it bit for bit.
//
// Every loop is bounded (probe length <= max_probe, band walk <= the key
// distance between its end blocks); no kernel waits on another thread.

#include <vector>

#include "vh_common.cuh"
#include "vh_device.cuh"
#include "vh_mc_tables.h"

namespace vh {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
// Smallest float >= 1e-5: `fabs(v) < 0.00001` in the reference compares a
// float against a double literal (src/tsdf.cu:1645-1650); for a float v that
// is exactly `fabsf(v) < kSnap`.
constexpr float kSnap = 0x1.4f8b5ap-17f;

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ unsigned long long ld_volatile(const unsigned long long *p) {
  return *(volatile const unsigned long long *)p;
}
__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) {
  return *(volatile const uint32_t *)p;
}

// Whole slot in one 16-byte access: {key, block | stamp << 32}, a relaxed
// GPU-scope load (sees other threads' claims; not cached in L1) with the
// table's L2 policy.
__device__ __forceinline__ ulonglong2 ld_volatile_slot(const Slot *p) {
  ulonglong2 r;
  asm volatile("ld.relaxed.gpu.global.L2::cache_hint.v2.u64 {%0, %1}, [%2], %3;"
               : "=l"(r.x), "=l"(r.y)
               : "l"(p), "l"(l2_keep_policy()));
  return r;
}

// Claims or finds `key`. Returns the slot index or kNoBlock (table full);
// *stamp is the slot's frame stamp as the probe saw it (kNoBlock for a slot
// claimed here or not found), so a caller can skip the stamp exchange when
// the slot already carries the current frame.
__device__ uint32_t slot_insert(const VolumeView &V, unsigned long long key, bool *created,
                                uint32_t *stamp) {
  const uint32_t h = (uint32_t)mix64(key) & V.slot_mask;
  *stamp = kNoBlock;
  for (int i = 0; i < V.max_probe; ++i) {
    const uint32_t s = (h + (uint32_t)i) & V.slot_mask;
    const ulonglong2 sl = ld_volatile_slot(V.slots + s);
    const unsigned long long k = sl.x;
    if (k == key) {
      *created = false;
      *stamp = (uint32_t)(sl.y >> 32);
      return s;
    }
    if (k == kEmptyKey) {
      unsigned long long old = atomicCAS(&V.slots[s].key, kEmptyKey, key);
      if (old == kEmptyKey) {
        *created = true;
        return s;
      }
      if (old == key) {
        *created = false;
        return s;
      }
    }
  }
  atomicOr(&V.st->error, kErrTableFull);
  *created = false;
  return kNoBlock;
}

// Block id for allocation ticket t of the open epoch (free list first).
__device__ __forceinline__ uint32_t take_block(const VolumeView &V, uint32_t t, uint32_t free0,
                                               uint32_t top0) {
  if (t < free0) {
    if (!VH_CHECK(V.st, free0 <= V.pool_cap)) return kNoBlock;
    const uint32_t b = V.free_list[free0 - 1u - t];
    return VH_CHECK(V.st, b < V.pool_cap) ? b : kNoBlock;
  }
  const unsigned long long id = (unsigned long long)top0 + (t - free0);
  if (id >= V.pool_cap) {
    atomicOr(&V.st->error, kErrPoolFull);
    return kNoBlock;
  }
  return (uint32_t)id;
}

// Called by every lane of a warp: lanes with `created` get pool blocks for
// their freshly claimed slots (one atomic per warp).
__device__ __forceinline__ void assign_blocks(const VolumeView &V, bool created, uint32_t slot,
                                              unsigned long long key, uint32_t free0,
                                              uint32_t top0) {
  const unsigned cm = __ballot_sync(kFull, created);
  if (!cm) return;
  const int lane = threadIdx.x & 31;
  const int first = __ffs(cm) - 1;
  uint32_t base = 0;
  if (lane == first) base = atomicAdd(&V.st->ticket, (uint32_t)__popc(cm));
  base = __shfl_sync(kFull, base, first);
  if (created) {
    const uint32_t b = take_block(V, base + (uint32_t)__popc(cm & lanemask_lt()), free0, top0);
    V.slots[slot].block = b;
    if (b != kNoBlock) V.block_keys[b] = key;
  }
}

// Called by every lane: stamps `slot` for this frame and appends it to the
// frame list if this lane is the first to touch it (one atomic per warp).
// `seen`: the slot's stamp as the probe read it (stamps only move forward
// within a frame, so seen == frame means another lane already appended it).
__device__ __forceinline__ void stamp_and_append(const VolumeView &V, bool leader, uint32_t slot,
                                                 uint32_t frame, uint32_t seen) {
  bool app = false;
  if (leader && slot != kNoBlock && seen != frame)
    app = atomicExch(&V.slots[slot].stamp, frame) != frame;
  const unsigned am = __ballot_sync(kFull, app);
  if (!am) return;
  const int lane = threadIdx.x & 31;
  const int first = __ffs(am) - 1;
  uint32_t base = 0;
  if (lane == first) base = atomicAdd(&V.st->frame_count, (uint32_t)__popc(am));
  base = __shfl_sync(kFull, base, first);
  if (app) {
    const uint32_t i = base + (uint32_t)__popc(am & lanemask_lt());
    if (i < V.frame_cap)
      V.frame_list[i] = slot;
    else
      atomicOr(&V.st->error, kErrFrameCap);
  }
}

// ---- band walk ---------------------------------------------------------------
// 6-connected walk over the block cells between two continuous block
// coordinates: exactly |dx|+|dy|+|dz| steps, each along the axis (with cells
// left to cross) whose next boundary comes first; ties go x, y, z.
struct BandWalk {
  int cx, cy, cz;
  int sx, sy, sz;
  int rx, ry, rz;
  float tx, ty, tz;
  float dx, dy, dz;
};

__device__ __forceinline__ void walk_axis(float ga, float gb, int &c, int &st, int &rem, float &tm,
                                          float &td) {
  c = (int)floorf(ga);
  const int e = (int)floorf(gb);
  const float dir = gb - ga;
  if (e > c) {
    st = 1;
    rem = e - c;
    td = 1.0f / dir;
    tm = ((float)(c + 1) - ga) / dir;
  } else if (e < c) {
    st = -1;
    rem = c - e;
    const float nd = -dir;
    td = 1.0f / nd;
    tm = (ga - (float)c) / nd;
  } else {
    st = 0;
    rem = 0;
    td = 0.0f;
    tm = 0.0f;
  }
}

__device__ __forceinline__ bool walk_next(BandWalk &w) {
  int best = -1;
  float bt = 0.0f;
  if (w.rx) {
    best = 0;
    bt = w.tx;
  }
  if (w.ry && (best < 0 || w.ty < bt)) {
    best = 1;
    bt = w.ty;
  }
  if (w.rz && (best < 0 || w.tz < bt)) best = 2;
  if (best == 0) {
    w.cx += w.sx;
    w.rx -= 1;
    w.tx = w.tx + w.dx;
  } else if (best == 1) {
    w.cy += w.sy;
    w.ry -= 1;
    w.ty = w.ty + w.dy;
  } else if (best == 2) {
    w.cz += w.sz;
    w.rz -= 1;
    w.tz = w.tz + w.dz;
  } else {
    return false;
  }
  return true;
}

// frame2cam (src/tsdf.cu:67-74) then cam2base (src/tsdf.cu:95-106), then the
// continuous block coordinate ((p / V) + 0.5) / 8.
__device__ __forceinline__ void pixel_to_grid(int u, int v, float z, const CamParams &C,
                                              const float P[12], float g[3]) {
  const float c0 = (((float)u - C.cx) * z) / C.fx;
  const float c1 = (((float)v - C.cy) * z) / C.fy;
  const float c2 = z;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    float a = c0 * P[r * 4 + 0];
    a = a + c1 * P[r * 4 + 1];
    a = a + c2 * P[r * 4 + 2];
    a = a + P[r * 4 + 3];
    float q = a / C.voxel;
    q = q + 0.5f;
    g[r] = q * 0.125f;
  }
}

template <typename T>
__device__ __forceinline__ float load_depth(const T *d, int i, float scale);
template <>
__device__ __forceinline__ float load_depth<uint16_t>(const uint16_t *d, int i, float scale) {
  return (float)__ldg(d + i) * scale;
}
template <>
__device__ __forceinline__ float load_depth<float>(const float *d, int i, float) {
  return __ldg(d + i);
}

// ---- depth pre-filter (VH_FLAG_DEPTH_FILTER) ---------------------------------------
// The reference only scales its depth (SaveFrame::frameLoad,
// src/SaveFrame.cpp:179-180).  With the flag set, each pixel's depth is
// smoothed by an edge-preserving bilateral filter over a 5x5 window:
// weights exp(-r^2 / (2 s^2)) exp(-(d - d0)^2 / (2 sr^2)) with s = 2 pixels
// and sr = 5 mm + 3 * 1.5e-3 d0^2 (three standard deviations of
// structured-light depth noise), neighbours that are invalid or farther than
// 3 sr from the centre depth left out; an invalid centre pixel stays invalid
// (0).  Allocation computes it for its own pixel from the raw image (the
// filter is fused into the allocation kernel's depth read), and
// vh_filter_depth writes the same values as an image; both come from this
// function in this translation unit, so they agree bit for bit.
template <typename DepthT>
__device__ __forceinline__ float filtered_depth(const CamParams &C, const DepthT *__restrict__ in,
                                                int idx) {
  const int u = idx % C.width, v = idx / C.width;
  const float d0 = load_depth<DepthT>(in, idx, C.depth_scale);
  if (!(d0 > C.min_depth && d0 <= C.max_depth)) return 0.0f;
  const float sr = 0.005f + 4.5e-3f * d0 * d0;
  const float inv_2sr2 = 1.0f / (2.0f * sr * sr), inv_2ss2 = 1.0f / 8.0f;  // s = 2 px
  float sum = 0.0f, wsum = 0.0f;
#pragma unroll
  for (int dy = -2; dy <= 2; ++dy)
#pragma unroll
    for (int dx = -2; dx <= 2; ++dx) {
      const int x = u + dx, y = v + dy;
      if (x < 0 || x >= C.width || y < 0 || y >= C.height) continue;
      const float d = load_depth<DepthT>(in, y * C.width + x, C.depth_scale);
      if (!(d > C.min_depth && d <= C.max_depth) || fabsf(d - d0) >= 3.0f * sr) continue;
      const float w = expf(-(float)(dx * dx + dy * dy) * inv_2ss2 - (d - d0) * (d - d0) * inv_2sr2);
      sum += w * d;
      wsum += w;
    }
  return sum / wsum;  // the centre contributes weight 1
}

template <typename DepthT>
__global__ void __launch_bounds__(256) k_depth_filter(CamParams C, const DepthT *__restrict__ depth,
                                                      const FrameIn *__restrict__ fin,
                                                      float *__restrict__ out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= C.width * C.height) return;
  const DepthT *in = depth ? depth : static_cast<const DepthT *>(fin->depth);
  out[idx] = filtered_depth<DepthT>(C, in, idx);
}

// ---- allocation ----------------------------------------------------------------
constexpr int kAllocChunk = 4;  // band steps of a warp collected before one resolve pass

// Resolves the warp's collected keys (wkeys[0, nkeys), shared, warp-private)
// in rounds of 32: probe or claim, hand out pool blocks, stamp and append.
// All rounds' probes are independent, so a warp pays one dependent chain per
// round instead of one per band step.  A key listed twice (two band steps
// of different lanes) is settled by the claim CAS and the stamp exchange.
__device__ __forceinline__ void resolve_keys(const VolumeView &V, const unsigned long long *wkeys,
                                             int nkeys, uint32_t frame, uint32_t free0,
                                             uint32_t top0) {
  const int lane = threadIdx.x & 31;
  for (int base = 0; base < nkeys; base += 32) {  // warp-uniform
    const bool has = base + lane < nkeys;
    const unsigned long long key = has ? wkeys[base + lane] : kEmptyKey;
    const unsigned peers = __match_any_sync(kFull, key);
    const bool leader = has && (__ffs(peers) - 1) == lane;
    bool created = false;
    uint32_t slot = kNoBlock, seen = kNoBlock;
    if (leader) slot = slot_insert(V, key, &created, &seen);
    assign_blocks(V, created, slot, key, free0, top0);
    stamp_and_append(V, leader, slot, frame, seen);
  }
}

// Pixel idx of one frame (all 32 lanes of the warp take part: the band walk
// is de-duplicated per warp).  Lanes with idx >= npx only follow the warp.
// wkeys: this warp's 32 * kAllocChunk key slots in shared memory.
template <typename DepthT, bool kFilter = false>
__device__ __forceinline__ void allocate_pixel(const VolumeView &V, const CamParams &C,
                                               const DepthT *__restrict__ depth,
                                               const uint8_t *__restrict__ rgb,
                                               const float *__restrict__ pose,
                                               uint2 *__restrict__ pix, int idx,
                                               unsigned long long *wkeys) {
  const int npx = C.width * C.height;
  const int lane = threadIdx.x & 31;
  float P[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) P[k] = __ldg(pose + k);
  const uint32_t frame = V.st->frame;
  const uint32_t free0 = V.st->free_count;
  const uint32_t top0 = V.st->pool_top;

  bool active = false;
  BandWalk w;
  if (idx < npx) {
    const float d = kFilter ? filtered_depth<DepthT>(C, depth, idx)
                            : load_depth<DepthT>(depth, idx, C.depth_scale);
    const uint32_t c = (uint32_t)__ldg(rgb + 3 * idx) | ((uint32_t)__ldg(rgb + 3 * idx + 1) << 8) |
                       ((uint32_t)__ldg(rgb + 3 * idx + 2) << 16);
    pix[idx] = make_uint2(__float_as_uint(d), c);
    if (d > 0.0f && d <= C.max_depth) {
      float z0 = d - C.trunc;
      if (z0 < C.min_depth) z0 = C.min_depth;
      const float z1 = d + C.trunc;
      if (z1 > z0) {
        const int u = idx % C.width, v = idx / C.width;
        float ga[3], gb[3];
        pixel_to_grid(u, v, z0, C, P, ga);
        pixel_to_grid(u, v, z1, C, P, gb);
        bool ok = true;
#pragma unroll
        for (int a = 0; a < 3; ++a)
          ok = ok && fabsf(ga[a]) < kGridLimit && fabsf(gb[a]) < kGridLimit;
        if (ok) {
          walk_axis(ga[0], gb[0], w.cx, w.sx, w.rx, w.tx, w.dx);
          walk_axis(ga[1], gb[1], w.cy, w.sy, w.ry, w.ty, w.dy);
          walk_axis(ga[2], gb[2], w.cz, w.sz, w.rz, w.tz, w.dz);
          active = true;
        } else {
          atomicOr(&V.st->error, kErrRange);
        }
      }
    }
  }
  // Collect each band step's warp-unique keys; resolve them when the list
  // could not take another step's 32, and at the end.
  int nkeys = 0;  // warp-uniform
  while (__any_sync(kFull, active)) {
    const unsigned long long key = active ? pack_key(w.cx, w.cy, w.cz) : kEmptyKey;
    const unsigned peers = __match_any_sync(kFull, key);
    const bool leader = active && (__ffs(peers) - 1) == lane;
    const unsigned lm = __ballot_sync(kFull, leader);
    if (leader) wkeys[nkeys + __popc(lm & lanemask_lt())] = key;
    nkeys += __popc(lm);
    if (active) active = walk_next(w);
    if (nkeys > 32 * (kAllocChunk - 1) || !__any_sync(kFull, active)) {
      __syncwarp();
      resolve_keys(V, wkeys, nkeys, frame, free0, top0);
      __syncwarp();
      nkeys = 0;
    }
  }
}

template <typename DepthT, bool kFilter>
__global__ void __launch_bounds__(256, 6) k_allocate(VolumeView V, CamParams C,
                                                  const FrameIn *__restrict__ fin,
                                                  const DepthT *__restrict__ depth,
                                                  uint2 *__restrict__ pix) {
  __shared__ unsigned long long keys[256 / 32][32 * kAllocChunk];
  const DepthT *d = depth ? depth : static_cast<const DepthT *>(fin->depth);
  allocate_pixel<DepthT, kFilter>(V, C, d, fin->rgb, fin->pose, pix, blockIdx.x * blockDim.x + threadIdx.x,
                         keys[threadIdx.x >> 5]);
}

// ---- integration ---------------------------------------------------------------
// Colour running average of IntegrateHashKernel (src/tsdf.cu:743-745):
// per channel trunc(fp32((c_old * w_old + c_new) / w_new)).  While
// w_old <= 65536 the numerator n = c_old * w_old + c_new is an integer below
// 2^24, exact in fp32, and the fp32 quotient of two integers with divisor
// w <= 131072 truncates to floor(n / w): it cannot round up to the next
// integer (that needs n / w within 2^-17 of it, but it differs from any
// integer by at least 1 / w) nor down past one.  So any exact floor(n / w)
// will do:
//  * w <= 2048: floor(n / w) = umulhi(n, m) for any m in
//    [2^32 / w, 2^32 / w + 2^32 / (255 w^2)), since n <= 255 w keeps
//    n (m - 2^32 / w) / 2^32 below 1 / w, the distance from n / w to the
//    next integer.  m = trunc(rcp(w) * 2^32 (1 + 2^-21)) + 1 with the
//    approximate reciprocal (__fdividef: at most 2 ulp, 2^-22 relative) lies
//    in that range: the 2^-21 bias covers the reciprocal's and the
//    product's rounding from below and stays inside the upper margin
//    (tests/blend_bound_check.c checks every n at both ends of the possible
//    m range for every w).  w_old = 0 keeps the new colour.
//  * w <= 65537: a reciprocal estimate (error < 1) corrected by one exact
//    integer remainder test.
// Larger weights use the fp32 formula itself.
// The equality holds for the rule with IEEE fp32 division (the oracle's).
// The reference builds with -use_fast_math, whose '/' is an approximate
// division: an exact quotient such as 300 / 3 can come out just below the
// integer there and truncate one lower, so its GPU build may differ from
// this by 1 on such voxels.
__device__ __forceinline__ uint32_t blend_colour(uint32_t old_rgb, uint32_t new_rgb, float w_old,
                                                 float w_new, float rcp_new) {
  uint32_t out = 0;
  if (w_old <= 2047.0f) {  // rcp_new = 1 / w_new correctly rounded (within the bound above)
    const uint32_t wo = (uint32_t)w_old;
    const uint32_t m = __float2uint_rz(rcp_new * 4294969344.0f) + 1u;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const uint32_t n = ((old_rgb >> (8 * c)) & 0xFFu) * wo + ((new_rgb >> (8 * c)) & 0xFFu);
      out |= __umulhi(n, m) << (8 * c);
    }
    return wo ? out : new_rgb;
  }
  if (w_old <= 65536.0f) {
    const uint32_t wo = (uint32_t)w_old, wn = wo + 1u;
    const float r = __fdividef(1.0f, w_new);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const uint32_t n = ((old_rgb >> (8 * c)) & 0xFFu) * wo + ((new_rgb >> (8 * c)) & 0xFFu);
      uint32_t q = __float2uint_rz((float)n * r);
      const int rem = (int)(n - q * wn);
      q = rem < 0 ? q - 1u : (rem >= (int)wn ? q + 1u : q);
      out |= (q & 0xFFu) << (8 * c);
    }
  } else {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float old_c = (float)((old_rgb >> (8 * c)) & 0xFFu);
      const float new_c = (float)((new_rgb >> (8 * c)) & 0xFFu);
      const float v = (old_c * w_old + new_c) / w_new;
      out |= (__float2uint_rz(v) & 0xFFu) << (8 * c);
    }
  }
  return out;
}

// One voxel of IntegrateHashKernel (src/tsdf.cu:690-745), sdf averaged with
// the old weight.
// Projection of one voxel centre (base2cam src/tsdf.cu:81-93, cam2frame
// src/tsdf.cu:75-79): returns the pixel index or -1 (behind the camera or
// outside the image), and the camera-frame z.  Branch-free so that the
// pixel gathers of a thread's four voxels can be issued together.
__device__ __forceinline__ int project_voxel(const CamParams &C, const float P[12], float wx,
                                             float wy, float wz, float &z_out) {
  const float t0 = wx - P[3], t1 = wy - P[7], t2 = wz - P[11];
  float x = P[0] * t0;
  x = x + P[4] * t1;
  x = x + P[8] * t2;
  float y = P[1] * t0;
  y = y + P[5] * t1;
  y = y + P[9] * t2;
  float z = P[2] * t0;
  z = z + P[6] * t1;
  z = z + P[10] * t2;
  z_out = z;
  const float uf = roundf(C.fx * (x / z) + C.cx);
  const float vf = roundf(C.fy * (y / z) + C.cy);
  const bool ok = z > 0.0f && uf >= 0.0f && uf < C.wf && vf >= 0.0f && vf < C.hf;
  return ok ? (int)vf * C.width + (int)uf : -1;
}

// a / b from y = 1 / b correctly rounded: q = a y, then one exact residual
// correction q + (a - b q) y (Markstein's theorem: with y correctly rounded
// and q within an ulp of a / b the corrected quotient is the correctly
// rounded a / b, barring overflow and underflow; tests/markstein_check.c
// checks it exhaustively against IEEE division for the divisors and
// dividend ranges of the integration update).  A zero dividend gives +0,
// which is what IEEE division gives for the +0 dividends that occur here.
__device__ __forceinline__ float div_by_rcp(float a, float b, float y) {
  const float q = __fmul_rn(a, y);
  return __fmaf_rn(__fmaf_rn(-b, q, a), y, q);
}

// Update of one voxel from its pixel (src/tsdf.cu:715-745), sdf averaged
// with the old weight.  The two divisions are the IEEE quotients, taken
// from correctly rounded reciprocals of T (host) and of the weight (table).
__device__ __forceinline__ bool update_voxel(const CamParams &C, uint2 px, float z, float &sdf,
                                             float &wt, uint32_t &rgb) {
  const float d = __uint_as_float(px.x);
  if (!(d > 0.0f && d <= C.max_depth)) return false;
  const float diff = d - z;
  if (diff <= -C.trunc) return false;
  const float dist = fminf(1.0f, div_by_rcp(diff, C.trunc, C.rtrunc));  // diff / T
  const float w_old = wt;
  const float w_new = w_old + 1.0f;
  const float num = sdf * w_old + dist;
  float r = 0.0f;
  if (w_new <= (float)kRcpMax) {
    r = __ldg(C.rcp_w + (int)w_new);
    sdf = div_by_rcp(num, w_new, r);
  } else {
    sdf = num / w_new;
  }
  rgb = blend_colour(rgb, px.y, w_old, w_new, r);
  wt = w_new;
  return true;
}

// One thread's run of kV voxels along x (kV = 2, 4 or 8): project all,
// gather all pixels, then update.  Returns the number of voxels updated.
template <int kV>
__device__ __forceinline__ uint32_t update_run(const CamParams &C, const float P[12],
                                               const uint2 *__restrict__ pix, int ix, float wy,
                                               float wz, float (&sdf)[kV], float (&wt)[kV],
                                               uint32_t (&rgb)[kV], DevState *st) {
  float z[kV];
  int idx[kV];
#pragma unroll
  for (int k = 0; k < kV; ++k) idx[k] = project_voxel(C, P, (float)(ix + k) * C.voxel, wy, wz, z[k]);
  const uint2 none = make_uint2(0u, 0u);  // depth 0 = invalid
  uint2 px[kV];
#pragma unroll
  for (int k = 0; k < kV; ++k)
    px[k] = idx[k] >= 0 && VH_CHECK(st, idx[k] < C.width * C.height) ? __ldg(pix + idx[k]) : none;
  uint32_t n = 0;
#pragma unroll
  for (int k = 0; k < kV; ++k) n += update_voxel(C, px[k], z[k], sdf[k], wt[k], rgb[k]);
  return n;
}

// Word <-> value of the pool's 4-byte fields (sdf and weight floats, colour).
__device__ __forceinline__ void from_bits(uint32_t b, float &v) { v = __uint_as_float(b); }
__device__ __forceinline__ void from_bits(uint32_t b, uint32_t &v) { v = b; }
__device__ __forceinline__ uint32_t to_bits(float v) { return __float_as_uint(v); }
__device__ __forceinline__ uint32_t to_bits(uint32_t v) { return v; }

// kV consecutive words at p (p aligned to 4 kV bytes), with 16-byte
// accesses (8-byte for kV = 2).
template <int kV, typename T>
__device__ __forceinline__ void load_words(const T *__restrict__ p, T (&v)[kV]) {
  static_assert(sizeof(T) == 4 && (kV == 2 || kV == 4 || kV == 8), "2, 4 or 8 words");
  if constexpr (kV == 2) {
    const uint2 a = *reinterpret_cast<const uint2 *>(p);
    from_bits(a.x, v[0]);
    from_bits(a.y, v[1]);
  } else {
#pragma unroll
    for (int h = 0; h < kV / 4; ++h) {
      const uint4 a = reinterpret_cast<const uint4 *>(p)[h];
      from_bits(a.x, v[4 * h + 0]);
      from_bits(a.y, v[4 * h + 1]);
      from_bits(a.z, v[4 * h + 2]);
      from_bits(a.w, v[4 * h + 3]);
    }
  }
}
template <int kV, typename T>
__device__ __forceinline__ void store_words(T *__restrict__ p, const T (&v)[kV]) {
  if constexpr (kV == 2) {
    *reinterpret_cast<uint2 *>(p) = make_uint2(to_bits(v[0]), to_bits(v[1]));
  } else {
#pragma unroll
    for (int h = 0; h < kV / 4; ++h)
      reinterpret_cast<uint4 *>(p)[h] = make_uint4(to_bits(v[4 * h + 0]), to_bits(v[4 * h + 1]),
                                                   to_bits(v[4 * h + 2]), to_bits(v[4 * h + 3]));
  }
}

// The slot of frame-list entry i and thread t's run of kV voxels of the
// block (voxels kV t .. kV t + kV - 1).
template <int kV>
struct VoxelRun {
  unsigned long long key;
  uint32_t block;
  float sdf[kV], wt[kV];
  uint32_t rgb[kV];
};

template <int kV>
__device__ __forceinline__ void load_run(const VolumeView &V, uint32_t i, int t, VoxelRun<kV> &q) {
  const ulonglong2 r = __ldg(V.frame_res + i);
  q.key = r.x;
  q.block = (uint32_t)r.y;
  if (q.key >= kTombKey || q.block == kNoBlock) return;
  if (!VH_CHECK(V.st, q.block < V.pool_cap)) {
    q.block = kNoBlock;
    return;
  }
  const float *base = V.pool + (size_t)q.block * kBlockWords + kV * t;
  load_words<kV>(base, q.sdf);
  load_words<kV>(base + kB3, q.wt);
  load_words<kV>(reinterpret_cast<const uint32_t *>(base + 2 * kB3), q.rgb);
}

// Frame-list entry i whose run (thread t = threadIdx.x) is loaded in `cur`:
// every thread updates and stores its kV voxels.  Returns the number of
// voxels this thread updated.
template <int kV>
__device__ __forceinline__ uint32_t integrate_run(const VolumeView &V, const CamParams &C,
                                                  const float (&P)[12],
                                                  const uint2 *__restrict__ pix, uint32_t i,
                                                  VoxelRun<kV> &cur) {
  const int t = threadIdx.x;
  const int li = kV * t, x0 = li & 7, y = (li >> 3) & 7, z = li >> 6;
  const bool live = cur.key < kTombKey && cur.block != kNoBlock;
  if (!live) return 0;
  int bx, by, bz;
  unpack_key(cur.key, bx, by, bz);
  const float wy = (float)(by * kB + y) * C.voxel;
  const float wz = (float)(bz * kB + z) * C.voxel;
  const uint32_t nu =
      update_run<kV>(C, P, pix, bx * kB + x0, wy, wz, cur.sdf, cur.wt, cur.rgb, V.st);
  if (nu) {
    float *base = V.pool + (size_t)cur.block * kBlockWords + kV * t;
    store_words<kV>(base, cur.sdf);
    store_words<kV>(base + kB3, cur.wt);
    store_words<kV>(reinterpret_cast<uint32_t *>(base + 2 * kB3), cur.rgb);
  }
  return nu;
}

// Integration launch shapes (the tuning's integrate_variant): voxels per
// thread, whether the next block's voxels are loaded before the current
// block is computed (two blocks in flight per thread, more registers), and
// the resident CTAs per SM the register budget is set for.
//   0: 4 voxels x 128 threads, 12 CTAs per SM (40 registers)
//   1: 4 voxels x 128 threads, prefetch, 8 CTAs per SM (64 registers)
//   2: 8 voxels x  64 threads (a whole x row per thread), 16 CTAs per SM (64)
//   3: 2 voxels x 256 threads, 6 CTAs per SM (40)
//   4: 4 voxels x 128 threads, 10 CTAs per SM (48)
//   5: 8 voxels x  64 threads, 12 CTAs per SM (80)
constexpr int kIntegrateVariants = 6;
// Persistent CTAs of 512 / kV threads, one voxel block per iteration, kV
// voxels per thread.
template <int kV, bool kPrefetch, int kMinCtas>
__global__ void __launch_bounds__(kB3 / kV, kMinCtas) k_integrate(VolumeView V, CamParams C, const uint2 *__restrict__ pix,
                const float *__restrict__ pose) {
  const uint32_t n = min(V.st->frame_count, V.frame_cap);
  float P[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) P[k] = __ldg(pose + k);
  const int t = threadIdx.x;
  uint32_t updated = 0;
  uint32_t i = blockIdx.x;
  VoxelRun<kV> cur;
  if (kPrefetch && i < n) load_run<kV>(V, i, t, cur);
  for (; i < n; i += gridDim.x) {
    VoxelRun<kV> nxt;
    if (kPrefetch) {
      const uint32_t j = i + gridDim.x;
      if (j < n) load_run<kV>(V, j, t, nxt);
    } else {
      load_run<kV>(V, i, t, cur);
    }
    updated += integrate_run<kV>(V, C, P, pix, i, cur);
    if (kPrefetch) cur = nxt;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) updated += __shfl_xor_sync(kFull, updated, o);
  if ((t & 31) == 0 && updated) atomicAdd(&V.st->voxels_updated, (unsigned long long)updated);
}

// ---- marching cubes --------------------------------------------------------------
constexpr int kH = 9;              // staged edge: 8 voxels + 1 halo
constexpr int kH3 = kH * kH * kH;  // 729 staged corners
constexpr int kHalo = kH3 - kB3;   // 217
// Staged layout x + 9 y + 88 z: the z pitch is 8 (mod 32) banks, so the 32
// lanes of a warp, which classify 8 x by 4 z cubes of one y row, read 32
// distinct banks for every corner.
constexpr int kZPitch = 88;
constexpr int kStaged = kZPitch * kH;  // 792 words
constexpr int kMcThreads = 128;     // threads per CTA of the batched MC and MC variants 0, 1
constexpr int kMcMaxThreads = 256;  // largest MC CTA (variant 2)
constexpr int kMaxCand = kB3 * 5;  // at most 5 triangles per cube

struct McShared {
  float sdf[kStaged];  // NaN = corner unusable (absent block or low weight)
  uint32_t rgb[kStaged];
  uint16_t tri[256][5];  // triangle t of a case: edges e0 | e1 << 4 | e2 << 8
  uint16_t edge[256];
  uint8_t ntri[256];
  uint32_t einfo[12];    // per edge, see edge_info()
  uint8_t cases[kB3];        // cube case, 0 when the cube emits nothing
  uint16_t cand[kMaxCand];   // candidate triangles: cube | triangle << 9
  uint32_t halo[kHalo];      // halo voxel: staged index | neighbour << 10 | voxel << 13
  uint32_t nb[8];
  uint32_t warp_sum[kMcMaxThreads / 32];
  uint32_t base;
  uint32_t next[2];  // the block after the current one (double-buffered)
};

__device__ __forceinline__ int hidx(int x, int y, int z) { return x + kH * y + kZPitch * z; }

// Cube j (0 .. 512 / kThreads - 1) of thread t: a warp covers 8 x by 4 z
// cubes of one y row per j, x = t & 7, z = (t >> 3 & 3) + 4 (j / R),
// y = (t >> 5) + W (j % R) with W = kThreads / 32 warps and R = 8 / W;
// returns x + 8 y + 64 z.  All 512 cubes once.
template <int kThreads>
__device__ __forceinline__ int mc_cube(int t, int j) {
  constexpr int W = kThreads / 32, R = 8 / W;
  const int x = t & 7, z = ((t >> 3) & 3) + 4 * (j / R), y = (t >> 5) + W * (j % R);
  return x + 8 * y + 64 * z;
}
__device__ __forceinline__ int corner_dx(int k) { return (kMcCornerBitsX >> k) & 1; }
__device__ __forceinline__ int corner_dy(int k) { return (kMcCornerBitsY >> k) & 1; }
__device__ __forceinline__ int corner_dz(int k) { return (kMcCornerBitsZ >> k) & 1; }

// Per-edge constants, packed: staged-index offset of corner a (7 bits) and
// of corner b (7 bits), corner a's offset bits x | y << 1 | z << 2 (3 bits),
// the axis along which the edge runs (2 bits) and whether it runs towards
// -axis (1 bit).
__device__ __forceinline__ uint32_t edge_info(int e) {
  const uint32_t code =
      (uint32_t)((e < 8 ? kMcEdgeCodeLo >> (8 * e) : kMcEdgeCodeHi >> (8 * (e - 8))) & 0x3Fu);
  const int a = (int)(code & 7u), b = (int)(code >> 3);
  const int ax = corner_dx(a), ay = corner_dy(a), az = corner_dz(a);
  const int bx = corner_dx(b), by = corner_dy(b), bz = corner_dz(b);
  const uint32_t oa = (uint32_t)hidx(ax, ay, az), ob = (uint32_t)hidx(bx, by, bz);
  const uint32_t axis = bx != ax ? 0u : (by != ay ? 1u : 2u);
  const uint32_t neg = (bx - ax) + (by - ay) + (bz - az) < 0 ? 1u : 0u;
  return oa | (ob << 7) | ((uint32_t)(ax | (ay << 1) | (az << 2)) << 14) | (axis << 17) |
         (neg << 19);
}

// Vertex of edge e: VertexInterp(p[a], p[b], val[a], val[b])
// (src/tsdf.cu:1640-1660) in global voxel units; (gx, gy, gz) is the global
// voxel of staged corner 0.  Corners are one voxel apart along one axis, so
// p1 + mu * (p2 - p1) changes only that coordinate: the others are
// p1 + mu * 0 = p1 exactly (mu is finite and >= 0 on a cut edge).
// With `colour`, the colour is interpolated and truncated like the
// reference's float-to-uchar store.
template <bool colour>
__device__ __forceinline__ float4 mc_vertex(const McShared &S, int e, int h0, int gx, int gy,
                                           int gz) {
  const uint32_t info = S.einfo[e];
  const int ia = h0 + (int)(info & 127u), ib = h0 + (int)((info >> 7) & 127u);
  const float v1 = S.sdf[ia], v2 = S.sdf[ib];
  float p[3] = {(float)(gx + (int)((info >> 14) & 1u)), (float)(gy + (int)((info >> 15) & 1u)),
                (float)(gz + (int)((info >> 16) & 1u))};
  const int axis = (int)((info >> 17) & 3u);
  const float step = (info >> 19) ? -1.0f : 1.0f;  // p2 - p1 along the axis
  float mu = 0.0f;
  bool interp = false;
  bool to_b = false;
  if (fabsf(0.0f - v1) < kSnap) {
    // p1
  } else if (fabsf(0.0f - v2) < kSnap) {
    to_b = true;  // p2
  } else if (fabsf(v1 - v2) < kSnap) {
    // p1
  } else {
    mu = (0.0f - v1) / (v2 - v1);
    interp = true;
  }
  float moved = axis == 0 ? p[0] : (axis == 1 ? p[1] : p[2]);
  if (interp)
    moved = moved + mu * step;
  else if (to_b)
    moved = moved + step;
  const float px = axis == 0 ? moved : p[0];
  const float py = axis == 1 ? moved : p[1];
  const float pz = axis == 2 ? moved : p[2];
  uint32_t out = 0;
  if (colour) {
    const uint32_t c1 = S.rgb[ia], c2 = S.rgb[ib];
    if (!interp) {
      out = to_b ? c2 : c1;
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int q1 = (int)((c1 >> (8 * c)) & 0xFFu), q2 = (int)((c2 >> (8 * c)) & 0xFFu);
        const float v = (float)q1 + mu * (float)(q2 - q1);
        out |= (__float2uint_rz(v) & 0xFFu) << (8 * c);
      }
    }
  }
  return make_float4(px, py, pz, __uint_as_float(out));
}

// Cube case of the cube with staged corner 0 at (x, y, z); -1 if a corner is
// unusable (src/tsdf.cu:930-986).
__device__ __forceinline__ int cube_case(const McShared &S, int x, int y, int z) {
  int ci = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const float v = S.sdf[hidx(x + corner_dx(k), y + corner_dy(k), z + corner_dz(k))];
    if (v != v) return -1;
    if (v < 0.0f) ci |= 1 << k;
  }
  return ci;
}

__device__ __forceinline__ bool same_pos(const float4 &a, const float4 &b) {
  return a.x == b.x && a.y == b.y && a.z == b.z;
}

// Exclusive CTA-wide scan of `v`; returns the prefix, total in *total.
// Contains one __syncthreads; the caller separates consecutive scans.
template <int kThreads>
__device__ __forceinline__ uint32_t cta_scan(McShared &S, uint32_t v, uint32_t *total) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) S.warp_sum[warp] = incl;
  __syncthreads();
  uint32_t before = 0, tot = 0;
#pragma unroll
  for (int q = 0; q < kThreads / 32; ++q) {
    const uint32_t ws = S.warp_sum[q];
    before += q < warp ? ws : 0u;
    tot += ws;
  }
  *total = tot;
  return before + incl - v;
}

// Persistent CTAs, one block (plus its +x/+y/+z halo) per iteration:
//   stage 9^3 corners -> classify 512 cubes -> expand into candidate
//   triangles (scan) -> one thread per candidate tests the reference's
//   degenerate-triangle rule -> compact (scan) -> one atomic per block ->
//   one thread per output float4, contiguous stores.
// Tables and halo map of the MC shared state (once per CTA; any CTA size).
__device__ __forceinline__ void mc_init_shared(McShared &S) {
  const int t = threadIdx.x;
  for (int i = t; i < 256; i += blockDim.x) {
    S.edge[i] = kMcEdgeMask[i];
    int n = 0;
    for (; n < 5 && kMcTri[i][3 * n] >= 0; ++n)
      S.tri[i][n] = (uint16_t)(kMcTri[i][3 * n] | (kMcTri[i][3 * n + 1] << 4) |
                               (kMcTri[i][3 * n + 2] << 8));
    for (int m = n; m < 5; ++m) S.tri[i][m] = 0;
    S.ntri[i] = (uint8_t)n;
  }
  if (t < 12) S.einfo[t] = edge_info(t);
  // halo: x == 8 (81), then y == 8 with x < 8 (72), then z == 8 with x, y < 8 (64)
  for (int hh = t; hh < kHalo; hh += blockDim.x) {
    int x, y, z;
    if (hh < 81) {
      x = 8;
      y = hh % 9;
      z = hh / 9;
    } else if (hh < 153) {
      x = (hh - 81) & 7;
      y = 8;
      z = (hh - 81) >> 3;
    } else {
      x = (hh - 153) & 7;
      y = (hh - 153) >> 3;
      z = 8;
    }
    const uint32_t nbi = (uint32_t)((x >> 3) | ((y >> 3) << 1) | ((z >> 3) << 2));
    const uint32_t li = (uint32_t)((x & 7) + 8 * (y & 7) + 64 * (z & 7));
    S.halo[hh] = (uint32_t)hidx(x, y, z) | (nbi << 10) | (li << 13);
  }
}

// One block of the list (scope_all: pool block i; else frame-list entry i):
// stage, classify, expand, test, compact and write its triangles, with a
// CTA of kThreads (128 or 256) threads.  Every thread of the CTA calls it
// with the same i; S must be free on entry.
template <int kThreads>
__device__ __forceinline__ void mc_block(McShared &S, const VolumeView &V, int scope_all,
                                         float min_weight, float4 *__restrict__ tris,
                                         uint32_t tri_cap, uint32_t i) {
  const int t = threadIdx.x;
  const float nanv = __int_as_float(0x7FC00000);
  // Every thread reads the block's key and id itself (broadcast loads), so
  // the voxel loads below start without waiting for a barrier.
  unsigned long long key;
  uint32_t own;
  if (scope_all) {
    key = __ldg(V.block_keys + i);
    own = key < kTombKey ? i : kNoBlock;
  } else {
    const ulonglong2 r = __ldg(V.frame_res + i);
    key = r.x;
    own = key < kTombKey ? (uint32_t)r.y : kNoBlock;
  }
  if (own == kNoBlock) return;  // same entry for every thread: uniform
  if (!VH_CHECK(V.st, own < V.pool_cap)) return;  // uniform as well
  int bx, by, bz;
  unpack_key(key, bx, by, bz);
  if (scope_all && t < 8) {
    const int nx = bx + (t & 1), ny = by + ((t >> 1) & 1), nz = bz + (t >> 2);
    S.nb[t] = t == 0 ? own
                     : (key_in_range(nx, ny, nz) ? block_of(V, pack_key(nx, ny, nz)) : kNoBlock);
  }
  {  // own block: kV voxels per thread, 16-byte (kV = 4) or 8-byte loads
    constexpr int kV = kB3 / kThreads;
    const int li = kV * t, x = li & 7, y = (li >> 3) & 7, z = li >> 6;
    const float *base = V.pool + (size_t)own * kBlockWords + li;
    float sd[kV], wt[kV];
    uint32_t cl[kV];
    load_words<kV>(base, sd);
    load_words<kV>(base + kB3, wt);
    load_words<kV>(reinterpret_cast<const uint32_t *>(base + 2 * kB3), cl);
    const int h = hidx(x, y, z);
#pragma unroll
    for (int k = 0; k < kV; ++k) {
      S.sdf[h + k] = wt[k] >= min_weight ? sd[k] : nanv;
      S.rgb[h + k] = cl[k];
    }
  }
  if (scope_all) __syncthreads();  // S.nb complete (uniform condition)
  {  // halo: every thread owns at most two entries (128 threads: t and
     // t + 128; 256 threads: t only, none from t = kHalo on); all loads
     // issued together
    const int h1 = t + kThreads;
    const bool has0 = kThreads <= kHalo || t < kHalo;
    const uint32_t info0 = has0 ? S.halo[t] : 0u;
    const uint32_t info1 = h1 < kHalo ? S.halo[h1] : 0u;
    const uint32_t nb0 = (info0 >> 10) & 7u, nb1 = (info1 >> 10) & 7u;
    uint32_t blk0 = scope_all ? S.nb[nb0] : __ldg(V.frame_nb + 8 * (size_t)i + nb0);
    uint32_t blk1 = scope_all ? S.nb[nb1] : __ldg(V.frame_nb + 8 * (size_t)i + nb1);
    if (!has0) blk0 = kNoBlock;
    if (h1 >= kHalo) blk1 = kNoBlock;
    if (!VH_CHECK(V.st, blk0 == kNoBlock || blk0 < V.pool_cap)) blk0 = kNoBlock;
    if (!VH_CHECK(V.st, blk1 == kNoBlock || blk1 < V.pool_cap)) blk1 = kNoBlock;
    const int li0 = (int)(info0 >> 13), li1 = (int)(info1 >> 13);
    float w0 = 0.f, s0 = nanv, w1 = 0.f, s1 = nanv;
    uint32_t c0 = 0, c1 = 0;
    if (blk0 != kNoBlock) {
      const float *base = V.pool + (size_t)blk0 * kBlockWords;
      w0 = __ldg(base + kB3 + li0);
      s0 = __ldg(base + li0);
      c0 = __ldg(reinterpret_cast<const uint32_t *>(base + 2 * kB3) + li0);
    }
    if (blk1 != kNoBlock) {
      const float *base = V.pool + (size_t)blk1 * kBlockWords;
      w1 = __ldg(base + kB3 + li1);
      s1 = __ldg(base + li1);
      c1 = __ldg(reinterpret_cast<const uint32_t *>(base + 2 * kB3) + li1);
    }
    if (has0) {
      S.sdf[info0 & 1023u] = blk0 != kNoBlock && w0 >= min_weight ? s0 : nanv;
      S.rgb[info0 & 1023u] = c0;
    }
    if (h1 < kHalo) {
      S.sdf[info1 & 1023u] = blk1 != kNoBlock && w1 >= min_weight ? s1 : nanv;
      S.rgb[info1 & 1023u] = c1;
    }
  }
  __syncthreads();
  // 1. classify this thread's cubes; count their candidate triangles
  constexpr int kCubes = kB3 / kThreads;
  uint32_t ncand_mine = 0;
  int cs[kCubes];
#pragma unroll
  for (int j = 0; j < kCubes; ++j) {
    const int c = mc_cube<kThreads>(t, j);
    int ci = cube_case(S, c & 7, (c >> 3) & 7, c >> 6);
    if (ci < 0 || S.edge[ci] == 0) ci = 0;
    cs[j] = ci;
    S.cases[c] = (uint8_t)ci;
    ncand_mine += S.ntri[ci];
  }
  uint32_t ncand;
  uint32_t off = cta_scan<kThreads>(S, ncand_mine, &ncand);
  if (ncand == 0) return;  // uniform: nothing to emit in this block
#pragma unroll
  for (int j = 0; j < kCubes; ++j) {
    const int c = mc_cube<kThreads>(t, j);
    const int nt = S.ntri[cs[j]];
    for (int tt = 0; tt < nt; ++tt) S.cand[off++] = (uint16_t)(c | (tt << 9));
  }
  __syncthreads();
  // 2. candidates in rounds of one per thread: the thread computes its
  //    candidate's three vertices once, the reference's degenerate test
  //    drops p0 == p1 || p1 == p2 (src/tsdf.cu:1055-1057), a CTA scan over
  //    the survivors gives each a slot in one contiguous range reserved
  //    with a single atomic, and the thread writes its 48-byte triangle.
  const int gx0 = bx * kB, gy0 = by * kB, gz0 = bz * kB;
  for (uint32_t r0 = 0; r0 < ncand; r0 += kThreads) {
    const uint32_t k = r0 + t;
    float4 p0, p1, p2;
    uint32_t ok = 0;
    if (k < ncand) {
      const uint32_t ent = S.cand[k];
      const int c = (int)(ent & 511u), tt = (int)(ent >> 9);
      const int x = c & 7, y = (c >> 3) & 7, z = c >> 6;
      const uint32_t tri = S.tri[S.cases[c]][tt];
      const int h0 = hidx(x, y, z);
      p0 = mc_vertex<true>(S, (int)(tri & 15u), h0, gx0 + x, gy0 + y, gz0 + z);
      p1 = mc_vertex<true>(S, (int)((tri >> 4) & 15u), h0, gx0 + x, gy0 + y, gz0 + z);
      p2 = mc_vertex<true>(S, (int)(tri >> 8), h0, gx0 + x, gy0 + y, gz0 + z);
      ok = !(same_pos(p0, p1) || same_pos(p1, p2));
    }
    uint32_t nvalid;
    const uint32_t pre = cta_scan<kThreads>(S, ok, &nvalid);
    if (t == 0) S.base = nvalid ? atomicAdd(&V.st->tri_count, nvalid) : 0u;
    __syncthreads();
    if (ok) {
      const uint32_t out = S.base + pre;
      if (out < tri_cap) {
        float4 *dst = tris + 3 * (size_t)out;
        dst[0] = p0;
        dst[1] = p1;
        dst[2] = p2;
      } else {
        atomicOr(&V.st->error, kErrTriCap);
      }
    }
  }
}

template <int kThreads, int kMinCtas>
__global__ void __launch_bounds__(kThreads, kMinCtas) k_mc(VolumeView V, int scope_all, float min_weight,
                                                      float4 *__restrict__ tris, uint32_t tri_cap,
                                                      DevState *host_state) {
  __shared__ McShared S;
  mc_init_shared(S);
  const uint32_t n = scope_all ? V.st->pool_top : min(V.st->frame_count, V.frame_cap);
  // A block emits anything from nothing to hundreds of triangles, so blocks
  // are handed out dynamically: a CTA's first block is its index, every
  // further one comes from a counter, fetched while the current block is
  // processed so the atomic's latency stays hidden.
  __syncthreads();
  uint32_t i = blockIdx.x;
  for (int par = 0; i < n; par ^= 1) {
    if (threadIdx.x == 0) S.next[par] = gridDim.x + atomicAdd(&V.st->mc_next, 1u);
    mc_block<kThreads>(S, V, scope_all, min_weight, tris, tri_cap, i);
    __syncthreads();  // S.next[par] visible; this block done with S
    i = S.next[par];
  }
  if (host_state) {  // the last CTA to finish copies the counters out
    __shared__ int last_cta;
    if (threadIdx.x == 0) {
      __threadfence();  // this CTA's counter updates before its arrival
      last_cta = atomicAdd(&V.st->mc_done, 1u) == gridDim.x - 1u;
    }
    __syncthreads();
    if (last_cta && threadIdx.x < 32) {
      if (threadIdx.x == 0) {
        __threadfence();
        V.st->mc_done = 0u;
      }
      __syncwarp();
      static_assert(sizeof(DevState) % 4 == 0 && sizeof(DevState) / 4 <= 32, "one warp");
      if (threadIdx.x < sizeof(DevState) / 4)
        reinterpret_cast<volatile uint32_t *>(host_state)[threadIdx.x] =
            reinterpret_cast<volatile const uint32_t *>(V.st)[threadIdx.x];
    }
  }
}

// ---- marching cubes into an indexed mesh (shared vertices per block) ----------
// The frame's mesh as vertices + faces instead of a triangle soup: per block
// every cut lattice edge is interpolated once (in both directions where the
// reference's corner order runs it both ways, a separate vertex only where
// the two results differ in a bit), the vertices are written once, and each
// triangle is three vertex numbers.  The triangles are exactly those of k_mc
// (same vertices bit for bit, same degenerate test); a vertex shared by
// cubes of two blocks is written by each block.
constexpr int kRows = kH * kH;         // corner rows (y, z), y and z in 0..8
constexpr int kEdgeRows = 3 * kRows;   // lattice-edge rows: axis * 81 + y + 9 z
// Capacities of one pass over a block.  A block whose cube cases need more
// is processed again in 8 passes of one cube layer each (at most 320
// triangles and 369 cut edges per layer), so no block is ever dropped.
constexpr int kICandCap = 1536;  // candidate triangles per pass
constexpr int kIEdgeCap = 512;   // cut lattice edges per pass
constexpr int kISlots = kIEdgeCap / kMcThreads;  // edge slots per thread

struct McIdxShared {
  float sdf[kStaged];  // NaN = corner unusable (absent block or low weight)
  uint32_t rgb[kStaged];
  // corner row (y, z): bit x (0..8) = sdf < 0, bit 16 + x = unusable
  uint32_t row[kRows];
  // lattice-edge row: bit x = the edge from corner (x, y, z) one voxel along
  // the row's axis is cut (both corners usable, signs differ)
  uint16_t cut[kEdgeRows];
  uint16_t first[kEdgeRows];  // slot of the row's first cut edge
  uint16_t elist[kIEdgeCap];  // cut edge of a slot: x | y << 4 | z << 8 | axis << 12
  // slot: the edge's vertex towards +axis and towards -axis (moved
  // coordinate, global voxel units) and their colours
  float4 vert[kIEdgeCap];
  // slot: block-local number of its +axis vertex; bit 15 set when the
  // -axis vertex differs and has the next number
  uint16_t vid[kIEdgeCap];
  uint16_t tri[256][5];  // triangle t of a case: edges e0 | e1 << 4 | e2 << 8
  uint16_t edge[256];
  uint8_t ntri[256];
  uint8_t einfo[12];          // per cube edge, see lattice_edge_info()
  uint8_t cases[kB3];         // cube case, 0 when the cube emits nothing
  uint16_t cand[kICandCap];   // candidate triangles: cube | triangle << 9
  uint32_t halo[kHalo];       // halo voxel: staged index | neighbour << 10 | voxel << 13
  uint32_t warp_sum[kMcThreads / 32];
  uint32_t vbase, fbase;
  uint32_t next[2];  // the block after the current one (double-buffered)
};

// Cube edge e as a lattice edge: the offset bits x | y << 1 | z << 2 of its
// lower corner (the smaller coordinate along the edge), the axis along which
// it runs (bits 3-4) and whether the reference's corner order runs it
// towards -axis (bit 5: from the upper to the lower corner).
__device__ __forceinline__ uint32_t lattice_edge_info(int e) {
  const uint32_t code =
      (uint32_t)((e < 8 ? kMcEdgeCodeLo >> (8 * e) : kMcEdgeCodeHi >> (8 * (e - 8))) & 0x3Fu);
  const int a = (int)(code & 7u), b = (int)(code >> 3);
  const int ax = corner_dx(a), ay = corner_dy(a), az = corner_dz(a);
  const int bx = corner_dx(b), by = corner_dy(b), bz = corner_dz(b);
  const uint32_t axis = bx != ax ? 0u : (by != ay ? 1u : 2u);
  const uint32_t neg = (bx - ax) + (by - ay) + (bz - az) < 0 ? 1u : 0u;
  const uint32_t lower = (uint32_t)((ax & bx) | ((ay & by) << 1) | ((az & bz) << 2));
  return lower | (axis << 3) | (neg << 5);
}

// VertexInterp(p1, p2, val1, val2) (src/tsdf.cu:1640-1660) for corners one
// voxel apart along one axis: only that coordinate moves, from p (p1's) by
// step = p2 - p1 = +-1; the colour is interpolated and truncated like the
// reference's float-to-uchar store.  The same arithmetic as mc_vertex.
__device__ __forceinline__ void interp_edge(float p, float step, float v1, float v2, uint32_t c1,
                                            uint32_t c2, float &moved, uint32_t &col) {
  float mu = 0.0f;
  bool interp = false;
  bool to_b = false;
  if (fabsf(0.0f - v1) < kSnap) {
    // p1
  } else if (fabsf(0.0f - v2) < kSnap) {
    to_b = true;  // p2
  } else if (fabsf(v1 - v2) < kSnap) {
    // p1
  } else {
    mu = (0.0f - v1) / (v2 - v1);
    interp = true;
  }
  moved = p;
  if (interp)
    moved = moved + mu * step;
  else if (to_b)
    moved = moved + step;
  if (!interp) {
    col = to_b ? c2 : c1;
    return;
  }
  uint32_t out = 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int q1 = (int)((c1 >> (8 * c)) & 0xFFu), q2 = (int)((c2 >> (8 * c)) & 0xFFu);
    const float v = (float)q1 + mu * (float)(q2 - q1);
    out |= (__float2uint_rz(v) & 0xFFu) << (8 * c);
  }
  col = out;
}

__device__ __forceinline__ void mci_init_shared(McIdxShared &S) {
  const int t = threadIdx.x;
  for (int i = t; i < 256; i += kMcThreads) {
    S.edge[i] = kMcEdgeMask[i];
    int n = 0;
    for (; n < 5 && kMcTri[i][3 * n] >= 0; ++n)
      S.tri[i][n] = (uint16_t)(kMcTri[i][3 * n] | (kMcTri[i][3 * n + 1] << 4) |
                               (kMcTri[i][3 * n + 2] << 8));
    for (int m = n; m < 5; ++m) S.tri[i][m] = 0;
    S.ntri[i] = (uint8_t)n;
  }
  if (t < 12) S.einfo[t] = (uint8_t)lattice_edge_info(t);
  // halo: x == 8 (81), then y == 8 with x < 8 (72), then z == 8 with x, y < 8 (64)
  for (int hh = t; hh < kHalo; hh += kMcThreads) {
    int x, y, z;
    if (hh < 81) {
      x = 8;
      y = hh % 9;
      z = hh / 9;
    } else if (hh < 153) {
      x = (hh - 81) & 7;
      y = 8;
      z = (hh - 81) >> 3;
    } else {
      x = (hh - 153) & 7;
      y = (hh - 153) >> 3;
      z = 8;
    }
    const uint32_t nbi = (uint32_t)((x >> 3) | ((y >> 3) << 1) | ((z >> 3) << 2));
    const uint32_t li = (uint32_t)((x & 7) + 8 * (y & 7) + 64 * (z & 7));
    S.halo[hh] = (uint32_t)hidx(x, y, z) | (nbi << 10) | (li << 13);
  }
}

// Cut-edge mask of lattice-edge row r (axis * 81 + y + 9 z) among the edges
// that the cubes of layers [z0, z1) use.
__device__ __forceinline__ uint32_t edge_row_mask(const McIdxShared &S, int r, int z0, int z1) {
  const int axis = r / kRows, rr = r - axis * kRows;
  const int y = rr % kH, z = rr / kH;
  const uint32_t w = S.row[rr];
  const uint32_t n = w & 0x1FFu, q = w >> 16;
  if (axis == 0) {  // x edges of layer z are used by cubes z - 1 and z
    if (z < z0 || z > z1) return 0u;
    return (n ^ (n >> 1)) & ~(q | (q >> 1)) & 0xFFu;
  }
  if (axis == 1) {
    if (y == 8 || z < z0 || z > z1) return 0u;
    const uint32_t w2 = S.row[rr + 1];
    return (n ^ w2) & ~(q | (w2 >> 16)) & 0x1FFu;
  }
  if (z == 8 || z < z0 || z >= z1) return 0u;  // z edges of layer z: cubes of layer z
  const uint32_t w2 = S.row[rr + kH];
  return (n ^ w2) & ~(q | (w2 >> 16)) & 0x1FFu;
}

// Cube cases of cubes (x0 .. x0 + 3, y, z) from the corner-row words: bit k
// of a case is corner k's sign (corner order of src/tsdf.cu's idxMap), 0
// for a cube with an unusable corner or no cut edge (src/tsdf.cu:930-986).
__device__ __forceinline__ void classify4(const McIdxShared &S, int x0, int y, int z, int cs[4]) {
  const uint32_t A = S.row[y + kH * z], B = S.row[y + 1 + kH * z];
  const uint32_t C = S.row[y + kH * (z + 1)], D = S.row[y + 1 + kH * (z + 1)];
  const uint32_t bad = (A | B | C | D) >> 16;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int x = x0 + j;
    const uint32_t a = (A >> x) & 3u, b = (B >> x) & 3u, c = (C >> x) & 3u, d = (D >> x) & 3u;
    // corners 0 (0,0,0) 3 (1,0,0) | 1 (0,1,0) 2 (1,1,0) | 4 (0,0,1) 7 (1,0,1) | 5 (0,1,1) 6 (1,1,1)
    int ci = (int)((a & 1u) | ((a & 2u) << 2) | (b << 1) | ((c & 1u) << 4) | ((c & 2u) << 6) |
                   (d << 5));
    if (((bad >> x) & 3u) || S.edge[ci] == 0) ci = 0;
    cs[j] = ci;
  }
}

// Exclusive CTA-wide scan for McIdxShared (as cta_scan): one __syncthreads.
__device__ __forceinline__ uint32_t cta_scan_idx(McIdxShared &S, uint32_t v, uint32_t *total) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) S.warp_sum[warp] = incl;
  __syncthreads();
  uint32_t before = 0, tot = 0;
#pragma unroll
  for (int q = 0; q < kMcThreads / 32; ++q) {
    const uint32_t ws = S.warp_sum[q];
    before += q < warp ? ws : 0u;
    tot += ws;
  }
  *total = tot;
  return before + incl - v;
}

// Frame-list entry i: stage the block and its halo, then per pass classify,
// list cut edges, interpolate each once, number and write the vertices
// (one atomic per pass), and write the surviving triangles as vertex
// numbers (one atomic per round).  S must be free on entry.
__device__ __forceinline__ void mci_block(McIdxShared &S, const VolumeView &V, float min_weight,
                                          float4 *__restrict__ verts, uint32_t vcap,
                                          int32_t *__restrict__ faces, uint32_t fcap, uint32_t i) {
  const int t = threadIdx.x;
  const float nanv = __int_as_float(0x7FC00000);
  const ulonglong2 res = __ldg(V.frame_res + i);
  const unsigned long long key = res.x;
  const uint32_t own = key < kTombKey ? (uint32_t)res.y : kNoBlock;
  if (own == kNoBlock) return;  // same entry for every thread: uniform
  if (!VH_CHECK(V.st, own < V.pool_cap)) return;  // uniform as well
  int bx, by, bz;
  unpack_key(key, bx, by, bz);
  {  // own block: 4 voxels per thread, 16-byte loads
    const float *base = V.pool + (size_t)own * kBlockWords;
    const float4 sd = reinterpret_cast<const float4 *>(base)[t];
    const float4 wt = reinterpret_cast<const float4 *>(base + kB3)[t];
    const uint4 cl = reinterpret_cast<const uint4 *>(base + 2 * kB3)[t];
    const int li = 4 * t, x = li & 7, y = (li >> 3) & 7, z = li >> 6;
    const int h = hidx(x, y, z);
    S.sdf[h + 0] = wt.x >= min_weight ? sd.x : nanv;
    S.sdf[h + 1] = wt.y >= min_weight ? sd.y : nanv;
    S.sdf[h + 2] = wt.z >= min_weight ? sd.z : nanv;
    S.sdf[h + 3] = wt.w >= min_weight ? sd.w : nanv;
    S.rgb[h + 0] = cl.x;
    S.rgb[h + 1] = cl.y;
    S.rgb[h + 2] = cl.z;
    S.rgb[h + 3] = cl.w;
  }
  {  // halo: every thread owns at most two entries; all loads issued together
    const int h1 = t + kMcThreads;
    const uint32_t info0 = S.halo[t];
    const uint32_t info1 = h1 < kHalo ? S.halo[h1] : 0u;
    const uint32_t nb0 = (info0 >> 10) & 7u, nb1 = (info1 >> 10) & 7u;
    uint32_t blk0 = __ldg(V.frame_nb + 8 * (size_t)i + nb0);
    uint32_t blk1 = h1 < kHalo ? __ldg(V.frame_nb + 8 * (size_t)i + nb1) : kNoBlock;
    if (!VH_CHECK(V.st, blk0 == kNoBlock || blk0 < V.pool_cap)) blk0 = kNoBlock;
    if (!VH_CHECK(V.st, blk1 == kNoBlock || blk1 < V.pool_cap)) blk1 = kNoBlock;
    const int li0 = (int)(info0 >> 13), li1 = (int)(info1 >> 13);
    float w0 = 0.f, s0 = nanv, w1 = 0.f, s1 = nanv;
    uint32_t c0 = 0, c1 = 0;
    if (blk0 != kNoBlock) {
      const float *base = V.pool + (size_t)blk0 * kBlockWords;
      w0 = __ldg(base + kB3 + li0);
      s0 = __ldg(base + li0);
      c0 = __ldg(reinterpret_cast<const uint32_t *>(base + 2 * kB3) + li0);
    }
    if (blk1 != kNoBlock) {
      const float *base = V.pool + (size_t)blk1 * kBlockWords;
      w1 = __ldg(base + kB3 + li1);
      s1 = __ldg(base + li1);
      c1 = __ldg(reinterpret_cast<const uint32_t *>(base + 2 * kB3) + li1);
    }
    S.sdf[info0 & 1023u] = blk0 != kNoBlock && w0 >= min_weight ? s0 : nanv;
    S.rgb[info0 & 1023u] = c0;
    if (h1 < kHalo) {
      S.sdf[info1 & 1023u] = blk1 != kNoBlock && w1 >= min_weight ? s1 : nanv;
      S.rgb[info1 & 1023u] = c1;
    }
  }
  __syncthreads();
  if (t < kRows) {  // corner-row words: sign and unusable bits of 9 corners
    const float *r = S.sdf + hidx(0, t % kH, t / kH);
    uint32_t w = 0;
#pragma unroll
    for (int x = 0; x < kH; ++x) {
      const float v = r[x];
      w |= (v < 0.0f ? 1u : 0u) << x;
      w |= (v != v ? 1u : 0u) << (16 + x);
    }
    S.row[t] = w;
  }
  __syncthreads();

  const int cy = (t >> 1) & 7, cz = t >> 4, cx0 = (t & 1) * 4;  // this thread's 4 cubes
  const int gx0 = bx * kB, gy0 = by * kB, gz0 = bz * kB;
  int z0 = 0, z1 = kB;
  bool layered = false;
  for (;;) {
    // 1. classify this thread's cubes and the cut masks of its edge rows
    int cs[4];
    classify4(S, cx0, cy, cz, cs);
    uint32_t ntri_mine = 0;
    const bool in_pass = cz >= z0 && cz < z1;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!in_pass) cs[j] = 0;
      S.cases[cx0 + j + kB * cy + kB * kB * cz] = (uint8_t)cs[j];
      ntri_mine += S.ntri[cs[j]];
    }
    const int r1 = t + kMcThreads;
    const uint32_t m0 = edge_row_mask(S, t, z0, z1);
    const uint32_t m1 = r1 < kEdgeRows ? edge_row_mask(S, r1, z0, z1) : 0u;
    const uint32_t ncut_mine = (uint32_t)(__popc(m0) + __popc(m1));
    uint32_t tot;
    const uint32_t off = cta_scan_idx(S, ntri_mine | (ncut_mine << 16), &tot);
    const uint32_t ncand = tot & 0xFFFFu, ncut = tot >> 16;
    if (!layered && (ncand > (uint32_t)kICandCap || ncut > (uint32_t)kIEdgeCap)) {
      layered = true;  // uniform: start again one layer at a time
      z1 = 1;
      __syncthreads();  // warp sums read before the next scan
      continue;
    }
    if (ncand) {
      // 2. expand candidate triangles and list the cut edges (slot order)
      uint32_t ct = off & 0xFFFFu;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = cx0 + j + kB * cy + kB * kB * cz;
        const int nt = S.ntri[cs[j]];
        for (int tt = 0; tt < nt; ++tt) S.cand[ct++] = (uint16_t)(c | (tt << 9));
      }
      uint32_t se = off >> 16;
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const int r = k ? r1 : t;
        if (r >= kEdgeRows) break;
        uint32_t m = k ? m1 : m0;
        S.cut[r] = (uint16_t)m;
        S.first[r] = (uint16_t)se;
        const int axis = r / kRows, rr = r - axis * kRows;
        const uint32_t yz = (uint32_t)((rr % kH) << 4 | (rr / kH) << 8 | axis << 12);
        while (m) {
          const int x = __ffs(m) - 1;
          m &= m - 1u;
          S.elist[se++] = (uint16_t)(yz | (uint32_t)x);
        }
      }
      __syncthreads();
      // 3. this thread's slots [kISlots t, kISlots t + kISlots): the vertex
      //    towards +axis VertexInterp(lower, upper) and towards -axis
      //    VertexInterp(upper, lower) (z edges are only run upwards); a
      //    separate -axis vertex only where the two differ
      uint32_t two = 0, nv_mine = 0;
#pragma unroll
      for (int j = 0; j < kISlots; ++j) {
        const uint32_t s = (uint32_t)(kISlots * t + j);
        if (s >= ncut) break;
        const uint32_t ent = S.elist[s];
        const int x = (int)(ent & 15u), y = (int)((ent >> 4) & 15u), z = (int)((ent >> 8) & 15u);
        const int axis = (int)(ent >> 12);
        const int lo = hidx(x, y, z);
        const int hi = lo + (axis == 0 ? 1 : (axis == 1 ? kH : kZPitch));
        const float vl = S.sdf[lo], vh = S.sdf[hi];
        const uint32_t cl = S.rgb[lo], ch = S.rgb[hi];
        const int g = axis == 0 ? gx0 + x : (axis == 1 ? gy0 + y : gz0 + z);
        float up, down = 0.0f;
        uint32_t cup, cdown = 0u;
        interp_edge((float)g, 1.0f, vl, vh, cl, ch, up, cup);
        bool sep = false;
        if (axis != 2) {
          interp_edge((float)(g + 1), -1.0f, vh, vl, ch, cl, down, cdown);
          sep = __float_as_uint(down) != __float_as_uint(up) || cdown != cup;
        }
        S.vert[s] = make_float4(up, down, __uint_as_float(cup), __uint_as_float(cdown));
        two |= (sep ? 1u : 0u) << j;
        nv_mine += sep ? 2u : 1u;
      }
      uint32_t nv;
      uint32_t local = cta_scan_idx(S, nv_mine, &nv);
#pragma unroll
      for (int j = 0; j < kISlots; ++j) {
        const uint32_t s = (uint32_t)(kISlots * t + j);
        if (s >= ncut) break;
        const uint32_t sep = (two >> j) & 1u;
        S.vid[s] = (uint16_t)(local | (sep << 15));
        local += 1u + sep;
      }
      if (t == 0) S.vbase = atomicAdd(&V.st->vert_count, nv);
      __syncthreads();
      // 4. the vertices, at vbase + their block-local numbers
      const uint32_t vbase = S.vbase;
#pragma unroll
      for (int j = 0; j < kISlots; ++j) {
        const uint32_t s = (uint32_t)(kISlots * t + j);
        if (s >= ncut) break;
        const uint32_t ent = S.elist[s];
        const int x = (int)(ent & 15u), y = (int)((ent >> 4) & 15u), z = (int)((ent >> 8) & 15u);
        const int axis = (int)(ent >> 12);
        const float4 sv = S.vert[s];
        const float px = (float)(gx0 + x), py = (float)(gy0 + y), pz = (float)(gz0 + z);
        const uint32_t vv = S.vid[s];
        const uint32_t o = vbase + (vv & 0x7FFFu);
        const uint32_t nvs = (vv >> 15) ? 2u : 1u;
        if (o + nvs <= vcap) {
          verts[o] = make_float4(axis == 0 ? sv.x : px, axis == 1 ? sv.x : py,
                                 axis == 2 ? sv.x : pz, sv.z);
          if (nvs == 2u)
            verts[o + 1] = make_float4(axis == 0 ? sv.y : px, axis == 1 ? sv.y : py, pz, sv.w);
        } else {
          atomicOr(&V.st->error, kErrTriCap);
        }
      }
      // 5. candidates in rounds of one per thread: the three vertices from
      //    the slots, the reference's degenerate test (p0 == p1 || p1 == p2,
      //    src/tsdf.cu:1055-1057), a CTA scan over the survivors, one atomic
      //    per round, each survivor's three vertex numbers
      for (uint32_t q0 = 0; q0 < ncand; q0 += kMcThreads) {
        const uint32_t k = q0 + (uint32_t)t;
        float4 p[3];
        uint32_t id[3] = {0u, 0u, 0u};
        uint32_t ok = 0;
        if (k < ncand) {
          const uint32_t ent = S.cand[k];
          const int c = (int)(ent & 511u), tt = (int)(ent >> 9);
          const int x = c & 7, y = (c >> 3) & 7, z = c >> 6;
          const uint32_t tri = S.tri[S.cases[c]][tt];
#pragma unroll
          for (int v = 0; v < 3; ++v) {
            const uint32_t info = S.einfo[(tri >> (4 * v)) & 15u];
            const int lx = x + (int)(info & 1u), ly = y + (int)((info >> 1) & 1u),
                      lz = z + (int)((info >> 2) & 1u);
            const int axis = (int)((info >> 3) & 3u);
            const int r = axis * kRows + ly + kH * lz;
            const uint32_t slot = S.first[r] + (uint32_t)__popc(S.cut[r] & ((1u << lx) - 1u));
            const float4 sv = S.vert[slot];
            const bool down = (info >> 5) & 1u;
            const float moved = down ? sv.y : sv.x;
            p[v] = make_float4(axis == 0 ? moved : (float)(gx0 + lx),
                               axis == 1 ? moved : (float)(gy0 + ly),
                               axis == 2 ? moved : (float)(gz0 + lz), 0.0f);
            const uint32_t vv = S.vid[slot];
            id[v] = vbase + (vv & 0x7FFFu) + ((down && (vv >> 15)) ? 1u : 0u);
          }
          ok = !(same_pos(p[0], p[1]) || same_pos(p[1], p[2]));
        }
        uint32_t nvalid;
        const uint32_t pre = cta_scan_idx(S, ok, &nvalid);
        if (t == 0) S.fbase = nvalid ? atomicAdd(&V.st->tri_count, nvalid) : 0u;
        __syncthreads();
        if (ok) {
          const uint32_t out = S.fbase + pre;
          if (out < fcap) {
            int32_t *dst = faces + 3 * (size_t)out;
            dst[0] = (int32_t)id[0];
            dst[1] = (int32_t)id[1];
            dst[2] = (int32_t)id[2];
          } else {
            atomicOr(&V.st->error, kErrTriCap);
          }
        }
      }
    }
    if (!layered || z1 == kB) return;
    __syncthreads();  // this layer's slots, lists and warp sums are free
    ++z0;
    ++z1;
  }
}

// Persistent CTAs over the frame list, blocks handed out by a counter as in
// k_mc; the last CTA to finish copies the counters to host_state.
__global__ void __launch_bounds__(kMcThreads, 8)
    k_mc_indexed(VolumeView V, float min_weight, float4 *__restrict__ verts, uint32_t vcap,
                 int32_t *__restrict__ faces, uint32_t fcap, DevState *host_state) {
  __shared__ McIdxShared S;
  mci_init_shared(S);
  const uint32_t n = min(V.st->frame_count, V.frame_cap);
  __syncthreads();
  uint32_t i = blockIdx.x;
  for (int par = 0; i < n; par ^= 1) {
    if (threadIdx.x == 0) S.next[par] = gridDim.x + atomicAdd(&V.st->mc_next, 1u);
    mci_block(S, V, min_weight, verts, vcap, faces, fcap, i);
    __syncthreads();  // S.next[par] visible; this block done with S
    i = S.next[par];
  }
  if (host_state) {  // the last CTA to finish copies the counters out
    __shared__ int last_cta;
    if (threadIdx.x == 0) {
      __threadfence();
      last_cta = atomicAdd(&V.st->mc_done, 1u) == gridDim.x - 1u;
    }
    __syncthreads();
    if (last_cta && threadIdx.x < 32) {
      if (threadIdx.x == 0) {
        __threadfence();
        V.st->mc_done = 0u;
      }
      __syncwarp();
      if (threadIdx.x < sizeof(DevState) / 4)
        reinterpret_cast<volatile uint32_t *>(host_state)[threadIdx.x] =
            reinterpret_cast<volatile const uint32_t *>(V.st)[threadIdx.x];
    }
  }
}

// ---- small state kernels --------------------------------------------------------
__device__ __forceinline__ void reconcile(const VolumeView &V) { reconcile_epoch(V); }

__device__ void frame_begin_state(const VolumeView &V) {
  reconcile(V);
  DevState *st = V.st;
  uint32_t f = st->frame + 1u;
  if (f == 0u || f == 0xFFFFFFFFu) f = 1u;  // 0xFFFFFFFF marks never-stamped slots
  st->frame = f;
  st->frame_count = 0;
  st->new_blocks = 0;
  st->voxels_updated = 0;
}

__device__ void mc_begin_state(const VolumeView &V) {
  reconcile(V);
  V.st->tri_count = 0;
  V.st->mc_next = 0;
  V.st->vert_count = 0;
}

// Opens a frame: stamp and counters (thread 0) and, with d_fin set, the
// frame's descriptor, passed by value so that a graph launch carries it in
// its kernel parameters instead of a copy on the stream.
__global__ void k_frame_begin(VolumeView V, FrameIn fin, FrameIn *d_fin) {
  if (threadIdx.x == 0) frame_begin_state(V);
  if (d_fin) {
    static_assert(sizeof(FrameIn) % 4 == 0, "word copy");
    const uint32_t *src = reinterpret_cast<const uint32_t *>(&fin);
    uint32_t *dst = reinterpret_cast<uint32_t *>(d_fin);
    for (int k = threadIdx.x; k < (int)(sizeof(FrameIn) / 4); k += blockDim.x) dst[k] = src[k];
  }
}

// The device counters into host-mapped memory, at the end of a frame.
__global__ void k_state_out(const DevState *__restrict__ st, DevState *host) {
  static_assert(sizeof(DevState) % 4 == 0 && sizeof(DevState) / 4 <= 32, "one warp");
  if (threadIdx.x < sizeof(DevState) / 4)
    reinterpret_cast<volatile uint32_t *>(host)[threadIdx.x] =
        reinterpret_cast<const uint32_t *>(st)[threadIdx.x];
}

__global__ void k_rcp_table(float *__restrict__ rcp) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w <= kRcpMax) rcp[w] = w ? __frcp_rn((float)w) : 0.0f;
}

__global__ void k_epoch_end(VolumeView V) {
  if (threadIdx.x == 0) reconcile(V);
}

__global__ void k_clear_list(VolumeView V) {
  if (threadIdx.x != 0) return;
  reconcile(V);
  uint32_t f = V.st->frame + 1u;
  if (f == 0u || f == 0xFFFFFFFFu) f = 1u;
  V.st->frame = f;
  V.st->frame_count = 0;
}

__global__ void k_mc_begin(VolumeView V) {
  if (threadIdx.x == 0) mc_begin_state(V);
}

// Frame-list entry i, lane k of its 8 threads: k = 0 writes frame_res[i] =
// {key, block} and frame_nb[8 i] = the block; k > 0 writes frame_nb[8 i + k]
// = the block at +(k & 1, k >> 1 & 1, k >> 2) (read by marching cubes).
__device__ __forceinline__ void resolve_entry(const VolumeView &V, uint32_t i, uint32_t k) {
  if (!VH_CHECK(V.st, i < V.frame_cap)) return;
  const uint32_t slot = V.frame_list[i];
  if (!VH_CHECK(V.st, slot <= V.slot_mask)) {
    if (k == 0) V.frame_res[i] = make_ulonglong2(kTombKey, (unsigned long long)kNoBlock);
    V.frame_nb[8 * (size_t)i + k] = kNoBlock;
    return;
  }
  const ulonglong2 sl = ld_slot_ro(V.slots + slot);
  uint32_t blk = (uint32_t)(sl.y & 0xFFFFFFFFull);
  if (!VH_CHECK(V.st, blk == kNoBlock || blk < V.pool_cap)) blk = kNoBlock;
  if (k == 0) V.frame_res[i] = make_ulonglong2(sl.x, (unsigned long long)blk);
  uint32_t nbid = kNoBlock;
  if (sl.x < kTombKey && blk != kNoBlock) {
    int bx, by, bz;
    unpack_key(sl.x, bx, by, bz);
    const int nx = bx + (int)(k & 1u), ny = by + (int)((k >> 1) & 1u), nz = bz + (int)(k >> 2);
    nbid = k == 0 ? blk
                  : (key_in_range(nx, ny, nz) ? block_of(V, pack_key(nx, ny, nz)) : kNoBlock);
    if (!VH_CHECK(V.st, nbid == kNoBlock || nbid < V.pool_cap)) nbid = kNoBlock;
  }
  V.frame_nb[8 * (size_t)i + k] = nbid;
}

// ---- batched scenes -----------------------------------------------------------------
// The stages of one frame for many independent scenes, each stage one launch
// over the work of all scenes (flattened (scene, item) index, items of a
// scene contiguous).  Per item the bodies above run unchanged with that
// scene's volume, camera and frame.

// Scene s with prefix[s] <= g < prefix[s + 1] (prefix non-decreasing,
// prefix[0] = 0 <= g < prefix[n]); empty scenes are skipped.
__device__ __forceinline__ int scene_of(const uint32_t *__restrict__ prefix, int n, uint32_t g) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(prefix + mid) <= g)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Copies scene s's descriptor into shared memory (whole CTA, then a barrier).
__device__ __forceinline__ void load_scene(SceneDesc &dst, const SceneDesc *__restrict__ d, int s) {
  static_assert(sizeof(SceneDesc) % 4 == 0, "word copy");
  const uint32_t *src = reinterpret_cast<const uint32_t *>(d + s);
  uint32_t *out = reinterpret_cast<uint32_t *>(&dst);
  for (int k = threadIdx.x; k < (int)(sizeof(SceneDesc) / 4); k += blockDim.x) out[k] = __ldg(src + k);
  __syncthreads();
}

__global__ void k_batch_frame_begin(const SceneDesc *__restrict__ d,
                                    const uint8_t *__restrict__ active, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n && active[s]) frame_begin_state(d[s].V);
}

// One thread per pixel of every scene; scene s owns global pixels
// [px_start[s], px_start[s + 1]), a multiple of the CTA size, so that a CTA
// (and a warp: the band walk de-duplicates keys per warp) never spans two
// scenes and the scene's descriptor is read once per CTA.
template <typename DepthT>
__global__ void __launch_bounds__(kBatchPixelThreads) k_batch_allocate(
    const SceneDesc *__restrict__ d, const uint8_t *__restrict__ active,
    const uint32_t *__restrict__ px_start, int n) {
  __shared__ SceneDesc sd;
  const uint32_t g0 = blockIdx.x * blockDim.x;
  if (g0 >= __ldg(px_start + n)) return;  // whole CTAs
  const int s = scene_of(px_start, n, g0);
  if (!active[s]) return;  // CTA-uniform
  load_scene(sd, d, s);
  __shared__ unsigned long long keys[kBatchPixelThreads / 32][32 * kAllocChunk];
  allocate_pixel<DepthT>(sd.V, sd.C, static_cast<const DepthT *>(sd.depth), sd.rgb, sd.pose,
                         sd.pix, (int)(g0 + threadIdx.x - __ldg(px_start + s)),
                         keys[threadIdx.x >> 5]);
}

// Closes every active scene's allocation epoch (CTA 0; with_mesh: also
// resets its marching-cubes counters), writes the prefix of the frame-list
// lengths for the later stages (CTA 0; prefix holds n + 2 words, the last
// one k_batch_mc's block counter) and resolves the frame lists of all
// scenes, 8 threads per entry (every CTA, from its own copy of the prefix
// in shared memory, n <= 1024).  The epoch fields CTA 0 updates are not
// the frame-list lengths the other CTAs read, as in k_frame_resolve.
__global__ void __launch_bounds__(256) k_batch_resolve(const SceneDesc *__restrict__ d,
                                                       const uint8_t *__restrict__ active, int n,
                                                       uint32_t *__restrict__ prefix,
                                                       int with_mesh) {
  __shared__ uint32_t sp[1025];
  __shared__ uint32_t wsum[8];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  uint32_t run = 0;
  for (int s0 = 0; s0 < n; s0 += 256) {
    const int s = s0 + t;
    uint32_t cnt = 0;
    if (s < n && active[s]) {
      const VolumeView &V = d[s].V;
      if (blockIdx.x == 0) {
        if (with_mesh)
          mc_begin_state(V);
        else
          reconcile(V);
      }
      cnt = min(V.st->frame_count, V.frame_cap);
    }
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += u;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    uint32_t before = 0, tot = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const uint32_t w = wsum[q];
      before += q < warp ? w : 0u;
      tot += w;
    }
    if (s < n) sp[s] = run + before + incl - cnt;
    run += tot;
    __syncthreads();  // wsum free for the next chunk
  }
  if (t == 0) sp[n] = run;
  __syncthreads();
  if (blockIdx.x == 0) {
    for (int s = t; s <= n; s += 256) prefix[s] = sp[s];
    if (t == 0) prefix[n + 1] = 0;  // k_batch_mc's hand-out counter
  }
  const uint32_t total8 = 8u * run;
  for (uint32_t g8 = blockIdx.x * blockDim.x + t; g8 < total8; g8 += gridDim.x * blockDim.x) {
    const uint32_t g = g8 >> 3;
    int lo = 0, hi = n;  // scene of entry g: the last s with sp[s] <= g
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (sp[mid] <= g)
        lo = mid;
      else
        hi = mid;
    }
    resolve_entry(d[lo].V, g - sp[lo], g8 & 7u);
  }
}

// Adds this CTA's count of updated voxels to scene `sd`'s counter.
__device__ __forceinline__ void flush_updated(const SceneDesc &sd, uint32_t updated) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) updated += __shfl_xor_sync(kFull, updated, o);
  if ((threadIdx.x & 31) == 0 && updated)
    atomicAdd(&sd.V.st->voxels_updated, (unsigned long long)updated);
}

// Persistent CTAs over the listed blocks of every scene; the scene's
// descriptor and pose live in shared memory while consecutive items stay in
// that scene.
__global__ void __launch_bounds__(128, 12) k_batch_integrate(const SceneDesc *__restrict__ d,
                                                         const uint32_t *__restrict__ prefix,
                                                         int n) {
  __shared__ SceneDesc sd;
  __shared__ float sp[12];
  const uint32_t total = __ldg(prefix + n);
  const int t = threadIdx.x;
  int cur = -1;
  uint32_t updated = 0;
  float P[12];
  for (uint32_t g = blockIdx.x; g < total; g += gridDim.x) {
    const int s = scene_of(prefix, n, g);
    if (s != cur) {  // uniform: every thread computes the same s
      if (cur >= 0) flush_updated(sd, updated);
      updated = 0;
      __syncthreads();  // sd free
      load_scene(sd, d, s);
      if (t < 12) sp[t] = __ldg(sd.pose + t);
      __syncthreads();
#pragma unroll
      for (int k = 0; k < 12; ++k) P[k] = sp[k];
      cur = s;
    }
    const uint32_t i = g - __ldg(prefix + s);
    VoxelRun<4> q;
    load_run<4>(sd.V, i, t, q);
    updated += integrate_run<4>(sd.V, sd.C, P, sd.pix, i, q);
  }
  if (cur >= 0) flush_updated(sd, updated);
}

// Per-frame marching cubes over the listed blocks of every scene.
template <int kMinCtas>
__global__ void __launch_bounds__(kMcThreads, kMinCtas) k_batch_mc(const SceneDesc *__restrict__ d,
                                                            const uint32_t *__restrict__ prefix,
                                                            int n, uint32_t *__restrict__ next) {
  __shared__ McShared S;
  __shared__ SceneDesc sd;
  mc_init_shared(S);
  const uint32_t total = __ldg(prefix + n);
  int cur = -1;
  __syncthreads();
  uint32_t g = blockIdx.x;
  for (int par = 0; g < total; par ^= 1) {  // dynamic hand-out, as in k_mc
    if (threadIdx.x == 0) S.next[par] = gridDim.x + atomicAdd(next, 1u);
    const int s = scene_of(prefix, n, g);
    if (s != cur) {  // the barrier closing the previous block freed sd
      load_scene(sd, d, s);
      cur = s;
    }
    mc_block<kMcThreads>(S, sd.V, 0, sd.C.mc_min_weight, sd.tris, sd.tri_cap, g - __ldg(prefix + s));
    __syncthreads();
    g = S.next[par];
  }
}

__global__ void k_batch_gather_state(const SceneDesc *__restrict__ d, int n,
                                     DevState *__restrict__ out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) out[s] = *d[s].V.st;
}

__global__ void k_batch_clear_errors(const SceneDesc *__restrict__ d, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) d[s].V.st->error = 0;
}

// ---- batched step in one persistent launch ------------------------------------------
// k_batch_step runs a whole batched step: the per-scene stage chain
// allocate -> resolve -> integrate [-> marching cubes] of every active scene
// in one launch of persistent 128-thread CTAs.  Each stage of a scene is cut
// into items; a CTA takes a ticket of whichever scene has items left in its
// current stage (StepSched::word), runs the item with the single-scene
// bodies (allocate_pixel, resolve_entry, integrate_run, mc_block), and the
// CTA that finishes a stage's last item opens the scene's next stage.  A
// scene's stages therefore follow one another as in separate launches while
// different scenes' stages overlap on the GPU.
//
// No CTA ever waits while holding an item: a ticket is taken only from an
// open stage, whose earlier stages are complete, and an idle CTA polls
// (bounded) until it finds an item or every scene is finished.  So the
// lowest unfinished item always runs and the launch ends whatever the
// residency.  Ordering between stages: every thread fences its writes, the
// CTA arrives on the stage's counter after a barrier, and the opener fences
// again before publishing the next stage; data written in one stage is read
// in a later one only, never cached before it was written (allocation reads
// slots through L2-coherent loads and the counters it reads do not change
// during the stage; the epoch is closed with volatile accesses).
constexpr int kStepThreads = 128;
constexpr int kStepPixels = 16 * kStepThreads;  // pixels per allocation item
constexpr int kStepEntries = 2 * kStepThreads;  // frame-list entries per resolve item
constexpr int kStepBlocks = 16;                 // listed blocks per integration item
constexpr int kStepMcBlocks = 4;                // listed blocks per marching-cubes item
static_assert(kStepEntries * 8 % kStepThreads == 0, "whole resolve rounds");
// An idle CTA gives up after this long without finding work while scenes
// are unfinished (never expected; the scenes left get kErrRetry).
constexpr unsigned long long kStepIdleLimitNs = 2000000000ull;
constexpr uint32_t kStepMaxPolls = 1u << 24;  // and after this many idle polls

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <bool kMesh>
struct StepShared;
template <>
struct StepShared<true> {
  McShared mc;  // allocation items borrow its staging words for their key lists
  __device__ unsigned long long *keys(int warp) {
    return reinterpret_cast<unsigned long long *>(mc.sdf) + warp * (32 * kAllocChunk);
  }
};
template <>
struct StepShared<false> {
  unsigned long long k[kStepThreads / 32][32 * kAllocChunk];
  __device__ unsigned long long *keys(int warp) { return k[warp]; }
};
static_assert(offsetof(McShared, rgb) == sizeof(float) * kStaged &&
                  (kStepThreads / 32) * 32 * kAllocChunk * sizeof(unsigned long long) <=
                      2 * sizeof(float) * kStaged,
              "allocation keys fit in the MC staging words");

// Opens the frame of every active scene and resets the step's hand-out
// (one CTA, a thread per scene, n <= blockDim.x <= 1024).
__global__ void k_batch_step_begin(const SceneDesc *__restrict__ d,
                                   const uint8_t *__restrict__ active, int n,
                                   StepSched *__restrict__ sched, StepGlobal *__restrict__ glob) {
  const int s = threadIdx.x;
  const bool act = s < n && active[s];
  if (s < n) {
    StepSched &q = sched[s];
    for (int k = 0; k < 4; ++k) {
      q.total[k] = 0;
      q.done[k] = 0;
    }
    q.count = 0;
    if (act) {
      frame_begin_state(d[s].V);
      const uint32_t npx = (uint32_t)d[s].C.width * (uint32_t)d[s].C.height;
      q.total[0] = (npx + kStepPixels - 1) / kStepPixels;
      q.word = 0ull;  // stage 0 (allocation), ticket 0
    } else {
      q.word = (unsigned long long)kStepDone << 32;
    }
  }
  const int nact = __syncthreads_count(act);
  if (s == 0) {
    glob->remaining = (uint32_t)nact;
    glob->gave_up = 0;
  }
}

__device__ __forceinline__ uint32_t ld_vol32(const uint32_t *p) {
  return *(volatile const uint32_t *)p;
}

// A ticket of an open stage of some scene, called by all lanes of warp 0:
// 32 scenes are looked at together from `hint` on, and the lanes whose scene
// shows a free ticket try it in order until one gets a valid one (the
// looks are only hints; the atomic decides).  Returns false, in every lane,
// when no scene had a free ticket.
__device__ __forceinline__ bool step_pick(StepSched *sched, int n, int hint, int *s_out,
                                          uint32_t *stage_out, uint32_t *item_out) {
  const int lane = threadIdx.x & 31;
  for (int r0 = 0; r0 < n; r0 += 32) {
    const int s = (hint + r0 + lane) % n;
    bool cand = false;
    if (r0 + lane < n) {
      const unsigned long long w = ld_volatile(&sched[s].word);
      const uint32_t st = (uint32_t)(w >> 32);
      cand = st < kStepDone && (uint32_t)w < ld_vol32(&sched[s].total[st]);
    }
    unsigned m = __ballot_sync(kFull, cand);
    while (m) {
      const int l = __ffs(m) - 1;
      m &= m - 1u;
      uint32_t ok = 0, st2 = 0, it = 0;
      if (lane == l) {
        const unsigned long long got = atomicAdd(&sched[s].word, 1ull);
        __threadfence();  // the stage's totals after the ticket
        st2 = (uint32_t)(got >> 32);
        it = (uint32_t)got;
        ok = st2 < kStepDone && it < ld_vol32(&sched[s].total[st2]) ? 1u : 0u;
      }
      if (__shfl_sync(kFull, ok, l)) {
        *s_out = __shfl_sync(kFull, s, l);
        *stage_out = __shfl_sync(kFull, st2, l);
        *item_out = __shfl_sync(kFull, it, l);
        return true;
      }
    }
  }
  return false;
}

// The allocation epoch of a scene closed as reconcile_epoch does (and the
// marching-cubes counters reset as mc_begin_state does), with volatile
// accesses: this launch's allocation items may have left the state's line
// in this SM's L1 before the tickets were counted.
__device__ __forceinline__ void step_close_epoch(const VolumeView &V, bool mesh) {
  volatile DevState *st = V.st;
  const uint32_t t = st->ticket;
  if (t) {
    const uint32_t free_count = st->free_count, pool_top = st->pool_top;
    const uint32_t from_free = min(t, free_count);
    st->free_count = free_count - from_free;
    const unsigned long long top = (unsigned long long)pool_top + (t - from_free);
    const uint32_t new_top = (uint32_t)min(top, (unsigned long long)V.pool_cap);
    st->new_blocks = st->new_blocks + from_free + (new_top - pool_top);
    st->pool_top = new_top;
    st->ticket = 0;
  }
  if (mesh) {
    st->tri_count = 0;
    st->mc_next = 0;
    st->vert_count = 0;
  }
}

// Called by thread 0 after the CTA finished item of `stage` of scene `s`
// (all its threads fenced, then a barrier): counts the item and, for the
// stage's last one, opens the scene's next non-empty stage.
__device__ __forceinline__ void step_finish(const VolumeView &V, StepSched &q, uint32_t stage, bool mesh,
                            StepGlobal *glob) {
  __threadfence();
  const uint32_t total = ld_vol32(&q.total[stage]);
  if (atomicAdd(&q.done[stage], 1u) + 1u != total) return;
  __threadfence();  // every item of the stage, before what the opener reads
  if (stage == 0) {
    step_close_epoch(V, mesh);
    const uint32_t c = min(ld_vol32(&V.st->frame_count), V.frame_cap);
    q.count = c;
    q.total[1] = (c + kStepEntries - 1) / kStepEntries;
    q.total[2] = (c + kStepBlocks - 1) / kStepBlocks;
    q.total[3] = mesh ? (c + kStepMcBlocks - 1) / kStepMcBlocks : 0u;
  }
  uint32_t next = stage + 1;
  while (next < kStepDone && ld_vol32(&q.total[next]) == 0u) ++next;
  __threadfence();  // totals and the closed epoch before the stage opens
  atomicExch(&q.word, (unsigned long long)next << 32);
  if (next == kStepDone) atomicSub(&glob->remaining, 1u);
}

// Stage bodies of k_batch_step.
template <typename DepthT>
__device__ __forceinline__ void step_allocate(const SceneDesc &sd, uint32_t item,
                                           unsigned long long *wkeys) {
  const int base = (int)(item * (uint32_t)kStepPixels) + (int)threadIdx.x;
#pragma unroll 1
  for (int r = 0; r < kStepPixels / kStepThreads; ++r)
    allocate_pixel<DepthT>(sd.V, sd.C, static_cast<const DepthT *>(sd.depth), sd.rgb, sd.pose,
                           sd.pix, base + r * kStepThreads, wkeys);
}

__device__ __forceinline__ void step_integrate(const SceneDesc &sd, const float *sp, uint32_t item,
                                            uint32_t count) {
  float P[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) P[k] = sp[k];
  uint32_t updated = 0;
  const uint32_t i0 = item * (uint32_t)kStepBlocks;
  const uint32_t i1 = min(i0 + (uint32_t)kStepBlocks, count);
#pragma unroll 1
  for (uint32_t i = i0; i < i1; ++i) {
    VoxelRun<4> q;
    load_run<4>(sd.V, i, (int)threadIdx.x, q);
    updated += integrate_run<4>(sd.V, sd.C, P, sd.pix, i, q);
  }
  flush_updated(sd, updated);
}

// Warp 0 picks the CTA's next item (lane 0 writes it to `c`).  `spec`
// (lane 0's) is the ticket lane 0 took while the previous item ran
// (StepCta::spec_scene >= 0): a ticket of that item's stage, which cannot
// close before that item is finished; a valid one is run next.  Otherwise
// scenes are scanned from the current one on, polling (bounded) while none
// has a free ticket and some are unfinished.  Returns the scene in every
// lane, or -1 when the step is over.
struct StepCta {
  int scene, cur, spec_scene;
  uint32_t stage, item, count, spec_stage, spec_total;
};

__device__ __forceinline__ int step_next(StepCta &c, unsigned long long spec,
                                         const SceneDesc *__restrict__ d, int n,
                                         StepSched *__restrict__ sched, StepGlobal *glob) {
  const int lane = threadIdx.x & 31;
  const int spec_scene = c.spec_scene, cur = c.cur;
  const uint32_t spec_stage = c.spec_stage, spec_total = c.spec_total;
  spec = __shfl_sync(kFull, spec, 0);
  __syncwarp();  // every lane has read c before lane 0 rewrites it
  int s = -1;
  uint32_t stage = 0, item = 0;
  if (spec_scene >= 0) {  // the same in every lane
    const uint32_t st2 = (uint32_t)(spec >> 32), it = (uint32_t)spec;
    if (st2 < kStepDone &&
        it < (st2 == spec_stage ? spec_total : ld_vol32(&sched[spec_scene].total[st2]))) {
      s = spec_scene;
      stage = st2;
      item = it;
    }
  }
  const int hint = cur >= 0 ? cur : (int)(blockIdx.x % (unsigned)n);
  unsigned long long idle_since = 0;
  for (uint32_t polls = 0; s < 0; ++polls) {
    if (step_pick(sched, n, hint, &s, &stage, &item)) break;
    uint32_t stop = 0;  // lane 0 decides: 1 every scene finished, 2 give up
    if (lane == 0) {
      if (ld_vol32(&glob->remaining) == 0u) {
        stop = 1u;
      } else {
        const unsigned long long now = global_ns();
        if (polls == 0) idle_since = now;
        if (polls >= kStepMaxPolls || now - idle_since > kStepIdleLimitNs) stop = 2u;
      }
    }
    stop = __shfl_sync(kFull, stop, 0);
    if (stop == 1u) break;
    if (stop == 2u) {  // never expected: report instead of waiting on
      if (lane == 0) {
        atomicAdd(&glob->gave_up, 1u);
        for (int k = 0; k < n; ++k)
          if ((uint32_t)(ld_volatile(&sched[k].word) >> 32) < kStepDone)
            atomicOr(&d[k].V.st->error, kErrRetry);
      }
      break;
    }
    __nanosleep(200);
  }
  if (lane == 0) {
    c.spec_scene = -1;
    c.scene = s;
    c.stage = stage;
    c.item = item;
    c.count = s >= 0 ? ld_vol32(&sched[s].count) : 0u;
  }
  return s;
}

// Register budget for 8 resident CTAs per SM (64 registers): with every
// stage body in one loop, budgets for 10-12 CTAs spill 0.2-0.4 KB per thread
// and measured 4-10 % slower on the batched-scenes workloads.
template <typename DepthT, bool kMesh>
__global__ void __launch_bounds__(kStepThreads, 8)
    k_batch_step(const SceneDesc *__restrict__ d, int n, StepSched *__restrict__ sched,
                 StepGlobal *__restrict__ glob) {
  __shared__ __align__(16) StepShared<kMesh> sh;
  __shared__ SceneDesc sd;
  __shared__ float sp[12];
  __shared__ StepCta c;  // the CTA's scheduling state (thread 0 writes it)
  if constexpr (kMesh) mc_init_shared(sh.mc);
  if (threadIdx.x == 0) {
    c.cur = -1;
    c.spec_scene = -1;
  }
  unsigned long long spec = 0;  // lane 0 of warp 0: the ticket taken while an item runs
  for (;;) {
    if (threadIdx.x < 32) {
      const int s = step_next(c, spec, d, n, sched, glob);
      if (threadIdx.x == 0 && s >= 0) {  // take the following ticket now; it is looked at after this item
        c.spec_stage = c.stage;
        c.spec_total = ld_vol32(&sched[s].total[c.stage]);
        spec = atomicAdd(&sched[s].word, 1ull);
        c.spec_scene = s;
      }
    }
    __syncthreads();
    const int s = c.scene;
    if (s < 0) break;  // uniform
    if (s != c.cur) {  // uniform; the previous item's barrier freed sd
      load_scene(sd, d, s);  // ends with a barrier: every thread has compared c.cur
      if (threadIdx.x < 12) sp[threadIdx.x] = __ldg(sd.pose + threadIdx.x);
      if (threadIdx.x == 0) c.cur = s;
      __syncthreads();
    }
    const uint32_t stage = c.stage, item = c.item;
    if (stage == 0) {  // allocation: kStepPixels pixels, every lane of each warp takes part
      step_allocate<DepthT>(sd, item, sh.keys(threadIdx.x >> 5));
    } else if (stage == 1) {  // resolve: kStepEntries entries, 8 threads each
      const uint32_t e0 = item * (uint32_t)kStepEntries, count = c.count;
#pragma unroll 1
      for (int r = 0; r < kStepEntries * 8 / kStepThreads; ++r) {
        const uint32_t g8 = (uint32_t)(r * kStepThreads) + threadIdx.x;
        const uint32_t e = e0 + (g8 >> 3);
        if (e < count) resolve_entry(sd.V, e, g8 & 7u);
      }
    } else if (stage == 2) {  // integration: kStepBlocks listed blocks
      step_integrate(sd, sp, item, c.count);
    } else if constexpr (kMesh) {  // marching cubes: kStepMcBlocks listed blocks
      const uint32_t i0 = item * (uint32_t)kStepMcBlocks;
      const uint32_t i1 = min(i0 + (uint32_t)kStepMcBlocks, c.count);
#pragma unroll 1
      for (uint32_t i = i0; i < i1; ++i) {
        if (i > i0) __syncthreads();  // the previous block is done with the shared state
        mc_block<kStepThreads>(sh.mc, sd.V, 0, sd.C.mc_min_weight, sd.tris, sd.tri_cap, i);
      }
    }
    __threadfence();  // this thread's writes of the item before the CTA arrives
    __syncthreads();  // also frees the shared state for the next item
    if (threadIdx.x == 0) step_finish(sd.V, sched[s], stage, kMesh, glob);
  }
}

// ---- hash surface -----------------------------------------------------------------
__global__ void __launch_bounds__(256) k_alloc_keys(VolumeView V, const int32_t *__restrict__ xyz,
                                                    uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t frame = V.st->frame;
  const uint32_t free0 = V.st->free_count, top0 = V.st->pool_top;
  bool active = false;
  unsigned long long key = kEmptyKey;
  if (i < n) {
    const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    if (key_in_range(x, y, z)) {
      key = pack_key(x, y, z);
      active = true;
    } else {
      atomicOr(&V.st->error, kErrRange);
    }
  }
  const unsigned peers = __match_any_sync(kFull, key);
  const bool leader = active && (__ffs(peers) - 1) == (int)(threadIdx.x & 31);
  bool created = false;
  uint32_t slot = kNoBlock, seen = kNoBlock;
  if (leader) slot = slot_insert(V, key, &created, &seen);
  assign_blocks(V, created, slot, key, free0, top0);
  stamp_and_append(V, leader, slot, frame, seen);
}

__global__ void __launch_bounds__(256) k_find_keys(VolumeView V, const int32_t *__restrict__ xyz,
                                                   uint32_t n, int32_t *__restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  uint32_t b = kNoBlock;
  if (key_in_range(x, y, z)) b = block_of(V, pack_key(x, y, z));
  out[i] = b == kNoBlock ? -1 : (int32_t)b;
}

// Erases keys: the slot becomes a tombstone, the block is zeroed and pushed
// onto the free list (no allocation runs concurrently with this kernel).
__global__ void __launch_bounds__(256) k_erase_keys(VolumeView V, const int32_t *__restrict__ xyz,
                                                    uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  if (!key_in_range(x, y, z)) return;
  const unsigned long long key = pack_key(x, y, z);
  const uint32_t h = (uint32_t)mix64(key) & V.slot_mask;
  for (int p = 0; p < V.max_probe; ++p) {
    const uint32_t s = (h + (uint32_t)p) & V.slot_mask;
    const unsigned long long k = ld_volatile(&V.slots[s].key);
    if (k == kEmptyKey) return;
    if (k != key) continue;
    if (atomicCAS(&V.slots[s].key, key, kTombKey) != key) return;  // erased by a duplicate
    const uint32_t b = V.slots[s].block;
    V.slots[s].block = kNoBlock;
    atomicAdd(&V.st->tombstones, 1u);
    atomicAdd(&V.st->erased, 1u);
    if (b != kNoBlock) {
      float4 *blk = reinterpret_cast<float4 *>(V.pool + (size_t)b * kBlockWords);
      for (int q = 0; q < kBlockWords / 4; ++q) blk[q] = make_float4(0.f, 0.f, 0.f, 0.f);
      V.block_keys[b] = kEmptyKey;
      __threadfence();
      const uint32_t f = atomicAdd(&V.st->free_count, 1u);
      V.free_list[f] = b;
    }
    return;
  }
}

// Rebuilds frame_res and frame_nb for the current block list (needed when
// the list changed without a frame, e.g. after alloc_keys or erase).
__global__ void __launch_bounds__(256) k_frame_nb(VolumeView V) {
  const uint32_t n = min(V.st->frame_count, V.frame_cap);
  const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  if ((idx >> 3) < n) resolve_entry(V, idx >> 3, idx & 7u);
}

// frame_res and frame_nb of every frame-list entry, 8 threads per entry
// (grid-stride), after allocation and before integration.  Thread 0 also
// closes the allocation epoch and, when marching cubes follows in this
// frame, resets its counters (no other thread reads those fields).
__global__ void __launch_bounds__(256) k_frame_resolve(VolumeView V, int mc_follows) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (mc_follows)
      mc_begin_state(V);
    else
      reconcile(V);
  }
  const uint32_t n8 = 8u * min(V.st->frame_count, V.frame_cap);
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < n8; g += gridDim.x * blockDim.x)
    resolve_entry(V, g >> 3, g & 7u);
}

__global__ void k_list_keys(VolumeView V, int32_t *__restrict__ xyz, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long key = V.slots[V.frame_list[i]].key;
  int x = 0, y = 0, z = 0;
  if (key < kTombKey) unpack_key(key, x, y, z);
  xyz[3 * i] = x;
  xyz[3 * i + 1] = y;
  xyz[3 * i + 2] = z;
}

// Overwrites the voxels of already inserted blocks; one CTA per block.
__global__ void __launch_bounds__(128) k_scatter_blocks(VolumeView V, const int32_t *__restrict__ xyz,
                                                        const float *__restrict__ sdf,
                                                        const float *__restrict__ w,
                                                        const uint8_t *__restrict__ rgb,
                                                        uint32_t n) {
  const uint32_t i = blockIdx.x;
  if (i >= n) return;
  const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  if (!key_in_range(x, y, z)) return;
  const uint32_t b = block_of(V, pack_key(x, y, z));
  if (b == kNoBlock) return;
  float *base = V.pool + (size_t)b * kBlockWords;
  for (int v = threadIdx.x; v < kB3; v += blockDim.x) {
    const size_t src = (size_t)i * kB3 + v;
    base[v] = sdf[src];
    base[kB3 + v] = w[src];
    const uint32_t c = (uint32_t)rgb[3 * src] | ((uint32_t)rgb[3 * src + 1] << 8) |
                       ((uint32_t)rgb[3 * src + 2] << 16);
    reinterpret_cast<uint32_t *>(base + 2 * kB3)[v] = c;
  }
}

inline unsigned grid_for(uint32_t n, unsigned threads) { return (n + threads - 1) / threads; }

}  // namespace

void launch_frame_begin(const VolumeView &V, const FrameIn *fin, FrameIn *d_fin, cudaStream_t s) {
  k_frame_begin<<<1, 32, 0, s>>>(V, fin ? *fin : FrameIn{}, fin ? d_fin : nullptr);
}
void launch_state_out(const VolumeView &V, DevState *host, cudaStream_t s) {
  k_state_out<<<1, 32, 0, s>>>(V.st, host);
}

cudaGraphNode_t find_frame_begin_node(cudaGraph_t g) {
  size_t n = 0;
  if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return nullptr;
  std::vector<cudaGraphNode_t> nodes(n);
  if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return nullptr;
  for (cudaGraphNode_t nd : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nd, &t) != cudaSuccess || t != cudaGraphNodeTypeKernel) continue;
    cudaKernelNodeParams p{};
    if (cudaGraphKernelNodeGetParams(nd, &p) != cudaSuccess) continue;
    if (p.func == reinterpret_cast<void *>(k_frame_begin)) return nd;
  }
  return nullptr;
}

cudaError_t update_frame_begin(cudaGraphExec_t e, cudaGraphNode_t n, const VolumeView &V,
                               const FrameIn &fin, FrameIn *d_fin) {
  VolumeView v = V;
  FrameIn f = fin;
  FrameIn *d = d_fin;
  void *args[3] = {&v, &f, &d};
  cudaKernelNodeParams p{};
  p.func = reinterpret_cast<void *>(k_frame_begin);
  p.gridDim = dim3(1);
  p.blockDim = dim3(32);
  p.sharedMemBytes = 0;
  p.kernelParams = args;
  p.extra = nullptr;
  return cudaGraphExecKernelNodeSetParams(e, n, &p);
}
void launch_epoch_end(const VolumeView &V, cudaStream_t s) { k_epoch_end<<<1, 32, 0, s>>>(V); }
void launch_rcp_table(float *rcp, cudaStream_t s) {
  k_rcp_table<<<(kRcpMax + 256) / 256, 256, 0, s>>>(rcp);
}
void launch_clear_list(const VolumeView &V, cudaStream_t s) { k_clear_list<<<1, 32, 0, s>>>(V); }
void launch_mc_begin(const VolumeView &V, cudaStream_t s) { k_mc_begin<<<1, 32, 0, s>>>(V); }

void launch_allocate(const VolumeView &V, const CamParams &C, const FrameIn *fin,
                     const void *depth, int fmt, bool filter, uint2 *pix, cudaStream_t s) {
  const unsigned grid = grid_for((uint32_t)C.width * (uint32_t)C.height, 256);
  const uint16_t *d16 = (const uint16_t *)depth;
  const float *d32 = (const float *)depth;
  if (fmt == 0 && filter)
    k_allocate<uint16_t, true><<<grid, 256, 0, s>>>(V, C, fin, d16, pix);
  else if (fmt == 0)
    k_allocate<uint16_t, false><<<grid, 256, 0, s>>>(V, C, fin, d16, pix);
  else if (filter)
    k_allocate<float, true><<<grid, 256, 0, s>>>(V, C, fin, d32, pix);
  else
    k_allocate<float, false><<<grid, 256, 0, s>>>(V, C, fin, d32, pix);
}

void launch_depth_filter(const CamParams &C, const void *depth, const FrameIn *fin, int fmt,
                         float *out, cudaStream_t s) {
  const unsigned grid = grid_for((uint32_t)C.width * (uint32_t)C.height, 256);
  if (fmt == 0)
    k_depth_filter<uint16_t><<<grid, 256, 0, s>>>(C, static_cast<const uint16_t *>(depth), fin, out);
  else
    k_depth_filter<float><<<grid, 256, 0, s>>>(C, static_cast<const float *>(depth), fin, out);
}

template <int kV, bool kPrefetch, int kMinCtas>
int integrate_occupancy() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_integrate<kV, kPrefetch, kMinCtas>, kB3 / kV,
                                                0);
  return n > 0 ? n : 1;
}

int integrate_ctas_per_sm(int variant) {
  switch (variant) {
    case 1: return integrate_occupancy<4, true, 8>();
    case 2: return integrate_occupancy<8, false, 16>();
    case 3: return integrate_occupancy<2, false, 6>();
    case 4: return integrate_occupancy<4, false, 10>();
    case 5: return integrate_occupancy<8, false, 12>();
    default: return integrate_occupancy<4, false, 12>();
  }
}

int integrate_variants() { return kIntegrateVariants; }

// MC launch shapes (the tuning's mc_variant): 0: 128 threads, register
// budget for 10 resident CTAs per SM; 1: 128 threads, 12 CTAs; 2: 256
// threads (2 voxels and 2 cubes per thread, rounds of 256 candidates), 5
// CTAs.
int mc_variants() { return 3; }

int mc_ctas_per_sm(int variant) {
  int n = 0;
  if (variant == 2)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mc<256, 5>, 256, 0);
  else if (variant == 1)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mc<kMcThreads, 12>, kMcThreads, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mc<kMcThreads, 10>, kMcThreads, 0);
  return n > 0 ? n : 1;
}

template <int kV, bool kPrefetch, int kMinCtas>
void launch_integrate_shape(const VolumeView &V, const CamParams &C, const uint2 *pix,
                            const float *pose, int grid, cudaStream_t s) {
  k_integrate<kV, kPrefetch, kMinCtas><<<grid, kB3 / kV, 0, s>>>(V, C, pix, pose);
}

void launch_integrate(const VolumeView &V, const CamParams &C, const uint2 *pix, const float *pose,
                      int grid, int variant, cudaStream_t s) {
  switch (variant) {
    case 1: launch_integrate_shape<4, true, 8>(V, C, pix, pose, grid, s); break;
    case 2: launch_integrate_shape<8, false, 16>(V, C, pix, pose, grid, s); break;
    case 3: launch_integrate_shape<2, false, 6>(V, C, pix, pose, grid, s); break;
    case 4: launch_integrate_shape<4, false, 10>(V, C, pix, pose, grid, s); break;
    case 5: launch_integrate_shape<8, false, 12>(V, C, pix, pose, grid, s); break;
    default: launch_integrate_shape<4, false, 12>(V, C, pix, pose, grid, s); break;
  }
}

void launch_mc(const VolumeView &V, int scope_all, float min_weight, float4 *tris,
               uint32_t tri_cap, int grid, int variant, DevState *host_state, cudaStream_t s) {
  if (variant == 2)
    k_mc<256, 5><<<grid, 256, 0, s>>>(V, scope_all, min_weight, tris, tri_cap, host_state);
  else if (variant == 1)
    k_mc<kMcThreads, 12><<<grid, kMcThreads, 0, s>>>(V, scope_all, min_weight, tris, tri_cap,
                                                      host_state);
  else
    k_mc<kMcThreads, 10><<<grid, kMcThreads, 0, s>>>(V, scope_all, min_weight, tris, tri_cap,
                                                      host_state);
}

int mc_indexed_ctas_per_sm() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mc_indexed, kMcThreads, 0);
  return n > 0 ? n : 1;
}

void launch_mc_indexed(const VolumeView &V, float min_weight, float4 *verts, uint32_t vcap,
                       int32_t *faces, uint32_t fcap, int grid, DevState *host_state,
                       cudaStream_t s) {
  k_mc_indexed<<<grid, kMcThreads, 0, s>>>(V, min_weight, verts, vcap, faces, fcap, host_state);
}

void launch_alloc_keys(const VolumeView &V, const int32_t *xyz, uint32_t n, cudaStream_t s) {
  if (n) k_alloc_keys<<<grid_for(n, 256), 256, 0, s>>>(V, xyz, n);
}
void launch_find_keys(const VolumeView &V, const int32_t *xyz, uint32_t n, int32_t *out,
                      cudaStream_t s) {
  if (n) k_find_keys<<<grid_for(n, 256), 256, 0, s>>>(V, xyz, n, out);
}
void launch_erase_keys(const VolumeView &V, const int32_t *xyz, uint32_t n, cudaStream_t s) {
  if (n) k_erase_keys<<<grid_for(n, 256), 256, 0, s>>>(V, xyz, n);
}
void launch_frame_resolve(const VolumeView &V, int grid, bool mc_follows, cudaStream_t s) {
  k_frame_resolve<<<grid, 256, 0, s>>>(V, mc_follows ? 1 : 0);
}
void launch_frame_nb(const VolumeView &V, cudaStream_t s) {
  k_frame_nb<<<grid_for(V.frame_cap * 8u, 256), 256, 0, s>>>(V);
}
void launch_list_keys(const VolumeView &V, int32_t *xyz, uint32_t n, cudaStream_t s) {
  if (n) k_list_keys<<<grid_for(n, 256), 256, 0, s>>>(V, xyz, n);
}
void launch_scatter_blocks(const VolumeView &V, const int32_t *xyz, const float *sdf,
                           const float *w, const uint8_t *rgb, uint32_t n, cudaStream_t s) {
  if (n) k_scatter_blocks<<<n, 128, 0, s>>>(V, xyz, sdf, w, rgb, n);
}

void launch_batch_frame_begin(const SceneDesc *d, const uint8_t *active, int n, cudaStream_t s) {
  k_batch_frame_begin<<<grid_for((uint32_t)n, 128), 128, 0, s>>>(d, active, n);
}
void launch_batch_allocate(const SceneDesc *d, const uint8_t *active, const uint32_t *px_start,
                           uint32_t total_px, int n, int fmt, cudaStream_t s) {
  const unsigned grid = grid_for(total_px, kBatchPixelThreads);
  if (!grid) return;
  if (fmt == 0)
    k_batch_allocate<uint16_t><<<grid, kBatchPixelThreads, 0, s>>>(d, active, px_start, n);
  else
    k_batch_allocate<float><<<grid, kBatchPixelThreads, 0, s>>>(d, active, px_start, n);
}
void launch_batch_resolve(const SceneDesc *d, const uint8_t *active, int n, uint32_t *prefix,
                          bool with_mesh, int grid, cudaStream_t s) {
  k_batch_resolve<<<grid, 256, 0, s>>>(d, active, n, prefix, with_mesh ? 1 : 0);
}
void launch_batch_integrate(const SceneDesc *d, const uint32_t *prefix, int n, int grid,
                            cudaStream_t s) {
  k_batch_integrate<<<grid, 128, 0, s>>>(d, prefix, n);
}
void launch_batch_mc(const SceneDesc *d, uint32_t *prefix, int n, int grid, int variant,
                     cudaStream_t s) {
  uint32_t *next = prefix + n + 1;  // reset by k_batch_resolve
  if (variant == 1)
    k_batch_mc<12><<<grid, kMcThreads, 0, s>>>(d, prefix, n, next);
  else
    k_batch_mc<10><<<grid, kMcThreads, 0, s>>>(d, prefix, n, next);
}
int batch_integrate_ctas_per_sm() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_integrate, 128, 0);
  return n > 0 ? n : 1;
}
int batch_mc_ctas_per_sm(int variant) {
  int n = 0;
  if (variant == 1)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_mc<12>, kMcThreads, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_mc<10>, kMcThreads, 0);
  return n > 0 ? n : 1;
}
void launch_batch_gather_state(const SceneDesc *d, int n, DevState *out, cudaStream_t s) {
  k_batch_gather_state<<<grid_for((uint32_t)n, 128), 128, 0, s>>>(d, n, out);
}
void launch_batch_clear_errors(const SceneDesc *d, int n, cudaStream_t s) {
  k_batch_clear_errors<<<grid_for((uint32_t)n, 128), 128, 0, s>>>(d, n);
}

int batch_step_ctas_per_sm(bool with_mesh) {
  int n = 0;  // the same for both depth formats
  if (with_mesh)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_step<uint16_t, true>, kStepThreads, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_step<uint16_t, false>, kStepThreads,
                                                  0);
  return n > 0 ? n : 1;
}

void launch_batch_step(const SceneDesc *d, const uint8_t *active, int n, StepSched *sched,
                       StepGlobal *glob, int fmt, bool with_mesh, int grid, cudaStream_t s) {
  if (n < 1 || n > kMaxBatchScenes || grid < 1) return;
  k_batch_step_begin<<<1, (unsigned)((n + 31) / 32 * 32), 0, s>>>(d, active, n, sched, glob);
  if (fmt == 0) {
    if (with_mesh)
      k_batch_step<uint16_t, true><<<grid, kStepThreads, 0, s>>>(d, n, sched, glob);
    else
      k_batch_step<uint16_t, false><<<grid, kStepThreads, 0, s>>>(d, n, sched, glob);
  } else {
    if (with_mesh)
      k_batch_step<float, true><<<grid, kStepThreads, 0, s>>>(d, n, sched, glob);
    else
      k_batch_step<float, false><<<grid, kStepThreads, 0, s>>>(d, n, sched, glob);
  }
}

}  // namespace vh

// VH_BUILD_CHECKED (include/vhsdf.h) when this file was compiled with the
// VH_CHECKED bounds checks.
extern "C" uint32_t vh_build_flags(void) {
#ifdef VH_CHECKED
  return 1u;
#else
  return 0u;
#endif
}
