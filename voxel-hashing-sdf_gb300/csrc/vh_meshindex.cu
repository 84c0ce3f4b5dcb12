// vh_meshindex.cu - indexed mesh on the GPU: vertices merged by exact
// position, numbered like GpuTsdfGenerator::tsdf2mesh (src/tsdf.cu:1760-1888).
//
// The reference walks its triangles on the host and keys an unordered_map
// on the three floats of each vertex (src/tsdf.cu:1777,1810-1821): the first
// occurrence of a position becomes the next vertex and keeps its colour.
// Triangle order on the GPU depends on scheduling, so the triangles are first
// sorted by (x, y, z of vertex 0, 1, 2 as floats, then the three colour
// words); numbering by first occurrence over that order is then fixed.
//   1. sort triangle ids by the 12-word key (least significant word first,
//      stable 32-bit radix sorts; floats mapped to order-preserving words
//      with -0 == +0);
//   2. vertex occurrences o = 3 t + j in that order, stably sorted by their
//      canonical position (-0 -> +0), so equal positions are contiguous with
//      ascending o;
//   3. the head of each run is the first occurrence; an exclusive scan over
//      the first-occurrence flags (indexed by o) numbers the vertices;
//   4. every occurrence takes the number of its run's head.
// Sorting and scanning use CUB (CUDA toolkit library); the key maps, run
// heads and gathers are the kernels below.

#include <cub/cub.cuh>

#include <cstring>
#include <vector>

#include "vh_internal.h"

namespace vh {
namespace {

__device__ __forceinline__ uint32_t canon_bits(float f) {
  return f == 0.0f ? 0u : __float_as_uint(f);
}

// Order-preserving word of a float (with -0 == +0): a < b as floats iff
// word(a) < word(b) as unsigned.
__device__ __forceinline__ uint32_t order_word(float f) {
  const uint32_t u = canon_bits(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Key word w (0 = most significant) of triangle tri: words 0..8 are the
// coordinates x, y, z of vertices 0, 1, 2, words 9..11 their colour bits.
__global__ void k_tri_word(const float4 *__restrict__ tris, const uint32_t *__restrict__ idx,
                           uint32_t n, int w, uint32_t *__restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 v = tris[3 * (size_t)idx[i] + (w < 9 ? w / 3 : w - 9)];
  if (w < 9) {
    const int a = w % 3;
    out[i] = order_word(a == 0 ? v.x : (a == 1 ? v.y : v.z));
  } else {
    out[i] = __float_as_uint(v.w);
  }
}

// Occurrence o = 3 t + j of sorted triangle t: canonical (y, z) as one
// 64-bit key and its own index as the value.
__global__ void k_occ_yz(const float4 *__restrict__ tris, const uint32_t *__restrict__ idx,
                         uint32_t n3, unsigned long long *__restrict__ key,
                         uint32_t *__restrict__ occ) {
  const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n3) return;
  const float4 v = tris[3 * (size_t)idx[o / 3] + o % 3];
  key[o] = ((unsigned long long)canon_bits(v.y) << 32) | canon_bits(v.z);
  occ[o] = o;
}

__device__ __forceinline__ float4 occ_vertex(const float4 *tris, const uint32_t *idx, uint32_t o) {
  return tris[3 * (size_t)idx[o / 3] + o % 3];
}

__global__ void k_occ_x(const float4 *__restrict__ tris, const uint32_t *__restrict__ idx,
                        const uint32_t *__restrict__ occ, uint32_t n3, uint32_t *__restrict__ key) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n3) return;
  key[p] = canon_bits(occ_vertex(tris, idx, occ[p]).x);
}

// head[p] = 1 where sorted occurrence p starts a run of equal positions;
// first[o] = 1 for the occurrence o that heads its run.
__global__ void k_heads(const float4 *__restrict__ tris, const uint32_t *__restrict__ idx,
                        const uint32_t *__restrict__ occ, uint32_t n3, uint32_t *__restrict__ head,
                        uint32_t *__restrict__ first) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n3) return;
  const float4 a = occ_vertex(tris, idx, occ[p]);
  bool h = p == 0;
  if (!h) {
    const float4 b = occ_vertex(tris, idx, occ[p - 1]);
    h = canon_bits(a.x) != canon_bits(b.x) || canon_bits(a.y) != canon_bits(b.y) ||
        canon_bits(a.z) != canon_bits(b.z);
  }
  head[p] = h;
  first[occ[p]] = h;
}

// run_first[r] = the occurrence heading run r (r = inclusive head count - 1).
__global__ void k_run_first(const uint32_t *__restrict__ occ, const uint32_t *__restrict__ head,
                            const uint32_t *__restrict__ run, uint32_t n3,
                            uint32_t *__restrict__ run_first) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n3 && head[p]) run_first[run[p] - 1] = occ[p];
}

// faces[o] = number of the vertex of occurrence o; vertices and colours of
// first occurrences written at their numbers (positions in metres).
__global__ void k_emit(const float4 *__restrict__ tris, const uint32_t *__restrict__ idx,
                       const uint32_t *__restrict__ occ, const uint32_t *__restrict__ run,
                       const uint32_t *__restrict__ run_first, const uint32_t *__restrict__ first,
                       const uint32_t *__restrict__ vid, uint32_t n3, float voxel,
                       int32_t *__restrict__ faces, float *__restrict__ vert,
                       uint8_t *__restrict__ col) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n3) return;
  const uint32_t o = occ[p];
  const uint32_t id = vid[run_first[run[p] - 1]];
  faces[o] = (int32_t)id;
  if (first[o]) {
    const float4 v = occ_vertex(tris, idx, o);
    vert[3 * (size_t)id] = v.x * voxel;
    vert[3 * (size_t)id + 1] = v.y * voxel;
    vert[3 * (size_t)id + 2] = v.z * voxel;
    const uint32_t c = __float_as_uint(v.w);
    col[3 * (size_t)id] = (uint8_t)(c & 0xFFu);
    col[3 * (size_t)id + 1] = (uint8_t)((c >> 8) & 0xFFu);
    col[3 * (size_t)id + 2] = (uint8_t)((c >> 16) & 0xFFu);
  }
}

inline unsigned blocks_for(uint64_t n) { return (unsigned)((n + 255) / 256); }

// Device scratch of one indexing call, freed on scope exit.
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

}  // namespace

vh_status index_mesh(vh_handle *h, const float4 *tris, int64_t n_in, float voxel,
                     std::vector<float> &vert, std::vector<uint8_t> &col,
                     std::vector<int32_t> &faces) {
  vert.clear();
  col.clear();
  faces.clear();
  if (n_in <= 0) return VH_OK;
  if (n_in > (int64_t)0x55555555) return handle_fail(h, VH_ERR_CAPACITY, "mesh too large to index");
  const uint32_t n = (uint32_t)n_in, n3 = 3 * n;
  const cudaStream_t st = handle_stream(h);
  Scratch s;
  uint32_t *idx_a, *idx_b, *word_a, *word_b, *occ_a, *occ_b, *kx_a, *kx_b, *head, *first, *vid,
      *run, *run_first;
  unsigned long long *kyz_a, *kyz_b;
  int32_t *d_faces;
  float *d_vert;
  uint8_t *d_col;
  bool ok = s.alloc(&idx_a, n) && s.alloc(&idx_b, n) && s.alloc(&word_a, n) &&
            s.alloc(&word_b, n) && s.alloc(&occ_a, n3) && s.alloc(&occ_b, n3) &&
            s.alloc(&kx_a, n3) && s.alloc(&kx_b, n3) && s.alloc(&kyz_a, n3) &&
            s.alloc(&kyz_b, n3) && s.alloc(&head, n3) && s.alloc(&first, n3) &&
            s.alloc(&vid, n3) && s.alloc(&run, n3) && s.alloc(&run_first, n3) &&
            s.alloc(&d_faces, n3) && s.alloc(&d_vert, 3 * (size_t)n3) && s.alloc(&d_col, 3 * (size_t)n3);
  if (!ok) return handle_fail(h, VH_ERR_CUDA, "mesh indexing: device allocation failed");
  // CUB temporary storage: the largest request of the calls below
  size_t tmp_bytes = 0, b1 = 0, b2 = 0, b3 = 0, b4 = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, b1, word_a, word_b, idx_a, idx_b, (int64_t)n, 0, 32, st);
  cub::DeviceRadixSort::SortPairs(nullptr, b2, kyz_a, kyz_b, occ_a, occ_b, (int64_t)n3, 0, 64, st);
  cub::DeviceRadixSort::SortPairs(nullptr, b3, kx_a, kx_b, occ_b, occ_a, (int64_t)n3, 0, 32, st);
  cub::DeviceScan::ExclusiveSum(nullptr, b4, first, vid, (int64_t)n3, st);
  tmp_bytes = std::max(std::max(b1, b2), std::max(b3, b4));
  size_t b5 = 0;
  cub::DeviceScan::InclusiveSum(nullptr, b5, head, run, (int64_t)n3, st);
  tmp_bytes = std::max(tmp_bytes, b5);
  void *tmp = nullptr;
  if (cudaMalloc(&tmp, tmp_bytes ? tmp_bytes : 1) != cudaSuccess)
    return handle_fail(h, VH_ERR_CUDA, "mesh indexing: device allocation failed");
  s.ptrs.push_back(tmp);

  // 1. triangle order: stable sorts by word 11 (least significant) ... 0
  std::vector<uint32_t> iota(n);
  for (uint32_t i = 0; i < n; ++i) iota[i] = i;
  if (cudaMemcpyAsync(idx_a, iota.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st) !=
      cudaSuccess)
    return handle_fail(h, VH_ERR_CUDA, "mesh indexing: upload failed");
  for (int w = 11; w >= 0; --w) {
    k_tri_word<<<blocks_for(n), 256, 0, st>>>(tris, idx_a, n, w, word_a);
    size_t tb = tmp_bytes;
    cub::DeviceRadixSort::SortPairs(tmp, tb, word_a, word_b, idx_a, idx_b, (int64_t)n, 0, 32, st);
    std::swap(idx_a, idx_b);
  }
  // 2. occurrences grouped by position, ascending within a position
  k_occ_yz<<<blocks_for(n3), 256, 0, st>>>(tris, idx_a, n3, kyz_a, occ_a);
  size_t tb = tmp_bytes;
  cub::DeviceRadixSort::SortPairs(tmp, tb, kyz_a, kyz_b, occ_a, occ_b, (int64_t)n3, 0, 64, st);
  k_occ_x<<<blocks_for(n3), 256, 0, st>>>(tris, idx_a, occ_b, n3, kx_a);
  tb = tmp_bytes;
  cub::DeviceRadixSort::SortPairs(tmp, tb, kx_a, kx_b, occ_b, occ_a, (int64_t)n3, 0, 32, st);
  // 3. run heads, first occurrences, vertex numbers
  k_heads<<<blocks_for(n3), 256, 0, st>>>(tris, idx_a, occ_a, n3, head, first);
  tb = tmp_bytes;
  cub::DeviceScan::ExclusiveSum(tmp, tb, first, vid, (int64_t)n3, st);
  tb = tmp_bytes;
  cub::DeviceScan::InclusiveSum(tmp, tb, head, run, (int64_t)n3, st);
  k_run_first<<<blocks_for(n3), 256, 0, st>>>(occ_a, head, run, n3, run_first);
  // 4. faces and vertices
  k_emit<<<blocks_for(n3), 256, 0, st>>>(tris, idx_a, occ_a, run, run_first, first, vid, n3, voxel,
                                         d_faces, d_vert, d_col);
  uint32_t last[2] = {0, 0};
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(&last[0], vid + (n3 - 1), 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&last[1], first + (n3 - 1), 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return handle_fail(h, VH_ERR_CUDA, "mesh indexing failed");
  const size_t nv = (size_t)last[0] + last[1];
  vert.resize(3 * nv);
  col.resize(3 * nv);
  faces.resize(n3);
  if (cudaMemcpyAsync(vert.data(), d_vert, sizeof(float) * 3 * nv, cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaMemcpyAsync(col.data(), d_col, 3 * nv, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(faces.data(), d_faces, sizeof(int32_t) * n3, cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return handle_fail(h, VH_ERR_CUDA, "mesh indexing: download failed");
  return VH_OK;
}

}  // namespace vh
