// A caller's own kernels over a volume's block hash, written against
// include/vhashing_device.cuh the way code that uses vhashing::HashTable's
// device members (operator[], find, Apply, Filter) would be.  Test program:
// tests/test_device_table.py compiles it with nvcc into a shared library and
// calls these entry points with the vh_device_table of a fused volume.
// Inputs and outputs are host arrays; device scratch is the test's own.
#include <cstdint>

#include "vhashing_device.cuh"

using vhashing::BlockKey;
using vhashing::BlockRef;
using vhashing::DeviceBlockTable;

namespace {

// find and operator[] per key: the pool index and the block's first sdf
// and last weight (-1000 where the key is absent).
__global__ void lookup_kernel(DeviceBlockTable t, const int32_t *xyz, int n, int32_t *ids,
                              float *sdf0, float *w511) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const BlockKey k{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
  ids[i] = t.find(k);
  const BlockRef r = t[k];
  sdf0[i] = r.valid() ? r.sdf[0] : -1000.0f;
  w511[i] = r.valid() ? r.weight[511] : -1000.0f;
}

// Apply: every live block adds its weights (whole numbers) and itself.
struct WeightSum {
  unsigned long long *total;
  unsigned long long *blocks;
  __device__ void operator()(BlockKey, BlockRef b) const {
    unsigned long long s = 0;
    for (int v = 0; v < VH_BLOCK_VOXELS; ++v) s += (unsigned long long)b.weight[v];
    atomicAdd(total, s);
    atomicAdd(blocks, 1ull);
  }
};

// Filter: blocks with a voxel observed at least w_min times.
struct Observed {
  float w_min;
  __device__ bool operator()(BlockKey, BlockRef b) const {
    for (int v = 0; v < VH_BLOCK_VOXELS; ++v)
      if (b.weight[v] >= w_min) return true;
    return false;
  }
};

// ApplyVoxels: caps every voxel's weight.
struct CapWeight {
  float cap;
  __device__ void operator()(BlockKey, int v, BlockRef b) const {
    if (b.weight[v] > cap) b.weight[v] = cap;
  }
};

cudaStream_t stream_of(const vh_device_table *t) { return static_cast<cudaStream_t>(t->stream); }

template <typename T>
struct Dev {
  T *p = nullptr;
  explicit Dev(size_t n) {
    if (cudaMalloc(&p, sizeof(T) * (n ? n : 1)) != cudaSuccess) p = nullptr;
  }
  ~Dev() { cudaFree(p); }
};

}  // namespace

extern "C" {

// 0 on success; else a CUDA error code or -1 (bad argument).
int dt_lookup(const vh_device_table *t, const int32_t *xyz, int n, int32_t *ids, float *sdf0,
              float *w511) {
  if (!t || n < 0) return -1;
  if (cudaSetDevice(t->device) != cudaSuccess) return -1;
  Dev<int32_t> dx(3 * (size_t)n), di(n);
  Dev<float> ds(n), dw(n);
  if (!dx.p || !di.p || !ds.p || !dw.p) return -1;
  const cudaStream_t s = stream_of(t);
  cudaMemcpyAsync(dx.p, xyz, sizeof(int32_t) * 3 * n, cudaMemcpyHostToDevice, s);
  if (n) lookup_kernel<<<(n + 127) / 128, 128, 0, s>>>(DeviceBlockTable(*t), dx.p, n, di.p, ds.p, dw.p);
  cudaMemcpyAsync(ids, di.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(sdf0, ds.p, sizeof(float) * n, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(w511, dw.p, sizeof(float) * n, cudaMemcpyDeviceToHost, s);
  return (int)cudaStreamSynchronize(s);
}

int dt_weight_sum(const vh_device_table *t, unsigned long long *total_and_blocks) {
  if (!t || cudaSetDevice(t->device) != cudaSuccess) return -1;
  Dev<unsigned long long> d(2);
  if (!d.p) return -1;
  const cudaStream_t s = stream_of(t);
  cudaMemsetAsync(d.p, 0, 2 * sizeof(unsigned long long), s);
  if (vhashing::Apply(DeviceBlockTable(*t), WeightSum{d.p, d.p + 1}) != VH_OK) return -2;
  cudaMemcpyAsync(total_and_blocks, d.p, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
  return (int)cudaStreamSynchronize(s);
}

int dt_filter(const vh_device_table *t, float w_min, int32_t *xyz, int32_t *ids, long long cap,
              unsigned long long *count) {
  if (!t || cap < 0 || cudaSetDevice(t->device) != cudaSuccess) return -1;
  Dev<int32_t> dx(3 * (size_t)cap), di((size_t)cap);
  Dev<unsigned long long> dc(1);
  if (!dx.p || !di.p || !dc.p) return -1;
  const cudaStream_t s = stream_of(t);
  if (vhashing::Filter(DeviceBlockTable(*t), Observed{w_min}, dx.p, di.p, cap, dc.p) != VH_OK)
    return -2;
  cudaMemcpyAsync(count, dc.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return -3;
  const unsigned long long m = *count < (unsigned long long)cap ? *count : (unsigned long long)cap;
  cudaMemcpyAsync(xyz, dx.p, sizeof(int32_t) * 3 * m, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(ids, di.p, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, s);
  return (int)cudaStreamSynchronize(s);
}

int dt_cap_weights(const vh_device_table *t, float cap) {
  if (!t || cudaSetDevice(t->device) != cudaSuccess) return -1;
  if (vhashing::ApplyVoxels(DeviceBlockTable(*t), CapWeight{cap}) != VH_OK) return -2;
  return (int)cudaStreamSynchronize(stream_of(t));
}

}  // extern "C"
