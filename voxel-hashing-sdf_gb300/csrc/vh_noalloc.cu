// vh_noalloc.cu - key lookup that allocates no device memory.
//
// vh_find_keys with host buffers copies the keys to a temporary device buffer
// and the answers back through another, both taken with cudaMalloc and given
// back with cudaFree on every call.  Some callers cannot allow that: a control
// loop with a latency budget cannot absorb cudaMalloc's unbounded cost or
// cudaFree's implicit device-wide synchronisation, which also stalls every
// other stream on the GPU; a component embedded in a host framework that owns
// all device memory is not permitted to allocate at all.  vh_find_keys_noalloc
// serves them: its scratch is a fixed array in this library's device image,
// created when the library is loaded onto a GPU and held until the process
// exits, so a call only copies, launches and copies back.

#include <mutex>

#include "vh_internal.h"

namespace {

// Keys (3 int32 each) followed by one int32 answer per key.
constexpr int64_t kMaxKeys = VH_FIND_NOALLOC_MAX_KEYS;
constexpr size_t kScratchWords = 4 * (size_t)kMaxKeys;

// Every GPU that loads the library holds this array (1 MiB) until exit.  In
// host code the name only stands in for the symbol; the device address comes
// from cudaGetSymbolAddress below.
static __device__ __align__(256) int32_t g_find_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
int32_t *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on `device`, looked up once per device
// with that device current (the caller's current device is restored).  The
// address stays valid while the device's primary context lives, i.e. until
// the process exits unless someone calls cudaDeviceReset on that device,
// which also invalidates every handle there (documented in vhsdf.h).
cudaError_t scratch_for(int device, int32_t **out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  if (!g_scratch_ptr[device]) {
    int prev = 0;
    cudaError_t e = cudaGetDevice(&prev);
    if (e != cudaSuccess) return e;
    if (prev != device && (e = cudaSetDevice(device)) != cudaSuccess) return e;
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_find_scratch);
    if (prev != device) cudaSetDevice(prev);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[device] = static_cast<int32_t *>(p);
  }
  *out = g_scratch_ptr[device];
  return cudaSuccess;
}

}  // namespace

extern "C" vh_status vh_find_keys_noalloc(vh_handle *h, const int32_t *xyz, int64_t n,
                                          int32_t *out_block) {
  VH_HANDLE_DEVICE(h);
  if (!h || n < 0 || (n && (!xyz || !out_block))) return VH_ERR_INVALID_ARG;
  if (n > kMaxKeys)
    return vh::handle_fail(h, VH_ERR_CAPACITY,
                           "vh_find_keys_noalloc: more keys than VH_FIND_NOALLOC_MAX_KEYS");
  if (!n) return VH_OK;
  int32_t *scratch = nullptr;
  cudaError_t e = scratch_for(vh::handle_device(h), &scratch);
  if (e != cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, "vh_find_keys_noalloc: scratch set-up failed");
  int32_t *d_keys = scratch;                  // 3n words
  int32_t *d_out = scratch + 3 * kMaxKeys;    // n words, all written by the kernel
  const cudaStream_t s = vh::handle_stream(h);
  if ((e = cudaMemcpyAsync(d_keys, xyz, sizeof(int32_t) * 3 * n, cudaMemcpyHostToDevice, s)) !=
      cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, cudaGetErrorString(e));
  vh::launch_find_keys(vh::handle_view(h), d_keys, (uint32_t)n, d_out, s);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, cudaGetErrorString(e));
  if ((e = cudaMemcpyAsync(out_block, d_out, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s)) !=
      cudaSuccess)
    return vh::handle_fail(h, VH_ERR_CUDA, cudaGetErrorString(e));
  return vh::handle_sync(h);
}
