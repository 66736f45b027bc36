// Fixed device scratch for dmg_split_run_noalloc().
//
// Some callers cannot allocate device memory at the point where they run a
// transform: code inside a region that a CUDA graph is capturing, a
// real-time loop that must not block on the allocator, or an application
// that hands all of HBM to its own pool up front.  For them the split FFT
// can keep its intermediate passes in this file-scope array instead of the
// upper half of the caller's workspace.  Every GPU that loads the library
// holds the array until the process exits.
//
// In host code the array's name is only a host-side stand-in, not a device
// address: the address is looked up with cudaGetSymbolAddress, once per
// device, with that device current, and then handed to the kernels.
#include <cuda_runtime.h>
#include <mutex>
#include "../host/dmg_internal.h"

#define DMG_NOALLOC_SCRATCH_BYTES (64ull << 20)  // 64 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[DMG_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_addr[kMaxDevices];
}  // namespace

extern "C" size_t dmg_noalloc_scratch_bytes(void) { return (size_t)DMG_NOALLOC_SCRATCH_BYTES; }

// Device address of the scratch array on the current device; the first call
// on a device looks it up (no allocation happens).
extern "C" int dmg_noalloc_scratch(void **ptr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return dmg_error(DMG_ERR_UNSUPPORTED, "device %d beyond %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return dmg_error(DMG_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    g_addr[dev] = p;
  }
  *ptr = g_addr[dev];
  return DMG_OK;
}
