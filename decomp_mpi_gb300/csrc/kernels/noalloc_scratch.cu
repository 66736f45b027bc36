// Fixed device scratch for dmg_split_run_noalloc().
//
// Some callers cannot allocate device memory at the point where they run a
// transform: a real-time loop that must not block on the allocator, or an
// application that hands all of HBM to its own pool up front.  For them the
// split FFT can keep its intermediate passes in this file-scope array
// instead of the upper half of the caller's workspace.
//
// When the array is reserved: CUDA loads a library's modules lazily, and
// the array belongs to this file's module, so a device holds the array from
// the first time the module is loaded on it until the process exits.  The
// library loads it when it uploads the tables of a plan small enough for the
// no-allocation run (dmg_noalloc_scratch_reserve, called from the upload
// that any regular run of the plan performs), so that the no-allocation call
// itself finds the array already in place.
//
// In host code the array's name is only a host-side stand-in, not a device
// address: the address is looked up with cudaGetSymbolAddress, with the
// device current, on every call (the lookup is cheap and never stale), and
// then handed to the kernels.
#include <cuda_runtime.h>
#include "../host/dmg_internal.h"

#define DMG_NOALLOC_SCRATCH_BYTES (64ull << 20)  // 64 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[DMG_NOALLOC_SCRATCH_BYTES];

extern "C" size_t dmg_noalloc_scratch_bytes(void) { return (size_t)DMG_NOALLOC_SCRATCH_BYTES; }

// Device address of the scratch array on the current device.
extern "C" int dmg_noalloc_scratch(void **ptr) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return dmg_error(DMG_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
  *ptr = p;
  return DMG_OK;
}

// Load this file's module on the current device (which reserves the array)
// without recording an error: 0 when the array is in place.  A failure is
// left for dmg_split_run_noalloc to report.
extern "C" int dmg_noalloc_scratch_reserve(void) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) {
    cudaGetLastError();  // not sticky: leave no error behind for the caller's next CUDA call
    return 1;
  }
  return 0;
}
