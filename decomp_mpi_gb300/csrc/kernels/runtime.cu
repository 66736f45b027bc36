// Device memory, stream and error helpers used by the host planner.
#include <cuda_runtime.h>
#include <cstdio>
#include "../host/dmg_internal.h"

static thread_local void *g_stream = nullptr;

extern "C" void dmg_set_stream(void *stream) { g_stream = stream; }
extern "C" void *dmg_get_stream(void) { return g_stream; }
extern "C" void *dmg_current_stream(void) { return g_stream; }

extern "C" int dmg_device_synchronize(void) {
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "cudaDeviceSynchronize: %s", cudaGetErrorString(e));
  return DMG_OK;
}

extern "C" int dmg_dev_alloc(void **ptr, size_t bytes) {
  cudaError_t e = cudaMalloc(ptr, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    return dmg_error(DMG_ERR_CUDA, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  }
  return DMG_OK;
}

extern "C" void dmg_dev_free(void *ptr) {
  if (ptr) cudaFree(ptr);
}

extern "C" int dmg_dev_upload(void *dst, const void *src, size_t bytes) {
  cudaError_t e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "cudaMemcpy H2D(%zu): %s", bytes, cudaGetErrorString(e));
  return DMG_OK;
}
