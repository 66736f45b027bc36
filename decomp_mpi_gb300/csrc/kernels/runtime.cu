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

// Copy between host and device on a stream and wait for it (file I/O paths).
extern "C" int dmg_copy_sync(void *dst, const void *src, size_t bytes, int to_host, void *stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, to_host ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "copy of %zu bytes: %s", bytes, cudaGetErrorString(e));
  return DMG_OK;
}

extern "C" int dmg_stream_sync(void *stream) {
  cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "cudaStreamSynchronize: %s", cudaGetErrorString(e));
  return DMG_OK;
}

// Streams, events and asynchronous copies for the request server.
extern "C" int dmg_rt_stream_create(void **s) {
  cudaStream_t st = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  *s = st;
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  return DMG_OK;
}
extern "C" void dmg_rt_stream_destroy(void *s) {
  if (s) cudaStreamDestroy(static_cast<cudaStream_t>(s));
}
extern "C" int dmg_rt_event_create(void **ev) {
  cudaEvent_t e = nullptr;
  cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  *ev = e;
  if (r != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "cudaEventCreate: %s", cudaGetErrorString(r));
  return DMG_OK;
}
extern "C" void dmg_rt_event_destroy(void *ev) {
  if (ev) cudaEventDestroy(static_cast<cudaEvent_t>(ev));
}
extern "C" int dmg_rt_event_record(void *ev, void *s) {
  cudaError_t r = cudaEventRecord(static_cast<cudaEvent_t>(ev), static_cast<cudaStream_t>(s));
  if (r != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "cudaEventRecord: %s", cudaGetErrorString(r));
  return DMG_OK;
}
// 1 when the work before the event has completed, 0 while it runs, an error code otherwise
extern "C" int dmg_rt_event_done(void *ev) {
  cudaError_t r = cudaEventQuery(static_cast<cudaEvent_t>(ev));
  if (r == cudaSuccess) return 1;
  if (r == cudaErrorNotReady) return 0;
  return -dmg_error(DMG_ERR_CUDA, "cudaEventQuery: %s", cudaGetErrorString(r));
}
// kind: 0 host->device, 1 device->host, 2 device->device
extern "C" int dmg_rt_copy_async(void *dst, const void *src, size_t bytes, int kind, void *s) {
  const cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice : kind == 1 ? cudaMemcpyDeviceToHost
                                                                          : cudaMemcpyDeviceToDevice;
  cudaError_t r = cudaMemcpyAsync(dst, src, bytes, k, static_cast<cudaStream_t>(s));
  if (r != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "cudaMemcpyAsync(%zu): %s", bytes, cudaGetErrorString(r));
  return DMG_OK;
}
extern "C" int dmg_rt_copy2d_async(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width,
                                   size_t height, int kind, void *s) {
  const cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice : kind == 1 ? cudaMemcpyDeviceToHost
                                                                          : cudaMemcpyDeviceToDevice;
  cudaError_t r = cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, k, static_cast<cudaStream_t>(s));
  if (r != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "cudaMemcpy2DAsync: %s", cudaGetErrorString(r));
  return DMG_OK;
}
extern "C" int dmg_rt_get_device(int *dev) {
  cudaError_t r = cudaGetDevice(dev);
  if (r != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(r));
  return DMG_OK;
}
extern "C" int dmg_rt_set_device(int dev) {
  cudaError_t r = cudaSetDevice(dev);
  if (r != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(r));
  return DMG_OK;
}

// CUDA-event pairs used by plan timing and the autotuner.
struct dmg_events {
  int count;
  cudaEvent_t *ev;
};

extern "C" void *dmg_split_create_events(int count) {
  dmg_events *e = new dmg_events;
  e->count = count;
  e->ev = new cudaEvent_t[count];
  for (int i = 0; i < count; ++i) cudaEventCreate(&e->ev[i]);
  return e;
}

extern "C" void dmg_split_destroy_events(void *p) {
  dmg_events *e = static_cast<dmg_events *>(p);
  if (!e) return;
  for (int i = 0; i < e->count; ++i) cudaEventDestroy(e->ev[i]);
  delete[] e->ev;
  delete e;
}

extern "C" int dmg_split_record_event(void *p, int idx, void *stream) {
  dmg_events *e = static_cast<dmg_events *>(p);
  if (!e || idx < 0 || idx >= e->count) return dmg_error(DMG_ERR_ARG, "event index %d", idx);
  cudaError_t err = cudaEventRecord(e->ev[idx], static_cast<cudaStream_t>(stream));
  if (err != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "cudaEventRecord: %s", cudaGetErrorString(err));
  return DMG_OK;
}

extern "C" int dmg_split_event_elapsed(void *p, int a, int b, float *ms) {
  dmg_events *e = static_cast<dmg_events *>(p);
  if (!e || a < 0 || b < 0 || a >= e->count || b >= e->count) return dmg_error(DMG_ERR_ARG, "event index");
  cudaError_t err = cudaEventSynchronize(e->ev[b]);
  if (err == cudaSuccess) err = cudaEventElapsedTime(ms, e->ev[a], e->ev[b]);
  if (err != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "event timing: %s", cudaGetErrorString(err));
  return DMG_OK;
}
