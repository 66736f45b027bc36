// Device throughput probe: the FP64 and FP32 FMA rates of the GPU the
// library runs on, used as the roofline denominator of the FP64 FFT passes
// (the measured peaks file covers HBM and bf16 tensor throughput only).
#include <cuda_runtime.h>
#include "../host/dmg_internal.h"

namespace {
template <typename T>
__global__ void fma_chain(T *out, int iters, T a, T b) {
  T x0 = threadIdx.x * (T)1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
    x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b;
    x1 = x1 * a + b;
    x2 = x2 * a + b;
    x3 = x3 * a + b;
    x4 = x4 * a + b;
    x5 = x5 * a + b;
    x6 = x6 * a + b;
    x7 = x7 * a + b;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
double rate(int iters) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = nsm * 8, threads = 256;
  T *out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chain<T><<<blocks, threads>>>(out, iters / 8, (T)0.999999, (T)1e-7);
  cudaEventRecord(e0);
  fma_chain<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess || ms <= 0) return -1.0;
  return 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
}
}  // namespace

// FMA throughput in TFLOP/s (an FMA counts two flops): which 0 = FP64, 1 = FP32.
extern "C" double dmg_probe_fma_tflops(int which) { return which == 0 ? rate<double>(2048) : rate<float>(16384); }
