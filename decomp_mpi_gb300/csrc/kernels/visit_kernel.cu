// Element-wise kernels over a distributed array gathered to global C order
// (the device visitors of include/dmg_visit.h): the scaling of decomp_scale
// (reference dimscale.c:7-67) and the index pattern of test.c:27.
#include <cuda_runtime.h>
#include <cstdint>
#include "../host/dmg_internal.h"

namespace {

// g[x] *= f0[x0] * f1[x1] * f2[x2] (conjugated when conj_f), left alone where the product is 0
template <typename R>
__global__ void scale_kernel(R *g, int L0, int L1, int L2, const R *f0, const R *f1, const R *f2, int conj_f) {
  const int64_t N = (int64_t)L0 * L1 * L2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const int x2 = (int)(i % L2);
    const int64_t r = i / L2;
    const int x1 = (int)(r % L1);
    const int x0 = (int)(r / L1);
    // running product in the reference's order: dimension 0 first
    R fr = f0[2 * x0], fi = f0[2 * x0 + 1];
    R ar = f1[2 * x1], ai = f1[2 * x1 + 1];
    const R tr = fr * ar - fi * ai, ti = fr * ai + fi * ar;
    ar = f2[2 * x2];
    ai = f2[2 * x2 + 1];
    fr = tr * ar - ti * ai;
    fi = tr * ai + ti * ar;
    if (fr == R(0) && fi == R(0)) continue;
    if (conj_f) fi = -fi;
    const R vr = g[2 * i], vi = g[2 * i + 1];
    g[2 * i] = fr * vr - fi * vi;
    g[2 * i + 1] = fr * vi + fi * vr;
  }
}

template <typename I>
__global__ void iota_kernel(I *g, int64_t N) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    g[i] = (I)i;
}

int grid_of(int64_t n) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int64_t g = (n + 255) / 256;
  if (g > (int64_t)nsm * 8) g = (int64_t)nsm * 8;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace

extern "C" int dmg_scale_global_launch(void *g, int complex64, int L0, int L1, int L2, const void *f0, const void *f1,
                                       const void *f2, int conj_f, void *stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t N = (int64_t)L0 * L1 * L2;
  if (complex64)
    scale_kernel<float><<<grid_of(N), 256, 0, s>>>(static_cast<float *>(g), L0, L1, L2, static_cast<const float *>(f0),
                                                   static_cast<const float *>(f1), static_cast<const float *>(f2),
                                                   conj_f);
  else
    scale_kernel<double><<<grid_of(N), 256, 0, s>>>(static_cast<double *>(g), L0, L1, L2,
                                                    static_cast<const double *>(f0), static_cast<const double *>(f1),
                                                    static_cast<const double *>(f2), conj_f);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "scale launch: %s", cudaGetErrorString(e));
  return DMG_OK;
}

extern "C" int dmg_iota_launch(void *g, int type_size, long long n, void *stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (type_size == 8)
    iota_kernel<long long><<<grid_of(n), 256, 0, s>>>(static_cast<long long *>(g), n);
  else if (type_size == 4)
    iota_kernel<int><<<grid_of(n), 256, 0, s>>>(static_cast<int *>(g), n);
  else
    return dmg_error(DMG_ERR_ARG, "index fill: elements of %d bytes (4 or 8)", type_size);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dmg_error(DMG_ERR_CUDA, "index fill launch: %s", cudaGetErrorString(e));
  return DMG_OK;
}
