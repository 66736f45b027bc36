// FFT pass kernels of the tensor-core form (complex64 data): the 1024-point
// lines run their two 32-point DFT products on the tensor cores, both
// directions; every other length runs the FP32 stages.  See fft_pass.cuh.
#include "fft_pass.cuh"

int dmg_fft_pass_launch_f32(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);

size_t dmg_fft_pass_smem_f32(const dmg_fft_pass *p);

size_t dmg_fft_pass_smem_tc(const dmg_fft_pass *p) {
  return p->n == 1024 && !p->radix_runtime ? smem_layout<float>(*p, true, true).total : dmg_fft_pass_smem_f32(p);
}

int dmg_fft_pass_launch_tc(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  if (p->n != 1024 || p->radix_runtime) return dmg_fft_pass_launch_f32(p, b, stream);
  const int st = check_batch<float>(*p, *b);
  if (st != DMG_OK) return st;
  // a tile's lines make the products' 128 rows: at most four 1024-point lines
  if (p->M1 * p->M2 > 4) return dmg_error(DMG_ERR_ARG, "tensor-core pass: %d lines per tile (at most 4)", p->M1 * p->M2);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return p->sign > 0 ? launch_k<float, 1, 1024, true>(*p, *b, s) : launch_k<float, -1, 1024, true>(*p, *b, s);
}
