// FFT pass kernels in one arithmetic (float); see fft_pass.cuh.
#include "fft_pass.cuh"

size_t dmg_fft_pass_smem_f32(const dmg_fft_pass *p) { return pass_smem<float>(*p); }

// the inverse direction's kernels (fft_pass_f32_inv.cu)
int dmg_fft_pass_launch_f32_inv(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);

int dmg_fft_pass_launch_f32(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  if (p->sign > 0) return dmg_fft_pass_launch_f32_inv(p, b, stream);
  return launch_pass<float, -1>(*p, *b, stream);
}
