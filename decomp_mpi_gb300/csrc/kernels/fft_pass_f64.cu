// FFT pass kernels in one arithmetic (double); see fft_pass.cuh.
#include "fft_pass.cuh"

size_t dmg_fft_pass_smem_f64(const dmg_fft_pass *p) { return pass_smem<double>(*p); }

// the inverse direction's kernels (fft_pass_f64_inv.cu)
int dmg_fft_pass_launch_f64_inv(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);

int dmg_fft_pass_launch_f64(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  if (p->sign > 0) return dmg_fft_pass_launch_f64_inv(p, b, stream);
  return launch_pass<double, -1>(*p, *b, stream);
}
