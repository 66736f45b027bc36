// FFT pass kernels in one arithmetic (double); see fft_pass.cuh.
#include "fft_pass.cuh"

size_t dmg_fft_pass_smem_f64(const dmg_fft_pass *p) { return pass_smem<double>(*p); }

int dmg_fft_pass_launch_f64(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  return launch_pass<double>(*p, *b, stream);
}
