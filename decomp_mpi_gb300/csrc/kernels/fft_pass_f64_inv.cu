// FFT pass kernels in one arithmetic (f64), inverse direction; see fft_pass.cuh.
#include "fft_pass.cuh"

int dmg_fft_pass_launch_f64_inv(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  return launch_pass<double, 1>(*p, *b, stream);
}
