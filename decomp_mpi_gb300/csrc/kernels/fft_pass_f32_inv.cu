// FFT pass kernels in one arithmetic (f32), inverse direction; see fft_pass.cuh.
#include "fft_pass.cuh"

int dmg_fft_pass_launch_f32_inv(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  return launch_pass<float, 1>(*p, *b, stream);
}
