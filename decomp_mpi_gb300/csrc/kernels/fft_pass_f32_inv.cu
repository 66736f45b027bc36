// FFT pass kernels in one arithmetic (float), inverse direction, power-of-two lengths; see fft_pass.cuh.
#include "fft_pass.cuh"

int dmg_fft_pass_f32_inv_pow2(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  return launch_pow2_group<float, 1>(*p, *b, stream);
}
