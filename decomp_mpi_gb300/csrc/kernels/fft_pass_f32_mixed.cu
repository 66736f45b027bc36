// FFT pass kernels in one arithmetic (float), forward direction, the lengths that are
// not powers of two (and the runtime-length kernel); see fft_pass.cuh.
#include "fft_pass.cuh"

int dmg_fft_pass_f32_fwd_mixed(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  return launch_other_group<float, -1>(*p, *b, stream);
}
