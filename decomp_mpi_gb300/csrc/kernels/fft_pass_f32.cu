// FFT pass kernels in one arithmetic (float); see fft_pass.cuh.
#include "fft_pass.cuh"

size_t dmg_fft_pass_smem_f32(const dmg_fft_pass *p) { return pass_smem<float>(*p); }

int dmg_fft_pass_launch_f32(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  return launch_pass<float>(*p, *b, stream);
}
