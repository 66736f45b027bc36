// FFT pass kernels in one arithmetic (df); see fft_pass.cuh.
#include "fft_pass.cuh"

size_t dmg_fft_pass_smem_df(const dmg_fft_pass *p) { return pass_smem<df>(*p); }

int dmg_fft_pass_launch_df(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  return launch_pass<df>(*p, *b, stream);
}
