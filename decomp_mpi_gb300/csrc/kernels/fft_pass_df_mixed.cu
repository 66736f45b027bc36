// FFT pass kernels in one arithmetic (double-float), forward direction, the lengths that are
// not powers of two (and the runtime-length kernel, alone or grouped); see fft_pass.cuh.
#include "fft_pass.cuh"

int dmg_fft_pass_df_fwd_mixed(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  return launch_other_group<df, -1>(*p, *b, stream);
}

int dmg_fft_pass_df_fwd_group(const dmg_fft_group *g, void *stream) {
  return launch_group<df, -1>(*g, static_cast<cudaStream_t>(stream));
}
