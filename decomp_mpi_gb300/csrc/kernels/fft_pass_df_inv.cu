// FFT pass kernels in one arithmetic (df), inverse direction; see fft_pass.cuh.
#include "fft_pass.cuh"

int dmg_fft_pass_launch_df_inv(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  return launch_pass<df, 1>(*p, *b, stream);
}
