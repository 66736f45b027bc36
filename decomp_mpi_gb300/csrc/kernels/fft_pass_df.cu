// FFT pass kernels in one arithmetic (df), forward direction; see fft_pass.cuh.
#include "fft_pass.cuh"

size_t dmg_fft_pass_smem_df(const dmg_fft_pass *p) { return pass_smem<df>(*p); }

// the inverse direction's kernels (fft_pass_df_inv.cu)
int dmg_fft_pass_launch_df_inv(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);

int dmg_fft_pass_launch_df(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  if (p->sign > 0) return dmg_fft_pass_launch_df_inv(p, b, stream);
  return launch_pass<df, -1>(*p, *b, stream);
}
