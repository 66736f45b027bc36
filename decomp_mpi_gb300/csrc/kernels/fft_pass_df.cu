// FFT pass kernels in one arithmetic (double-float): the checks and the choice of
// translation unit, and the forward direction's power-of-two lengths; see fft_pass.cuh.
#include "fft_pass.cuh"

size_t dmg_fft_pass_smem_df_wide(const dmg_fft_pass *p);
int dmg_fft_pass_df_wide(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);
int dmg_fft_pass_df_inv_wide(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);

size_t dmg_fft_pass_smem_df(const dmg_fft_pass *p) { return p->wide ? dmg_fft_pass_smem_df_wide(p) : pass_smem<df>(*p); }

// the other groups of lengths and the inverse direction (fft_pass_df_inv.cu,
// fft_pass_df_mixed.cu, fft_pass_df_inv_mixed.cu)
int dmg_fft_pass_df_inv_pow2(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);
int dmg_fft_pass_df_fwd_mixed(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);
int dmg_fft_pass_df_inv_mixed(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);

int dmg_fft_pass_launch_df(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  const int st = check_batch<df>(*p, *b);
  if (st != DMG_OK) return st;
  const bool inv = p->sign > 0;
  if (p->wide) return inv ? dmg_fft_pass_df_inv_wide(p, b, stream) : dmg_fft_pass_df_wide(p, b, stream);
  if (pow2_group(p->n) && !p->radix_runtime)
    return inv ? dmg_fft_pass_df_inv_pow2(p, b, stream) : launch_pow2_group<df, -1>(*p, *b, stream);
  return inv ? dmg_fft_pass_df_inv_mixed(p, b, stream) : dmg_fft_pass_df_fwd_mixed(p, b, stream);
}
