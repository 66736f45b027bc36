// FFT pass kernels in one arithmetic (double): the checks and the choice of
// translation unit, and the forward direction's power-of-two lengths; see fft_pass.cuh.
// native FP64 passes: 128-thread blocks, three per SM, 1024-value complex128 tiles
#define DMG_FFT_NT DMG_FFT_FP64_NT
#define DMG_FFT_MINB DMG_FFT_FP64_MINB
#define DMG_FFT_TILE_TARGET(es) ((es) == 8 ? 4096 : DMG_FFT_TILE_TARGET_FP64)
#include "fft_pass.cuh"

size_t dmg_fft_pass_smem_f64(const dmg_fft_pass *p) { return pass_smem<double>(*p); }

// the other groups of lengths and the inverse direction (fft_pass_f64_inv.cu,
// fft_pass_f64_mixed.cu, fft_pass_f64_inv_mixed.cu)
int dmg_fft_pass_f64_inv_pow2(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);
int dmg_fft_pass_f64_fwd_mixed(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);
int dmg_fft_pass_f64_inv_mixed(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream);

int dmg_fft_pass_launch_f64(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  const int st = check_batch<double>(*p, *b);
  if (st != DMG_OK) return st;
  // the power-of-two kernels' buffers hold this translation unit's tiles
  if (pow2_group(p->n) && !p->radix_runtime && p->M1 * p->M2 > pow2_lines(sizeof(double2), p->n))
    return dmg_error(DMG_ERR_ARG, "fft pass: %d lines of %d points exceed the FP64 tile", p->M1 * p->M2, p->n);
  const bool inv = p->sign > 0;
  if (pow2_group(p->n) && !p->radix_runtime)
    return inv ? dmg_fft_pass_f64_inv_pow2(p, b, stream) : launch_pow2_group<double, -1>(*p, *b, stream);
  return inv ? dmg_fft_pass_f64_inv_mixed(p, b, stream) : dmg_fft_pass_f64_fwd_mixed(p, b, stream);
}
