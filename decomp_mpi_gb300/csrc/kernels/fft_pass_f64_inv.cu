// FFT pass kernels in one arithmetic (double), inverse direction, power-of-two lengths; see fft_pass.cuh.
// native FP64 passes: 128-thread blocks, three per SM, 1024-value complex128 tiles
#define DMG_FFT_NT DMG_FFT_FP64_NT
#define DMG_FFT_MINB DMG_FFT_FP64_MINB
#define DMG_FFT_TILE_TARGET(es) ((es) == 8 ? 4096 : DMG_FFT_TILE_TARGET_FP64)
#include "fft_pass.cuh"

int dmg_fft_pass_f64_inv_pow2(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  return launch_pow2_group<double, 1>(*p, *b, stream);
}
