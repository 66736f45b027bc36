// FFT pass kernels in one arithmetic (double), inverse direction, the lengths that are
// not powers of two (and the runtime-length kernel, alone or grouped); see fft_pass.cuh.
// native FP64 passes: 128-thread blocks, three per SM, 1024-value complex128 tiles
#define DMG_FFT_NT DMG_FFT_FP64_NT
#define DMG_FFT_MINB DMG_FFT_FP64_MINB
#define DMG_FFT_TILE_TARGET(es) ((es) == 8 ? 4096 : DMG_FFT_TILE_TARGET_FP64)
#include "fft_pass.cuh"

int dmg_fft_pass_f64_inv_mixed(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  return launch_other_group<double, 1>(*p, *b, stream);
}

int dmg_fft_pass_f64_inv_group(const dmg_fft_group *g, void *stream) {
  return launch_group<double, 1>(*g, static_cast<cudaStream_t>(stream));
}
