// FFT pass kernels with wide tiles (float arithmetic, inverse direction, power-of-two
// lengths): one 512-thread block per SM and tiles of twice the values of the
// two-block kernels, so that passes whose lines are strided in memory move
// rows twice as long.  The same kernel as fft_pass.cuh's, compiled with these
// sizes.
#define DMG_FFT_NT 512
#define DMG_FFT_MINB 1
#define DMG_FFT_TILE_MAX 8192
#define DMG_FFT_TILE_TARGET(es) ((es) == 8 ? 8192 : 4096)
// the transform axis's offsets stay in shared memory up to the per-block limit
#define DMG_FFT_T0_SMEM_LIMIT 230400
#include "fft_pass.cuh"

int dmg_fft_pass_f32_inv_wide(const dmg_fft_pass *p, const dmg_fft_batch *b, void *stream) {
  return launch_pow2_group<float, 1>(*p, *b, stream);
}
