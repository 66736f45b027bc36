// Host-only dump of the power-of-two stage layouts the pass kernels use: for
// each value type (8- and 16-byte), length NF and stage, the radix schedule
// and the swizzle g of the buffer the stage reads.  tests/test_swizzle.py
// compiles this with nvcc and checks the dump on the CPU (no GPU needed).
#include <cstdio>
#include "fft_pass.cuh"

template <typename T, int NF, int LP>
void dump_stage() {
  if constexpr (LP < NF) {
    constexpr int R = fixed_radix(NF, LP);
    constexpr int tile = DMG_FFT_TILE_TARGET(sizeof(C2<T>));
    std::printf("stage es=%d nf=%d lp=%d r=%d\n", (int)sizeof(C2<T>), NF, LP, R);
    if constexpr (LP > 1) {
      std::printf("g");
      for (int x = 0; x < tile; ++x) std::printf(" %d", HopSwz<T, NF, LP>::g(x));
      std::printf("\n");
    }
    dump_stage<T, NF, LP * R>();
  }
}

template <typename T>
void dump_type() {
  dump_stage<T, 16, 1>();
  dump_stage<T, 32, 1>();
  dump_stage<T, 64, 1>();
  dump_stage<T, 128, 1>();
  dump_stage<T, 256, 1>();
  dump_stage<T, 512, 1>();
  dump_stage<T, 1024, 1>();
  dump_stage<T, 2048, 1>();
}

int main() {
  dump_type<float>();
  dump_type<df>();
  return 0;
}
