#ifndef DMG_FFT_PARAMS_H
#define DMG_FFT_PARAMS_H
/*
 * Launch parameters of one FFT pass, shared by the C planner and the CUDA
 * source.
 *
 * The global coordinate of dimension d is split as x_d = y_d + A_d * z_d
 * (y_d < A_d, z_d < B_d).  Sub-axis s (0..5) is y of dim s/2 when s is even
 * and z of dim s/2 when s is odd.  A pass transforms every line along one
 * sub-axis t (length n) and moves the data from an input layout to an
 * output layout, each given by per-dimension address tables over x_d.
 *
 * A block holds a tile of n x M1 x M2 values: the transform sub-axis t and
 * two vector sub-axes v1, v2 (lines next to each other in memory), and
 * loads/stores them in the orders that make the accesses contiguous.
 *
 * A "line" pass transforms a whole dimension at once: the planner passes
 * A_d = L_d, B_d = 1 for every dimension, so that sub-axis 2d is x_d.  Its
 * output order along the transformed dimension is the split FFT's slot
 * order: slot s holds frequency k = s / pA + pB * (s % pA) (the plan's A_d
 * and B_d), applied when the tile is stored (forward) or loaded (inverse).
 */
#include <stdint.h>

#define DMG_FFT_MAXDIM 3
#define DMG_FFT_MAXFAC 16

struct dmg_fft_layout {
  const int64_t *tab[DMG_FFT_MAXDIM]; /* separable: address part per x_d; ranked: type offset */
  const int32_t *rk[DMG_FFT_MAXDIM];  /* ranked: rank part per x_d */
  const int64_t *rstride;             /* ranked: [ndim][nranks] strides */
  int64_t pitch;                      /* ranked: elements per virtual rank */
  int64_t base;                       /* element offset added to every address */
  int32_t nranks;
  int32_t ranked;
};

struct dmg_fft_pass {
  int32_t ndim;
  int32_t A[DMG_FFT_MAXDIM], B[DMG_FFT_MAXDIM], L[DMG_FFT_MAXDIM];
  int32_t t, v1, v2;           /* sub-axes (v1/v2 = -1 when absent) */
  int32_t n, nv1, nv2;         /* their lengths */
  int32_t M1, M2;              /* tile extents along v1, v2 */
  int32_t nt1, nt2;            /* tiles along v1, v2 */
  int32_t nbatch;
  int32_t bsub[6], blen[6];    /* batch sub-axes and lengths */
  int64_t ntiles;
  int32_t load_order[3];       /* tile axes (0 = t, 1 = v1, 2 = v2), fastest first */
  int32_t store_order[3];
  /* the same geometry in the form the kernel uses without indexing arrays:
   * for tile axis k (0 t, 1 v1, 2 v2): the dimension it belongs to (-1 when
   * absent) and whether it is the z sub-axis; and its position (0 fastest,
   * 1, 2 slowest) in the load and the store orders */
  int32_t kdim[3], kisz[3];
  int32_t load_pos[3], store_pos[3];
  int32_t nfac;
  int32_t fac[DMG_FFT_MAXFAC]; /* radices, first stage first */
  int32_t radix_runtime;       /* run the radices above in the runtime-length kernel even where the length has
                                  a compile-time schedule */
  const void *roots;           /* n roots exp(-2 pi i k / n), double2 or float2 */
  int32_t sign;                /* -1 forward, +1 inverse */
  /* split twiddle of the transformed dimension d = t/2 (t a z sub-axis):
   * 0 none; 1 multiply after the transform by exp(-2 pi i y_d k_d / L_d);
   * 2 multiply by its conjugate before the transform */
  int32_t twiddle;
  /* per dim: the split twiddles exp(-2 pi i y k / L_d) (y < A_d, k < B_d)
   * at k * A_d + y (twk) and at y * B_d + k (twy), so that lanes stepping
   * along either read neighbouring entries */
  const void *twk[DMG_FFT_MAXDIM], *twy[DMG_FFT_MAXDIM];
  /* double-float passes (dtype 2): whether the input / output is stored as
   * complex128 (converted at load / store, scaled by 2^-E / 2^E) rather
   * than as double-float pairs; E = *scale_exp */
  int32_t in_fp64, out_fp64;
  const int32_t *scale_exp;
  /* slot order along the transform axis on the load / store side (line
   * passes): tile coordinate s along t is layout slot s, whose value sits at
   * line position s / perm_a + perm_b * (s % perm_a) */
  int32_t perm_in, perm_out, perm_a, perm_b;
  /* the side's address is base + f0(c0) + f1(c1) + f2(c2) over the tile
   * axes (layout not ranked and the tile axes in different dimensions): the
   * kernel tabulates f0, f1, f2 once per tile */
  int32_t sep_in, sep_out;
  /* separable side whose transform-axis table is the same for every tile
   * (no batch sub-axis in that dimension) and whose entries lie within
   * 2^31 of the first: the kernel may keep them in shared memory as int32
   * offsets from that entry */
  int32_t t0_rel_in, t0_rel_out;
  /* a side whose layout is separable over dimensions but two of whose tile
   * axes (semi_a < semi_b) lie in one dimension: its address is the tables
   * of the other dimensions plus that dimension's table at the coordinate
   * both axes make up */
  int32_t semi_in, semi_out, semi_a, semi_b;
  /* a separable side (sep_*) whose tile axes semi_a and semi_b lie in one
   * dimension whose table is the sum of a part along each of its two
   * sub-axes (tab[y + A z] = tab[y] + tab[A z] - tab[0]): the transform
   * axis's and the vector axis's entries both count the tile's start in that
   * dimension, which the side's base takes off once */
  int32_t pair_in, pair_out;
  struct dmg_fft_layout in, out;
  /* device word set to 1 when a tensor-core pass gave up waiting for its
   * products (NULL: not reported) */
  int32_t *status;
  /* the tile holds more than DMG_FFT_TILE_TARGET values: the wide kernel */
  int32_t wide;
};

/* Threads per pass block; the most values a tile may hold, and the number
 * the planner aims at (32 KB per tile buffer) for a value of es bytes. */
#ifndef DMG_FFT_NT
#define DMG_FFT_NT 256
#endif
#ifndef DMG_FFT_TILE_MAX
#define DMG_FFT_TILE_MAX 4096
#endif
#ifndef DMG_FFT_TILE_TARGET
#define DMG_FFT_TILE_TARGET(es) ((es) == 8 ? 4096 : 2048)
#endif
/* Native FP64 passes (complex128): 128-thread blocks, three per SM, with
 * tiles of 1024 values.  The passes are bound by the FP64 pipe; more and
 * smaller blocks keep it busier while other blocks gather, scatter or wait
 * at a barrier (about 4 % faster than two 256-thread blocks with 2048-value
 * tiles at 512^3).  The FP64 translation units compile the pass kernel with
 * these sizes and the planner gives FP64 passes tiles of at most this many
 * values (a whole line where a line is longer). */
#define DMG_FFT_FP64_NT 128
#define DMG_FFT_FP64_MINB 3
#define DMG_FFT_TILE_TARGET_FP64 1024
/* Wide passes: one 512-thread block per SM with tiles of twice the values,
 * so that passes whose lines are strided in memory move rows twice as long
 * (FP32 and double-float power-of-two lengths; the plan's tile size asks for
 * them). */
#define DMG_FFT_WIDE_NT 512
#define DMG_FFT_WIDE_TILE(es) ((es) == 8 ? 8192 : 4096)

/* Jobs of one batched launch: the same pass (same plan, so the same tables)
 * over several arrays.  scale_exp: per job, for double-float passes that
 * read or write complex128. */
#define DMG_FFT_MAXBATCH 16
struct dmg_fft_batch {
  int32_t count;
  const void *src[DMG_FFT_MAXBATCH];
  void *dst[DMG_FFT_MAXBATCH];
  const int32_t *scale_exp[DMG_FFT_MAXBATCH];
};

/* Passes of different plans (any lengths; each pass run by the
 * runtime-length stages) in one launch: job j's pass runs on blocks
 * first_block .. first_block + nblocks - 1 of the grid as if they were its
 * own launch (the launcher fills in first_block and nblocks). */
#define DMG_FFT_MAXGROUP 16
struct dmg_fft_group_job {
  struct dmg_fft_pass p;
  struct dmg_fft_batch bt;
  int64_t first_block, nblocks;
};
struct dmg_fft_group {
  int32_t count;
  struct dmg_fft_group_job job[DMG_FFT_MAXGROUP];
};

#ifdef __cplusplus
extern "C" {
#endif
/* One launch over a group of passes of one arithmetic (dtype as below) and
 * direction, each with radix_runtime set. */
int dmg_fft_pass_launch_group(const struct dmg_fft_group *g, int dtype, void *stream);
/* One launch of a pass over every job of a batch (the tiles of all jobs
 * share the persistent blocks). */
int dmg_fft_pass_launch_batch(const struct dmg_fft_pass *p, int dtype, const struct dmg_fft_batch *b, void *stream);
/* dtype 0: complex128 in FP64 arithmetic, 1: complex64 in FP32, 2: complex128
 * data in double-float (FP32 pair) arithmetic, 3: complex64 with the
 * 1024-point passes' DFTs on the tensor cores (FP16 hi + lo operands, FP32
 * accumulation; other lengths as dtype 1). */
int dmg_fft_pass_launch(const struct dmg_fft_pass *p, int dtype, const void *src, void *dst, void *stream);
/* Largest biased FP64 exponent of max(|re|, |im|) over the N = prod(L)
 * complex128 elements of a layout, into *out (which the call first sets to 0). */
int dmg_fft_maxexp_launch(const struct dmg_fft_layout *lay, int ndim, const int32_t *A, const int32_t *L,
                          const void *src, int32_t *out, void *stream);
/* Shared memory bytes a pass needs. */
size_t dmg_fft_pass_smem(const struct dmg_fft_pass *p, int dtype);
#ifdef __cplusplus
}
#endif
#endif
