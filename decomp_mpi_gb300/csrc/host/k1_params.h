#ifndef DMG_K1_PARAMS_H
#define DMG_K1_PARAMS_H
/*
 * Launch parameters of the reshape permutation kernel, shared by the C
 * planner and the CUDA source.
 *
 * The kernel moves, for every global coordinate g = (g_0, ..., g_{n-1}),
 *     dst[addr_dst(g)] = src[addr_src(g)]
 * in units of `unit` bytes, skipping g when either address is negative (the
 * side does not hold g).  An address is built per side from small per-axis
 * tables:
 *   separable:  addr = sum_a tab[a][g_a]
 *   ranked:     R = sum_a rk[a][g_a];  addr = R*pitch + sum_a tab[a][g_a] * rstride[a*nranks + R]
 * The ranked form serves decompositions whose memory strides differ between
 * virtual ranks (packed layouts with uneven blocks).
 */
#include <stdint.h>

#define DMG_MAXAX 8

struct dmg_k1_side {
  const int64_t *tab[DMG_MAXAX]; /* per axis: address part (separable) or type offset (ranked) */
  const int32_t *rk[DMG_MAXAX];  /* ranked: rank part per axis (negative = not held) */
  const int64_t *rstride;        /* ranked: [naxes][nranks] stride of each rank, in units */
  int64_t pitch;                 /* ranked: per-rank pitch in units */
  int32_t nranks;
  int32_t ranked;
};

struct dmg_k1_params {
  int32_t naxes;
  int32_t len[DMG_MAXAX];
  int32_t ax0, ax1;      /* tile axes; ax1 < 0 for a one-axis tile */
  int32_t e0, e1;        /* tile extents along ax0, ax1 */
  int32_t nt0, nt1;      /* tiles along ax0, ax1 */
  int32_t nbatch;        /* number of batch axes */
  int32_t batch_ax[DMG_MAXAX]; /* batch axes, fastest-varying first */
  int64_t ntiles;        /* nt0 * nt1 * product of batch lengths */
  int32_t load_fast;     /* 0: ax0 varies fastest while loading, 1: ax1 */
  int32_t store_fast;    /* same while storing */
  struct dmg_k1_side src, dst;
};

/* Several reshapes in one launch (any sizes and decompositions, each with
 * both sides contiguous along its tile's first axis, all moving units of one
 * size with the same ranked / separable sides): job j's tiles are numbered
 * from first_tile = the sum of the earlier jobs' ntiles. */
#define DMG_K1_MAXGROUP 16
struct dmg_k1_group_job {
  struct dmg_k1_params p;
  const void *src;
  void *dst;
  int64_t first_tile;
};
struct dmg_k1_group {
  int32_t count;
  int64_t total_tiles;
  struct dmg_k1_group_job job[DMG_K1_MAXGROUP];
};

#ifdef __cplusplus
extern "C" {
#endif
/* Launch the permutation kernel; unit is 1, 2, 4, 8 or 16 bytes. */
int dmg_k1_launch(const struct dmg_k1_params *p, int unit, const void *src, void *dst, void *stream);
/* One launch over a group of reshapes (see dmg_k1_group). */
int dmg_k1_launch_group(const struct dmg_k1_group *g, int unit, void *stream);
#ifdef __cplusplus
}
#endif
#endif
