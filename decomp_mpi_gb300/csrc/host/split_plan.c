/*
 * Split (two-stage) 3D FFT plans on the virtual grid.
 *
 * Planning follows the reference (split_fft.c:36-77, 249-614, 747-788): the
 * same factor choice, processor grids, A (interleaved) and B (blocked)
 * decompositions, workspace check and output descriptor, so that the result
 * lands in the same slots of the workspace.  Execution is different: instead
 * of reshape -> FFTW -> twiddle -> reshape -> FFTW, every dimension's stage-1
 * and stage-2 transform is one GPU pass that gathers its lines from the
 * previous layout through address tables, so the reshapes and the twiddle are
 * fused into the transforms.  A forward run is
 *   stage 1: one pass per dimension with B_d > 1 (last dimension first),
 *            the first reading `dat` in the start layout, all writing the A
 *            layout, the last multiplying by the twiddle;
 *   stage 2: one pass per dimension with A_d > 1, the first reading the A
 *            layout (the A->B move), all writing the B layout;
 * alternating between the two halves of each rank's workspace so that the
 * last pass writes workspace[r*length + 0 ..).  The inverse runs the passes
 * in reverse with the conjugate twiddle and ends in `dat`.
 */
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "dmg_internal.h"
#include "fft_params.h"
#include "k1_params.h"
#include "split_fft.h"
#include "block_decomp.h"
#include "interleave_decomp.h"
#include "factor_reverse_decomp.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define MAXPASS (2 * DMG_FFT_MAXDIM)

enum { LAY_START = 0, LAY_A = 1, LAY_B = 2 };
enum { BUF_DAT = 0, BUF_WORK = 1, BUF_SCRATCH = 2 };

typedef struct {
  int ranked;
  int nranks;
  int64_t pitch;
  int32_t *rk[DMG_FFT_MAXDIM];
  int64_t *tab[DMG_FFT_MAXDIM];
  int64_t *rstride; /* [ndim][nranks] */
  /* device copies */
  const int64_t *d_tab[DMG_FFT_MAXDIM];
  const int32_t *d_rk[DMG_FFT_MAXDIM];
  const int64_t *d_rstride;
} fft_layout;

typedef struct {
  struct dmg_fft_pass p;
  int line;                 /* a whole-dimension pass of the lines schedule */
  int in_lay, out_lay;      /* LAY_* */
  int in_buf, out_buf;      /* BUF_* */
  int64_t in_base, out_base;
} pass_rec;

struct dmg_split_impl {
  int dtype; /* DMG_C128 or DMG_C64 */
  int arith; /* DMG_ARITH_FP64, DMG_ARITH_DF (complex128) or DMG_ARITH_FP32 (complex64) */
  int32_t *d_scale; /* device int: largest input exponent (double-float runs) */
  int32_t *d_status; /* device int: 1 when a tensor-core pass gave up waiting for its products */
  int esize; /* bytes per element */
  int ndim;
  int A[DMG_FFT_MAXDIM], B[DMG_FFT_MAXDIM], L[DMG_FFT_MAXDIM];
  int grid_a[DMG_FFT_MAXDIM], grid_b[DMG_FFT_MAXDIM];
  int use_first, use_second;
  int schedule;        /* DMG_SCHEDULE_*: as asked */
  int tile_values;     /* values per pass tile (0: the default for the element size) */
  int radix;           /* DMG_RADIX_*: the passes' radix schedules */
  int lines;           /* the passes built are the lines schedule */
  long long length;    /* per-rank workspace length */
  long long ext;       /* largest extent of A and B */
  long long dat_pitch; /* per-rank pitch of dat */
  Decomp start;        /* borrowed */
  fft_layout lay[3];
  pass_rec fwd[MAXPASS], inv[MAXPASS];
  int nfwd, ninv;
  /* the same passes with the upper-half intermediates in the fixed scratch
   * array (per-rank pitch = ext), for dmg_split_run_noalloc */
  fft_layout lay_s[3];
  pass_rec fwd_s[MAXPASS], inv_s[MAXPASS];
  size_t scratch_bytes;
  void *dev; /* one device allocation for every table */
  int dev_valid;
  int dev_id; /* the CUDA device the tables were uploaded on */
  void *dat, *work;
  int timing;
  void *events;
  int timed_dir, timed_passes, collected;
  char desc[768];
};

/* timing helpers live in the CUDA runtime source */
void *dmg_split_create_events(int count);
void dmg_split_destroy_events(void *ev);
int dmg_split_record_event(void *ev, int idx, void *stream);
int dmg_split_event_elapsed(void *ev, int a, int b, float *ms);

/* ---------------------------------------------------------------- decomposition builders */

Decomp makeInterleavedDecomp(int ndim, MPI_Comm comm, int A[], int B[], int grid[]) {
  DimDecomp axis[DMG_MAXAX];
  if (ndim < 1 || ndim > DMG_MAXAX) return NULL;
  for (int i = 0; i < ndim; ++i) {
    DimDecomp blk = makeBlockDecomp(A[i], grid[i]);
    axis[i] = blk ? makeInterleaveDecomp(blk, B[i]) : NULL;
    freeDimDecomp(blk);
    if (!axis[i]) {
      for (int k = 0; k < i; ++k) freeDimDecomp(axis[k]);
      dmg_error(DMG_ERR_ARG, "makeInterleavedDecomp: bad factors in dim %d", i);
      return NULL;
    }
  }
  return makePackedDecomp(comm, ndim, axis);
}

Decomp makeBlockedDecomp(int ndim, MPI_Comm comm, int A[], int B[], int grid[]) {
  DimDecomp axis[DMG_MAXAX];
  if (ndim < 1 || ndim > DMG_MAXAX) return NULL;
  for (int i = 0; i < ndim; ++i) {
    axis[i] = makeBlockDecompWithFactor(A[i] * B[i], A[i], grid[i]);
    if (!axis[i]) {
      for (int k = 0; k < i; ++k) freeDimDecomp(axis[k]);
      dmg_error(DMG_ERR_ARG, "makeBlockedDecomp: bad factors in dim %d", i);
      return NULL;
    }
  }
  return makePackedDecomp(comm, ndim, axis);
}

unsigned int gcd(unsigned int u, unsigned int v) {
  while (v) {
    unsigned int t = u % v;
    u = v;
    v = t;
  }
  return u;
}

/* ---------------------------------------------------------------- layouts */

static void layout_free(fft_layout *l) {
  for (int d = 0; d < DMG_FFT_MAXDIM; ++d) {
    free(l->rk[d]);
    free(l->tab[d]);
  }
  free(l->rstride);
  memset(l, 0, sizeof(*l));
}

/* Address tables of a decomposition that holds every global coordinate. */
static int layout_build(fft_layout *l, Decomp D, long long pitch, const char *what) {
  memset(l, 0, sizeof(*l));
  int nd = D->ndim;
  l->nranks = D->proc_used;
  l->pitch = pitch;
  for (int d = 0; d < nd; ++d)
    if (D->dims[d]->rank_memory_stride) l->ranked = 1;
  for (int d = 0; d < nd; ++d) {
    AxisDecomp a = D->dims[d];
    DimDecomp dd = a->decomp;
    int L = dd->coord_size;
    l->rk[d] = (int32_t *)malloc((size_t)L * sizeof(int32_t));
    l->tab[d] = (int64_t *)malloc((size_t)L * sizeof(int64_t));
    if (!l->rk[d] || !l->tab[d]) return dmg_error(DMG_ERR_NOMEM, "split plan: out of host memory");
    for (int x = 0; x < L; ++x) {
      int p = dd->rank_offset(dd, x);
      int off = dd->type_offset(dd, x);
      if (p < 0 || p >= dd->proc_size || off < 0 || off > a->pos_max_local[p])
        return dmg_error(DMG_ERR_ARG, "split plan: %s decomposition does not hold coordinate %d of dim %d", what,
                         x, d);
      l->rk[d][x] = a->rank_stride * p;
      l->tab[d][x] = l->ranked ? off : (int64_t)a->rank_stride * p * pitch + (int64_t)a->memory_stride * off;
    }
  }
  if (l->ranked) {
    int P = l->nranks;
    l->rstride = (int64_t *)malloc((size_t)nd * P * sizeof(int64_t));
    if (!l->rstride) return dmg_error(DMG_ERR_NOMEM, "split plan: out of host memory");
    for (int d = 0; d < nd; ++d)
      for (int r = 0; r < P; ++r) l->rstride[(size_t)d * P + r] = dmg_axis_stride(D->dims[d], r);
  }
  return dmg_check_proper_grid(D, what);
}

static int64_t layout_addr_host(const fft_layout *l, int nd, const int *x) {
  int64_t a = 0;
  if (!l->ranked) {
    for (int d = 0; d < nd; ++d) a += l->tab[d][x[d]];
    return a;
  }
  int64_t R = 0;
  for (int d = 0; d < nd; ++d) R += l->rk[d][x[d]];
  a = R * l->pitch;
  for (int d = 0; d < nd; ++d) a += l->tab[d][x[d]] * l->rstride[(size_t)d * l->nranks + R];
  return a;
}

/* Sub-axis s of a pass is y (s even) or z (s odd) of dimension s/2 for the
 * factors A, B the pass uses: the plan's for split passes, A = L, B = 1 for
 * line passes (so that sub-axis 2d is x_d). */
static int sub_len(const int *A, const int *B, int s) { return (s & 1) ? B[s / 2] : A[s / 2]; }

/* |address step| when sub-axis s moves by one from the origin */
static int64_t sub_step(const struct dmg_split_impl *im, const fft_layout *l, const int *A, int s) {
  int x0[DMG_FFT_MAXDIM] = {0, 0, 0}, x1[DMG_FFT_MAXDIM] = {0, 0, 0};
  int d = s / 2;
  x1[d] = (s & 1) ? A[d] : 1;
  if (x1[d] >= im->L[d]) return INT64_MAX / 4;
  int64_t st = layout_addr_host(l, im->ndim, x1) - layout_addr_host(l, im->ndim, x0);
  return st < 0 ? -st : st;
}

/* radices of n: 8s, then 4, 2, 3, 5, then other primes (fours: 4s, then 2,
 * 3, 5, other primes) */
static int factorize(int n, int32_t *fac, int fours) {
  int k = 0;
  while (!fours && n % 8 == 0) {
    fac[k++] = 8;
    n /= 8;
  }
  while (n % 4 == 0) {
    if (k >= DMG_FFT_MAXFAC) return -1;
    fac[k++] = 4;
    n /= 4;
  }
  if (n % 2 == 0) {
    fac[k++] = 2;
    n /= 2;
  }
  while (n % 3 == 0) {
    if (k >= DMG_FFT_MAXFAC) return -1;
    fac[k++] = 3;
    n /= 3;
  }
  while (n % 5 == 0) {
    if (k >= DMG_FFT_MAXFAC) return -1;
    fac[k++] = 5;
    n /= 5;
  }
  for (int f = 7; f * f <= n; f += 2)
    while (n % f == 0) {
      if (k >= DMG_FFT_MAXFAC) return -1;
      fac[k++] = f;
      n /= f;
    }
  if (n > 1) {
    if (k >= DMG_FFT_MAXFAC) return -1;
    fac[k++] = n;
  }
  return k;
}

static void order_by_step(const int64_t *step, int32_t *order) {
  int idx[3] = {0, 1, 2};
  for (int i = 0; i < 3; ++i)
    for (int j = i + 1; j < 3; ++j)
      if (step[idx[j]] < step[idx[i]]) {
        int t = idx[i];
        idx[i] = idx[j];
        idx[j] = t;
      }
  for (int i = 0; i < 3; ++i) order[i] = idx[i];
}

/* Geometry of a pass along sub-axis t (of the factors A, B) from layout li
 * to lo. */
/* whether dimension d's table of a separable layout is the sum of a part
 * along y and a part along z (x = y + A z, x < L), in its rank part and its
 * offset part each (so for every rank pitch: the scratch copies of the
 * layouts differ in pitch only) */
static int pair_separable(const fft_layout *l, int d, int A, int L) {
  if (l->ranked || A < 1 || L % A) return 0;
  const int64_t *t = l->tab[d];
  const int32_t *r = l->rk[d];
  for (int x = 0; x < L; ++x) {
    const int y = x % A, az = x - x % A;
    if (t[x] - t[y] - t[az] + t[0] != 0 || (int64_t)r[x] - r[y] - r[az] + r[0] != 0) return 0;
  }
  return 1;
}

static int pass_geometry(const struct dmg_split_impl *im, struct dmg_fft_pass *p, int t, const fft_layout *li,
                         const fft_layout *lo, const int *A, const int *B) {
  memset(p, 0, sizeof(*p));
  p->ndim = im->ndim;
  for (int d = 0; d < DMG_FFT_MAXDIM; ++d) {
    p->A[d] = d < im->ndim ? A[d] : 1;
    p->B[d] = d < im->ndim ? B[d] : 1;
    p->L[d] = d < im->ndim ? im->L[d] : 1;
  }
  p->t = t;
  p->n = sub_len(A, B, t);
  if (p->n > 4096) return dmg_error(DMG_ERR_UNSUPPORTED, "FFT factor %d exceeds 4096", p->n);
  p->nfac = factorize(p->n, p->fac, im->radix == DMG_RADIX_PLAN4);
  p->radix_runtime = im->radix != DMG_RADIX_FIXED;
  if (p->nfac < 0) return dmg_error(DMG_ERR_UNSUPPORTED, "FFT length %d has too many prime factors", p->n);
  /* vector sub-axes: the most contiguous in either layout */
  int64_t best[2] = {INT64_MAX, INT64_MAX};
  int pick[2] = {-1, -1};
  for (int s = 0; s < 2 * im->ndim; ++s) {
    if (s == t || sub_len(A, B, s) <= 1) continue;
    int64_t a = sub_step(im, li, A, s), b = sub_step(im, lo, A, s);
    int64_t sc = a < b ? a : b;
    if (sc < best[0]) {
      best[1] = best[0];
      pick[1] = pick[0];
      best[0] = sc;
      pick[0] = s;
    } else if (sc < best[1]) {
      best[1] = sc;
      pick[1] = s;
    }
  }
  p->v1 = pick[0];
  p->v2 = pick[1];
  p->nv1 = p->v1 >= 0 ? sub_len(A, B, p->v1) : 1;
  p->nv2 = p->v2 >= 0 ? sub_len(A, B, p->v2) : 1;
  /* tile values: the plan's choice; more than the two-block kernels hold
   * only for the wide kernels' case (FP32 or double-float, power-of-two
   * length from 256 to 2048, compile-time radix schedule, not the
   * tensor-core 1024-point stage, whose products take four lines) */
  int target = im->tile_values > 0 ? im->tile_values : DMG_FFT_TILE_TARGET(im->esize);
  /* native FP64 passes run in smaller blocks with tiles of at most
   * DMG_FFT_TILE_TARGET_FP64 values */
  if (im->arith == DMG_ARITH_FP64 && (im->tile_values == 0 || target > DMG_FFT_TILE_TARGET_FP64))
    target = DMG_FFT_TILE_TARGET_FP64;
  /* (the wide kernels' shared memory holds their tiles for lines of 256
   * points or more; shorter lines pad and tabulate too much per tile) */
  const int pow2n = p->n >= 256 && p->n <= 2048 && (p->n & (p->n - 1)) == 0;
  /* by default, FP32 passes whose lines are strided on the load side (a
   * vector axis lies closer in memory than the transform axis) take the wide
   * tiles: twice the row length there made such passes about 6 % faster at
   * 1024^3, while passes along contiguous lines ran slower in the wide kernel */
  if (im->tile_values == 0 && im->esize == 8 && pow2n && p->v1 >= 0 &&
      sub_step(im, li, A, t) > sub_step(im, li, A, p->v1))
    target = DMG_FFT_WIDE_TILE(im->esize);
  if (target > DMG_FFT_TILE_TARGET(im->esize) &&
      (im->arith == DMG_ARITH_FP64 || !pow2n || im->radix != DMG_RADIX_FIXED ||
       (im->arith == DMG_ARITH_TC16 && p->n == 1024)))
    target = DMG_FFT_TILE_TARGET(im->esize);
  int room = target / p->n;
  if (room < 1) room = 1;
  p->M1 = p->nv1 < room ? p->nv1 : room;
  room /= p->M1;
  if (room < 1) room = 1;
  p->M2 = p->nv2 < room ? p->nv2 : room;
  p->wide = (int64_t)p->M1 * p->M2 * p->n > DMG_FFT_TILE_TARGET(im->esize);
  p->nt1 = (p->nv1 + p->M1 - 1) / p->M1;
  p->nt2 = (p->nv2 + p->M2 - 1) / p->M2;
  p->nbatch = 0;
  p->ntiles = (int64_t)p->nt1 * p->nt2;
  for (int s = 2 * im->ndim - 1; s >= 0; --s) {
    if (s == t || s == p->v1 || s == p->v2 || sub_len(A, B, s) <= 1) continue;
    p->bsub[p->nbatch] = s;
    p->blen[p->nbatch] = sub_len(A, B, s);
    p->ntiles *= p->blen[p->nbatch];
    p->nbatch++;
  }
  int64_t si[3], so[3];
  si[0] = sub_step(im, li, A, t);
  so[0] = sub_step(im, lo, A, t);
  si[1] = p->v1 >= 0 ? sub_step(im, li, A, p->v1) : INT64_MAX - 1;
  so[1] = p->v1 >= 0 ? sub_step(im, lo, A, p->v1) : INT64_MAX - 1;
  si[2] = p->v2 >= 0 ? sub_step(im, li, A, p->v2) : INT64_MAX;
  so[2] = p->v2 >= 0 ? sub_step(im, lo, A, p->v2) : INT64_MAX;
  order_by_step(si, p->load_order);
  order_by_step(so, p->store_order);
  const int axes[3] = {t, p->v1, p->v2};
  for (int k = 0; k < 3; ++k) {
    p->kdim[k] = axes[k] >= 0 ? axes[k] / 2 : -1;
    p->kisz[k] = axes[k] >= 0 ? (axes[k] & 1) : 0;
  }
  for (int i = 0; i < 3; ++i) {
    p->load_pos[p->load_order[i]] = i;
    p->store_pos[p->store_order[i]] = i;
  }
  /* a side is separable over the tile when its layout is and no two tile
   * axes share a dimension */
  int distinct = (p->kdim[1] < 0 || p->kdim[1] != p->kdim[0]) && (p->kdim[2] < 0 || p->kdim[2] != p->kdim[0]) &&
                 (p->kdim[2] < 0 || p->kdim[2] != p->kdim[1]);
  p->sep_in = distinct && !li->ranked;
  p->sep_out = distinct && !lo->ranked;
  /* exactly two tile axes in one dimension (the third, if any, elsewhere) */
  p->semi_a = p->semi_b = -1;
  for (int a = 0; a < 3 && p->semi_a < 0; ++a)
    for (int b = a + 1; b < 3; ++b)
      if (p->kdim[a] >= 0 && p->kdim[a] == p->kdim[b]) {
        const int c = 3 - a - b;
        if (p->kdim[c] < 0 || p->kdim[c] != p->kdim[a]) {
          p->semi_a = a;
          p->semi_b = b;
        }
        break;
      }
  p->semi_in = !distinct && p->semi_a >= 0 && !li->ranked;
  p->semi_out = !distinct && p->semi_a >= 0 && !lo->ranked;
  /* the shared dimension's table is the sum of a part along each of its
   * sub-axes (interleaved layouts, blocks holding whole multiples of A): the
   * side walks as a separable one */
  if (p->semi_a >= 0) {
    const int d = p->kdim[p->semi_a];
    if (p->semi_in && pair_separable(li, d, A[d], im->L[d])) {
      p->semi_in = 0;
      p->sep_in = p->pair_in = 1;
    }
    if (p->semi_out && pair_separable(lo, d, A[d], im->L[d])) {
      p->semi_out = 0;
      p->sep_out = p->pair_out = 1;
    }
  }
  return DMG_OK;
}

/* ---------------------------------------------------------------- twiddles and roots */

/* exp(-2 pi i m / L) with the quarter turns exact (reference split_fft.c:376-393) */
static void twiddle_value(long long m, int L, double *re, double *im) {
  double angle = -(2.0 * M_PI) * ((double)m / (double)L);
  double c = cos(angle), s = sin(angle);
  long long rem = m % L;
  if (rem == 0) {
    c = 1.0;
    s = 0.0;
  } else if (4 * rem == L) {
    c = 0.0;
    s = -1.0;
  } else if (2 * rem == L) {
    c = -1.0;
    s = 0.0;
  } else if (4 * rem == 3 * (long long)L) {
    c = -0.0;
    s = 1.0;
  }
  *re = c;
  *im = s;
}

/* ---------------------------------------------------------------- device state */

static void impl_free_device(struct dmg_split_impl *im) {
  if (im->dev) dmg_dev_free(im->dev);
  im->dev = NULL;
  im->dev_valid = 0;
}

static void impl_free(struct dmg_split_impl *im) {
  if (!im) return;
  impl_free_device(im);
  if (im->events) dmg_split_destroy_events(im->events);
  for (int k = 0; k < 3; ++k) {
    layout_free(&im->lay[k]);
    layout_free(&im->lay_s[k]);
  }
  free(im);
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

/* whether a separable side's transform-axis entries qualify for the
 * kernel's int32 shared-memory copy (see dmg_fft_pass.t0_rel_in) */
static int t0_rel32(const fft_layout *l, const struct dmg_fft_pass *p) {
  if (l->ranked) return 0;
  const int d0 = p->kdim[0];
  /* (a vector axis in the same dimension moves the table's start per tile) */
  if (p->kdim[1] == d0 || p->kdim[2] == d0) return 0;
  for (int b = 0; b < p->nbatch; ++b)
    if ((p->bsub[b] >> 1) == d0) return 0;
  const int mult0 = p->kisz[0] ? p->A[d0] : 1;
  const int64_t *t = l->tab[d0];
  for (int i = 0; i < p->n; ++i) {
    const int64_t v = t[(int64_t)i * mult0] - t[0];
    if (v < INT32_MIN || v > INT32_MAX) return 0;
  }
  return 1;
}

static void fill_side(struct dmg_fft_layout *fl, const fft_layout *hl, int nd, int64_t base) {
  memset(fl, 0, sizeof(*fl));
  for (int d = 0; d < nd; ++d) {
    fl->tab[d] = hl->d_tab[d];
    fl->rk[d] = hl->d_rk[d];
  }
  fl->rstride = hl->d_rstride;
  fl->pitch = hl->pitch;
  fl->nranks = hl->nranks;
  fl->ranked = hl->ranked;
  fl->base = base;
}

size_t dmg_noalloc_scratch_bytes(void);
int dmg_noalloc_scratch(void **ptr);
int dmg_noalloc_scratch_reserve(void);

/* Upload layout, root and twiddle tables; point every pass at them. */
static int impl_upload(struct dmg_split_impl *im) {
  impl_free_device(im);
  int dev_id = 0;
  int st0 = dmg_rt_get_device(&dev_id);
  if (st0 != DMG_OK) return st0;
  int nd = im->ndim;
  size_t cs = im->dtype == DMG_C128 ? 16 : 8;
  size_t bytes = 0;
  fft_layout *all[6] = {&im->lay[0], &im->lay[1], &im->lay[2], &im->lay_s[0], &im->lay_s[1], &im->lay_s[2]};
  for (int k = 0; k < 6; ++k) {
    if (!all[k]->tab[0]) continue;
    for (int d = 0; d < nd; ++d) bytes += align256((size_t)im->L[d] * 8) + align256((size_t)im->L[d] * 4);
    if (all[k]->ranked) bytes += align256((size_t)nd * all[k]->nranks * 8);
  }
  for (int k = 0; k < im->nfwd; ++k) bytes += align256((size_t)im->fwd[k].p.n * cs);
  for (int d = 0; d < nd; ++d) bytes += 2 * align256((size_t)im->L[d] * cs);
  bytes += 256; /* scale exponent */
  char *host = (char *)calloc(1, bytes + 256);
  if (!host) return dmg_error(DMG_ERR_NOMEM, "split plan: out of host memory for the device tables");
  void *dev = NULL;
  int st = dmg_dev_alloc(&dev, bytes + 256);
  if (st != DMG_OK) {
    free(host);
    return st;
  }
  size_t pos = 0;
  for (int k = 0; k < 6; ++k) {
    fft_layout *l = all[k];
    if (!l->tab[0]) continue;
    for (int d = 0; d < nd; ++d) {
      memcpy(host + pos, l->tab[d], (size_t)im->L[d] * 8);
      l->d_tab[d] = (const int64_t *)((char *)dev + pos);
      pos += align256((size_t)im->L[d] * 8);
      memcpy(host + pos, l->rk[d], (size_t)im->L[d] * 4);
      l->d_rk[d] = (const int32_t *)((char *)dev + pos);
      pos += align256((size_t)im->L[d] * 4);
    }
    if (l->ranked) {
      memcpy(host + pos, l->rstride, (size_t)nd * l->nranks * 8);
      l->d_rstride = (const int64_t *)((char *)dev + pos);
      pos += align256((size_t)nd * l->nranks * 8);
    }
  }
  const void *roots_dev[MAXPASS];
  for (int k = 0; k < im->nfwd; ++k) {
    int n = im->fwd[k].p.n;
    for (int i = 0; i < n; ++i) {
      /* exp(-2 pi i k / n), evaluated in long double and rounded once */
      long double a = -2.0L * 3.141592653589793238462643383279502884L * (long double)i / (long double)n;
      if (im->arith == DMG_ARITH_DF) {
        /* double-float: each component as hi + lo floats */
        long double c = cosl(a), sn = sinl(a);
        float ch = (float)c, sh = (float)sn;
        /* (re.hi, im.hi, re.lo, im.lo): the kernels' paired layout */
        float *f = (float *)(host + pos) + 4 * i;
        f[0] = ch;
        f[1] = sh;
        f[2] = (float)(c - (long double)ch);
        f[3] = (float)(sn - (long double)sh);
      } else if (cs == 16) {
        ((double *)(host + pos))[2 * i] = (double)cosl(a);
        ((double *)(host + pos))[2 * i + 1] = (double)sinl(a);
      } else {
        ((float *)(host + pos))[2 * i] = (float)cosl(a);
        ((float *)(host + pos))[2 * i + 1] = (float)sinl(a);
      }
    }
    roots_dev[k] = (char *)dev + pos;
    pos += align256((size_t)n * cs);
  }
  /* split twiddles exp(-2 pi i y k / L) for y < A, k < B, in two orders:
   * k-major (entry k A + y) and y-major (entry y B + k) */
  const void *twk_dev[DMG_FFT_MAXDIM] = {NULL, NULL, NULL}, *twy_dev[DMG_FFT_MAXDIM] = {NULL, NULL, NULL};
  for (int d = 0; d < nd; ++d) {
    const int A = im->A[d], B = im->B[d];
    for (int order = 0; order < 2; ++order) {
      for (int y = 0; y < A; ++y) {
        for (int k = 0; k < B; ++k) {
          const int e = order == 0 ? k * A + y : y * B + k;
          double re, iv;
          twiddle_value((long long)y * k, im->L[d], &re, &iv);
          if (im->arith == DMG_ARITH_DF) {
            float *f = (float *)(host + pos) + 4 * e;
            f[0] = (float)re;
            f[1] = (float)iv;
            f[2] = (float)(re - (double)f[0]);
            f[3] = (float)(iv - (double)f[1]);
          } else if (cs == 16) {
            ((double *)(host + pos))[2 * e] = re;
            ((double *)(host + pos))[2 * e + 1] = iv;
          } else {
            ((float *)(host + pos))[2 * e] = (float)re;
            ((float *)(host + pos))[2 * e + 1] = (float)iv;
          }
        }
      }
      if (order == 0) twk_dev[d] = (char *)dev + pos;
      else twy_dev[d] = (char *)dev + pos;
      pos += align256((size_t)im->L[d] * cs);
    }
  }
  im->d_scale = (int32_t *)((char *)dev + pos);
  im->d_status = im->d_scale + 1; /* zero from the upload */
  pos += 256;
  st = dmg_dev_upload(dev, host, pos);
  free(host);
  if (st != DMG_OK) {
    dmg_dev_free(dev);
    return st;
  }
  im->dev = dev;
  im->dev_valid = 1;
  im->dev_id = dev_id;
  for (int dir = 0; dir < 2; ++dir) {
    pass_rec *list = dir == 0 ? im->fwd : im->inv;
    int cnt = dir == 0 ? im->nfwd : im->ninv;
    for (int k = 0; k < cnt; ++k) {
      int fk = dir == 0 ? k : im->nfwd - 1 - k; /* the inverse mirrors the forward list */
      list[k].p.roots = roots_dev[fk];
      for (int d = 0; d < DMG_FFT_MAXDIM; ++d) {
        list[k].p.twk[d] = twk_dev[d];
        list[k].p.twy[d] = twy_dev[d];
      }
      /* double-float runs keep float pairs between passes: only the first
       * pass reads complex128 and only the last writes it */
      list[k].p.in_fp64 = im->arith == DMG_ARITH_DF && k == 0;
      list[k].p.out_fp64 = im->arith == DMG_ARITH_DF && k == cnt - 1;
      list[k].p.scale_exp = im->d_scale;
      list[k].p.status = im->d_status;
      fill_side(&list[k].p.in, &im->lay[list[k].in_lay], nd, list[k].in_base);
      fill_side(&list[k].p.out, &im->lay[list[k].out_lay], nd, list[k].out_base);
      list[k].p.t0_rel_in = list[k].p.sep_in && t0_rel32(&im->lay[list[k].in_lay], &list[k].p);
      list[k].p.t0_rel_out = list[k].p.sep_out && t0_rel32(&im->lay[list[k].out_lay], &list[k].p);
      /* scratch variant: an upper-half side moves to the fixed array */
      pass_rec *sr = dir == 0 ? &im->fwd_s[k] : &im->inv_s[k];
      *sr = list[k];
      if (sr->in_buf == BUF_WORK && sr->in_base != 0) {
        sr->in_buf = BUF_SCRATCH;
        sr->in_base = 0;
        fill_side(&sr->p.in, &im->lay_s[sr->in_lay], nd, 0);
      }
      if (sr->out_buf == BUF_WORK && sr->out_base != 0) {
        sr->out_buf = BUF_SCRATCH;
        sr->out_base = 0;
        fill_side(&sr->p.out, &im->lay_s[sr->out_lay], nd, 0);
      }
    }
  }
  /* a plan small enough for dmg_split_run_noalloc: make the module that
   * holds the fixed scratch array resident on this device now (modules load
   * lazily, and loading one reserves its __device__ arrays), so that the
   * no-allocation call finds the array in place instead of reserving it
   * itself; if that fails here, that call reports the error */
  if (im->scratch_bytes <= dmg_noalloc_scratch_bytes()) dmg_noalloc_scratch_reserve();
  return DMG_OK;
}

/* Forward and inverse pass lists of the split schedule. */
/* how a pass side is addressed: separable over the tile axes, two axes in
 * one dimension, or per value */
static const char *side_kind(int sep, int semi, int pair) {
  return pair ? "(paired)" : sep ? "" : (semi ? "(shared dim)" : "(per value)");
}

/* A pass's tile axes fastest first in memory, as letters: t the transform
 * axis, a and b the first and second vector axes. */
static void axis_letters(const int32_t *order, char *out) {
  for (int i = 0; i < 3; ++i) out[i] = order[i] == 0 ? 't' : (order[i] == 1 ? 'a' : 'b');
  out[3] = 0;
}

static int build_passes_split(struct dmg_split_impl *im) {
  int nd = im->ndim;
  int subs[MAXPASS], stage[MAXPASS];
  int K = 0;
  if (!im->use_second)
    for (int d = nd - 1; d >= 0; --d)
      if (im->B[d] > 1) {
        subs[K] = 2 * d + 1;
        stage[K++] = 1;
      }
  int n1 = K;
  if (!im->use_first)
    for (int d = nd - 1; d >= 0; --d)
      if (im->A[d] > 1) {
        subs[K] = 2 * d;
        stage[K++] = 2;
      }
  im->nfwd = im->ninv = K;
  const int64_t upper = im->ext;
  int final_lay = im->use_first ? LAY_A : LAY_B;
  for (int k = 0; k < K; ++k) {
    pass_rec *f = &im->fwd[k];
    /* forward: pass k reads the previous output (pass 0 reads dat) and
     * writes the upper or lower half so that pass K-1 writes the lower one */
    int out_lay = stage[k] == 1 ? LAY_A : LAY_B;
    if (k == K - 1) out_lay = final_lay;
    int in_lay = k == 0 ? LAY_START : (stage[k - 1] == 1 ? LAY_A : LAY_B);
    f->in_lay = in_lay;
    f->out_lay = out_lay;
    f->in_buf = k == 0 ? BUF_DAT : BUF_WORK;
    f->out_buf = BUF_WORK;
    f->out_base = ((K - 1 - k) % 2 == 0) ? 0 : upper;
    f->in_base = k == 0 ? 0 : im->fwd[k - 1].out_base;
    int st = pass_geometry(im, &f->p, subs[k], &im->lay[in_lay], &im->lay[out_lay], im->A, im->B);
    if (st != DMG_OK) return st;
    f->line = 0;
    f->p.sign = -1;
    /* each stage-1 pass applies its own dimension's factor exp(-2 pi i y_d k1_d / L_d)
     * after its transform; the factor is constant along the other dimensions'
     * lines, so it commutes with the remaining stage-1 passes */
    f->p.twiddle = (stage[k] == 1 && K > n1 && im->A[subs[k] / 2] > 1) ? 1 : 0;
  }
  for (int k = 0; k < K; ++k) {
    /* inverse pass k undoes forward pass K-1-k: it reads what that pass
     * wrote and writes what it read, except that the half is chosen so
     * that no pass reads and writes the same half */
    const pass_rec *f = &im->fwd[K - 1 - k];
    pass_rec *b = &im->inv[k];
    b->in_lay = f->out_lay;
    b->out_lay = f->in_lay;
    b->in_buf = BUF_WORK;
    b->out_buf = k == K - 1 ? BUF_DAT : BUF_WORK;
    b->in_base = k == 0 ? 0 : im->inv[k - 1].out_base;
    b->out_base = k == K - 1 ? 0 : (b->in_base == 0 ? upper : 0);
    int st = pass_geometry(im, &b->p, f->p.t, &im->lay[b->in_lay], &im->lay[b->out_lay], im->A, im->B);
    if (st != DMG_OK) return st;
    b->line = 0;
    b->p.sign = +1;
    b->p.twiddle = f->p.twiddle ? 2 : 0;
  }
  im->lines = 0;
  int pos = snprintf(im->desc, sizeof(im->desc), "A=[%d,%d,%d] B=[%d,%d,%d] split passes=%d:", im->A[0],
                     nd > 1 ? im->A[1] : 1, nd > 2 ? im->A[2] : 1, im->B[0], nd > 1 ? im->B[1] : 1,
                     nd > 2 ? im->B[2] : 1, K);
  for (int k = 0; k < K && pos < (int)sizeof(im->desc) - 64; ++k) {
    const struct dmg_fft_pass *p = &im->fwd[k].p;
    char lo[4], so[4];
    axis_letters(p->load_order, lo);
    axis_letters(p->store_order, so);
    pos += snprintf(im->desc + pos, sizeof(im->desc) - pos,
                    " [t=%d n=%d v1=%d x%d v2=%d x%d tiles=%lld%s in=%s%s out=%s%s]", p->t, p->n, p->v1, p->M1, p->v2,
                    p->M2, (long long)p->ntiles, p->twiddle ? " tw" : "", lo, side_kind(p->sep_in, p->semi_in, p->pair_in), so,
                    side_kind(p->sep_out, p->semi_out, p->pair_out));
  }
  return DMG_OK;
}

/* Longest dimension the lines schedule takes by default: a tile of
 * DMG_FFT_TILE_TARGET values then still holds 2 lines side by side.  (At
 * 1024^3 complex128, lines with 2-line tiles take half the time of the
 * split schedule's 6 passes.) */
static int line_max(const struct dmg_split_impl *im) { return DMG_FFT_TILE_TARGET(im->esize) / 2; }

static int lines_possible(const struct dmg_split_impl *im) {
  for (int d = 0; d < im->ndim; ++d)
    if (im->L[d] > DMG_FFT_TILE_TARGET(im->esize)) return 0;
  return 1;
}

/* Forward and inverse pass lists of the lines schedule. */
static int build_passes_line(struct dmg_split_impl *im) {
  int nd = im->ndim;
  int dims[DMG_FFT_MAXDIM], K = 0;
  for (int d = nd - 1; d >= 0; --d)
    if (im->L[d] > 1) dims[K++] = d;
  int LA[DMG_FFT_MAXDIM], LB[DMG_FFT_MAXDIM];
  for (int d = 0; d < DMG_FFT_MAXDIM; ++d) {
    LA[d] = d < nd ? im->L[d] : 1;
    LB[d] = 1;
  }
  im->nfwd = im->ninv = K;
  const int64_t upper = im->ext;
  const int fin = im->use_first ? LAY_A : LAY_B;
  for (int k = 0; k < K; ++k) {
    pass_rec *f = &im->fwd[k];
    const int d = dims[k];
    f->line = 1;
    f->in_lay = k == 0 ? LAY_START : fin;
    f->out_lay = fin;
    f->in_buf = k == 0 ? BUF_DAT : BUF_WORK;
    f->out_buf = BUF_WORK;
    f->out_base = ((K - 1 - k) % 2 == 0) ? 0 : upper;
    f->in_base = k == 0 ? 0 : im->fwd[k - 1].out_base;
    int st = pass_geometry(im, &f->p, 2 * d, &im->lay[f->in_lay], &im->lay[f->out_lay], LA, LB);
    if (st != DMG_OK) return st;
    f->p.sign = -1;
    if (im->A[d] > 1 && im->B[d] > 1) {
      f->p.perm_out = 1;
      f->p.perm_a = im->A[d];
      f->p.perm_b = im->B[d];
    }
  }
  for (int k = 0; k < K; ++k) {
    const pass_rec *f = &im->fwd[K - 1 - k];
    pass_rec *b = &im->inv[k];
    b->line = 1;
    b->in_lay = f->out_lay;
    b->out_lay = f->in_lay;
    b->in_buf = BUF_WORK;
    b->out_buf = k == K - 1 ? BUF_DAT : BUF_WORK;
    b->in_base = k == 0 ? 0 : im->inv[k - 1].out_base;
    b->out_base = k == K - 1 ? 0 : (b->in_base == 0 ? upper : 0);
    int st = pass_geometry(im, &b->p, f->p.t, &im->lay[b->in_lay], &im->lay[b->out_lay], LA, LB);
    if (st != DMG_OK) return st;
    b->p.sign = +1;
    b->p.perm_in = f->p.perm_out;
    b->p.perm_a = f->p.perm_a;
    b->p.perm_b = f->p.perm_b;
  }
  im->lines = 1;
  int pos = snprintf(im->desc, sizeof(im->desc), "A=[%d,%d,%d] B=[%d,%d,%d] lines passes=%d:", im->A[0],
                     nd > 1 ? im->A[1] : 1, nd > 2 ? im->A[2] : 1, im->B[0], nd > 1 ? im->B[1] : 1,
                     nd > 2 ? im->B[2] : 1, K);
  for (int k = 0; k < K && pos < (int)sizeof(im->desc) - 64; ++k) {
    const struct dmg_fft_pass *p = &im->fwd[k].p;
    char lo[4], so[4];
    axis_letters(p->load_order, lo);
    axis_letters(p->store_order, so);
    pos += snprintf(im->desc + pos, sizeof(im->desc) - pos,
                    " [d=%d n=%d v1=%d x%d v2=%d x%d tiles=%lld%s in=%s%s out=%s%s]", p->t / 2, p->n,
                    p->v1 >= 0 ? p->v1 / 2 : -1, p->M1, p->v2 >= 0 ? p->v2 / 2 : -1, p->M2, (long long)p->ntiles,
                    p->perm_out ? " slots" : "", lo, side_kind(p->sep_in, p->semi_in, p->pair_in), so,
                    side_kind(p->sep_out, p->semi_out, p->pair_out));
  }
  return DMG_OK;
}

/* Pass lists for the schedule asked for (auto: lines when every dimension
 * is at most line_max long). */
static int build_passes(struct dmg_split_impl *im) {
  int use_lines;
  if (im->schedule == DMG_SCHEDULE_LINES) {
    if (!lines_possible(im))
      return dmg_error(DMG_ERR_UNSUPPORTED, "lines schedule: a dimension is longer than %d",
                       DMG_FFT_TILE_TARGET(im->esize));
    use_lines = 1;
  } else if (im->schedule == DMG_SCHEDULE_SPLIT) {
    use_lines = 0;
  } else {
    use_lines = 1;
    for (int d = 0; d < im->ndim; ++d)
      if (im->L[d] > line_max(im)) use_lines = 0;
  }
  memset(im->fwd, 0, sizeof(im->fwd));
  memset(im->inv, 0, sizeof(im->inv));
  return use_lines ? build_passes_line(im) : build_passes_split(im);
}

/* kernel dtype of a plan's arithmetic */
static int arith_dtype(const struct dmg_split_impl *im) {
  return im->arith == DMG_ARITH_FP64 ? 0 : im->arith == DMG_ARITH_FP32 ? 1 : im->arith == DMG_ARITH_DF ? 2 : 3;
}

/* largest exponent of the run's complex128 input, for the double-float scaling */
static int launch_maxexp(struct dmg_split_impl *im, const pass_rec *first, const void *src, void *stream) {
  int32_t L[DMG_FFT_MAXDIM], A[DMG_FFT_MAXDIM];
  for (int d = 0; d < DMG_FFT_MAXDIM; ++d) {
    L[d] = im->L[d];
    A[d] = im->A[d];
  }
  return dmg_fft_maxexp_launch(&first->p.in, im->ndim, A, L, src, im->d_scale, stream);
}

/* ---------------------------------------------------------------- public API */

SplitPlan dmg_build_plan_typed(int flags, int use_first, int use_second, Decomp start, int ndim, int A[], int B[],
                            int L[], int grid_a[], int grid_b[], void *dat, long long length, void *workspace,
                            int dtype) {
  if (!start || ndim != start->ndim) {
    dmg_error(DMG_ERR_ARG, "buildParallelPlan: ndim does not match the start decomposition");
    return NULL;
  }
  if ((flags & FORCE_USE_FIRST) && !use_first) return NULL;
  if (ndim > DMG_FFT_MAXDIM) {
    dmg_error(DMG_ERR_UNSUPPORTED, "split FFT: %d dimensions (at most %d)", ndim, DMG_FFT_MAXDIM);
    return NULL;
  }
  for (int i = 0; i < ndim; ++i) {
    if (A[i] < 1 || B[i] < 1 || A[i] * B[i] != L[i] || L[i] != start->dims[i]->decomp->coord_size) {
      raise_error(start->comm, "Invalid factor");
      return NULL;
    }
  }
  SplitPlan plan = (SplitPlan)calloc(1, sizeof(struct split_fft_plan));
  struct dmg_split_impl *im = (struct dmg_split_impl *)calloc(1, sizeof(*im));
  if (!plan || !im) {
    free(plan);
    free(im);
    dmg_error(DMG_ERR_NOMEM, "split plan: out of memory");
    return NULL;
  }
  plan->impl = im;
  plan->comm = start->comm;
  plan->src = (fftw_complex *)dat;
  plan->work = (fftw_complex *)workspace;
  im->dtype = dtype;
  im->arith = dtype == DMG_C128 ? DMG_ARITH_DF : DMG_ARITH_FP32;
  im->esize = dtype == DMG_C128 ? 16 : 8;
  im->ndim = ndim;
  im->use_first = use_first;
  im->use_second = use_second;
  im->length = length;
  im->start = start;
  im->dat = dat;
  im->work = workspace;
  for (int i = 0; i < DMG_FFT_MAXDIM; ++i) {
    im->A[i] = i < ndim ? A[i] : 1;
    im->B[i] = i < ndim ? B[i] : 1;
    im->L[i] = i < ndim ? L[i] : 1;
    im->grid_a[i] = i < ndim ? grid_a[i] : 1;
    im->grid_b[i] = i < ndim ? grid_b[i] : 1;
  }
  plan->A = makeInterleavedDecomp(ndim, start->comm, A, B, grid_a);
  if (!plan->A) goto fail;
  long long ext = extent64(plan->A);
  if (!use_first) {
    plan->B = makeBlockedDecomp(ndim, start->comm, A, B, grid_b);
    if (!plan->B) goto fail;
    long long eb = extent64(plan->B);
    if (eb > ext) ext = eb;
  }
  if (2 * ext > length) {
    dmg_error(DMG_ERR_WORKSPACE, "Not enough workspace need=%lld have=%lld", 2 * ext, length);
    goto fail;
  }
  im->ext = ext;
  plan->extent = ext > INT_MAX ? -1 : (int)ext;
  if ((flags & PREFER_LARGE_FFT) && !use_first) {
    /* a common factor in the blocking redundancy of A and B rejects the plan (split_fft.c:309-333) */
    for (int i = 0; i < ndim; ++i) {
      InterleaveDecomp ad = (InterleaveDecomp)plan->A->dims[i]->decomp;
      unsigned a_red = ((BlockDecomp)ad->nested)->blocksize;
      unsigned b_red = ((BlockDecomp)plan->B->dims[i]->decomp)->blocksize / A[i];
      if (gcd(a_red, b_red) > 1) goto fail_quiet;
    }
  }
  int base = im->esize;
  plan->start_to_A = makeReshapePlan(start->comm, base, start, plan->A);
  plan->A_to_start = makeReshapePlan(start->comm, base, plan->A, start);
  if (!plan->start_to_A || !plan->A_to_start) goto fail;
  if (!(use_first || use_second)) {
    plan->A_to_B = makeReshapePlan(start->comm, base, plan->A, plan->B);
    plan->B_to_A = makeReshapePlan(start->comm, base, plan->B, plan->A);
    if (!plan->A_to_B || !plan->B_to_A) goto fail;
  }
  im->dat_pitch = extent64(start);
  if (layout_build(&im->lay[LAY_START], start, im->dat_pitch, "start") != DMG_OK) goto fail;
  if (layout_build(&im->lay[LAY_A], plan->A, length, "A") != DMG_OK) goto fail;
  if (!use_first && layout_build(&im->lay[LAY_B], plan->B, length, "B") != DMG_OK) goto fail;
  if (build_passes(im) != DMG_OK) goto fail;
  /* scratch copies of the intermediate layouts: rank r's region at r * ext */
  if (layout_build(&im->lay_s[LAY_A], plan->A, ext, "A") != DMG_OK) goto fail;
  if (!use_first && layout_build(&im->lay_s[LAY_B], plan->B, ext, "B") != DMG_OK) goto fail;
  {
    int nr = im->lay_s[LAY_A].nranks;
    if (!use_first && im->lay_s[LAY_B].nranks > nr) nr = im->lay_s[LAY_B].nranks;
    im->scratch_bytes = (size_t)nr * (size_t)ext * (size_t)im->esize;
  }
  plan->plan_a = (!use_second && im->nfwd > 0) ? (void *)im : NULL;
  plan->plan_b = NULL;
  for (int i = 0; i < ndim; ++i)
    if (!use_first && A[i] > 1) plan->plan_b = (void *)im;
  plan->plan_b_back = plan->plan_b;
  plan->plan_a_back = plan->plan_a;
  if (!use_first) {
    AxisDecomp flipped[DMG_FFT_MAXDIM];
    for (int i = 0; i < ndim; ++i) flipped[i] = makeFactorReverseAxisDecomp(A[i], B[i], plan->B->dims[i]);
    plan->B_flipped = makeDecomp(ndim, flipped);
  }
  plan->A_factors = (int *)calloc((size_t)ndim, sizeof(int));
  for (int i = 0; i < ndim; ++i) plan->A_factors[i] = A[i];
  plan->times = (double *)calloc(NUM_TIMERS, sizeof(double));
  plan->twiddle = NULL;
  return plan;
fail:
fail_quiet:
  freeSplitPlan(plan);
  return NULL;
}

SplitPlan buildParallelPlan(int flags, int use_first, int use_second, Decomp start, int ndim, int A[], int B[],
                            int L[], int a_grid[], int b_grid[], fftw_complex *dat, int length,
                            fftw_complex workspace[]) {
  return dmg_build_plan_typed(flags, use_first, use_second, start, ndim, A, B, L, a_grid, b_grid, dat, length, workspace,
                    DMG_C128);
}

static SplitPlan propose(int flags, Decomp start, int *initial_factor, void *dat, long long length, void *workspace,
                         int dtype) {
  if (!start) return NULL;
  int nd = start->ndim;
  if (nd > DMG_FFT_MAXDIM) {
    dmg_error(DMG_ERR_UNSUPPORTED, "split FFT: %d dimensions (at most %d)", nd, DMG_FFT_MAXDIM);
    return NULL;
  }
  int A[DMG_FFT_MAXDIM], B[DMG_FFT_MAXDIM], L[DMG_FFT_MAXDIM];
  int use_first = 1, use_second = 1;
  for (int i = 0; i < nd; ++i) {
    B[i] = initial_factor[i];
    L[i] = sizeDimDecomp(start->dims[i]->decomp);
    if (B[i] < 1 || L[i] % B[i] != 0) {
      raise_error(start->comm, "Invalid factor");
      return NULL;
    }
    A[i] = L[i] / B[i];
    use_second = use_second && B[i] == 1;
    use_first = use_first && A[i] == 1;
  }
  if (use_second && (flags & PREFER_STAGE1)) return NULL;
  int *ga = makeProcessorGrid(start->comm, nd, A);
  int *gb = makeProcessorGrid(start->comm, nd, B);
  SplitPlan p = dmg_build_plan_typed(flags, use_first, use_second, start, nd, A, B, L, ga, gb, dat, length, workspace, dtype);
  free(ga);
  free(gb);
  return p;
}

SplitPlan proposeParallelPlan(int flags, Decomp start, int *initial_factor, fftw_complex *dat, int length,
                              fftw_complex workspace[]) {
  return propose(flags, start, initial_factor, dat, length, workspace, DMG_C128);
}

SplitPlan makeParallelPlan(Decomp start, int *initial_factor, fftw_complex *dat, int length, fftw_complex workspace[]) {
  return propose(NO_FLAGS, start, initial_factor, dat, length, workspace, DMG_C128);
}

SplitPlan dmg_makeParallelPlanTyped(Decomp start, int *initial_factor, void *dat, long long length, void *workspace,
                                    int dtype) {
  return propose(NO_FLAGS, start, initial_factor, dat, length, workspace, dtype);
}

/* factor choice of makeSplitPlan (reference split_fft.c:578-607) */
static void split_factors(int slab, Decomp start, int *B) {
  int nd = start->ndim;
  for (int i = 0; i < nd; ++i) {
    int LL = sizeDimDecomp(start->dims[i]->decomp);
    int AA = 1, BB = LL;
    if (slab == 1) {
      if (i == nd - 1) {
        BB = 1;
        AA = LL;
      }
    } else {
      for (int qq = 1; qq < LL; ++qq) {
        if (LL % qq == 0) {
          int pp = LL / qq;
          if (qq > AA && qq <= pp) {
            AA = qq;
            BB = pp;
          }
        }
      }
    }
    B[i] = BB;
  }
}

SplitPlan dmg_makeSplitPlanTyped(int slab, Decomp start, void *dat, long long length, void *workspace, int dtype) {
  if (!start) return NULL;
  if (start->ndim > DMG_FFT_MAXDIM) {
    dmg_error(DMG_ERR_UNSUPPORTED, "split FFT: %d dimensions (at most %d)", start->ndim, DMG_FFT_MAXDIM);
    return NULL;
  }
  int B[DMG_FFT_MAXDIM];
  split_factors(slab, start, B);
  SplitPlan p = dmg_makeParallelPlanTyped(start, B, dat, length, workspace, dtype);
  if (!p && dmg_last_error_code() == DMG_OK) raise_error(start->comm, "Cannot generate plan");
  return p;
}

SplitPlan makeSplitPlan(int slab, Decomp start, fftw_complex *dat, int length, fftw_complex workspace[]) {
  return dmg_makeSplitPlanTyped(slab, start, dat, length, workspace, DMG_C128);
}

Decomp getTransformed(SplitPlan plan) { return plan ? plan->B_flipped : NULL; }

Decomp getTransformedExact(SplitPlan plan) {
  if (!plan || !plan->B) return NULL;
  struct dmg_split_impl *im = plan->impl;
  AxisDecomp ax[DMG_FFT_MAXDIM];
  for (int i = 0; i < im->ndim; ++i) ax[i] = makeFactorReverseAxisDecomp(im->B[i], im->A[i], plan->B->dims[i]);
  return makeDecomp(im->ndim, ax);
}

void freeSplitPlan(SplitPlan plan) {
  if (!plan) return;
  freeReshapePlan(plan->start_to_A);
  freeReshapePlan(plan->A_to_start);
  freeReshapePlan(plan->A_to_B);
  freeReshapePlan(plan->B_to_A);
  if (plan->A) freeDecomp(plan->A);
  if (plan->B) freeDecomp(plan->B);
  if (plan->B_flipped) freeDecomp(plan->B_flipped);
  free(plan->A_factors);
  free(plan->times);
  impl_free(plan->impl);
  free(plan);
}

int dmg_split_set_buffers(SplitPlan plan, void *dat, void *workspace) {
  if (!plan) return dmg_error(DMG_ERR_ARG, "dmg_split_set_buffers: NULL plan");
  plan->impl->dat = dat;
  plan->impl->work = workspace;
  plan->src = (fftw_complex *)dat;
  plan->work = (fftw_complex *)workspace;
  return DMG_OK;
}

int dmg_split_set_dat_pitch(SplitPlan plan, long long pitch) {
  if (!plan) return dmg_error(DMG_ERR_ARG, "dmg_split_set_dat_pitch: NULL plan");
  struct dmg_split_impl *im = plan->impl;
  if (pitch < extent64(im->start)) return dmg_error(DMG_ERR_BOUNDS, "dat pitch %lld below extent", pitch);
  layout_free(&im->lay[LAY_START]);
  im->dat_pitch = pitch;
  int st = layout_build(&im->lay[LAY_START], im->start, pitch, "start");
  if (st != DMG_OK) return st;
  impl_free_device(im);
  return dmg_reshape_set_pitch(plan->start_to_A, pitch, 0) | dmg_reshape_set_pitch(plan->A_to_start, 0, pitch);
}

int dmg_split_set_arith(SplitPlan plan, int arith) {
  if (!plan) return dmg_error(DMG_ERR_ARG, "dmg_split_set_arith: NULL plan");
  struct dmg_split_impl *im = plan->impl;
  if (im->dtype == DMG_C64 ? (arith != DMG_ARITH_FP32 && arith != DMG_ARITH_TC16)
                           : (arith != DMG_ARITH_FP64 && arith != DMG_ARITH_DF))
    return dmg_error(DMG_ERR_ARG, "dmg_split_set_arith: arithmetic %d does not apply to this element type", arith);
  if (arith != im->arith) {
    const int old = im->arith;
    im->arith = arith;
    /* the passes' tiles depend on the arithmetic (wide tiles), and the
     * tables differ between arithmetics */
    int st = build_passes(im);
    if (st != DMG_OK) {
      im->arith = old;
      build_passes(im);
      return st;
    }
    impl_free_device(im);
  }
  return DMG_OK;
}

int dmg_split_get_arith(SplitPlan plan) { return plan ? plan->impl->arith : -1; }

int dmg_split_device_status(SplitPlan plan) {
  if (!plan) return -dmg_error(DMG_ERR_ARG, "dmg_split_device_status: NULL plan");
  struct dmg_split_impl *im = plan->impl;
  if (!im->dev_valid) return 0; /* nothing has run since the tables were (re)made */
  int32_t v = 0;
  int st = dmg_copy_sync(&v, im->d_status, sizeof(v), 1, NULL);
  return st != DMG_OK ? -st : v;
}

long long dmg_split_extent64(SplitPlan plan) { return plan ? plan->impl->ext : -1; }

int dmg_split_set_schedule(SplitPlan plan, int schedule) {
  if (!plan) return dmg_error(DMG_ERR_ARG, "dmg_split_set_schedule: NULL plan");
  if (schedule != DMG_SCHEDULE_AUTO && schedule != DMG_SCHEDULE_LINES && schedule != DMG_SCHEDULE_SPLIT)
    return dmg_error(DMG_ERR_ARG, "dmg_split_set_schedule: schedule %d", schedule);
  struct dmg_split_impl *im = plan->impl;
  int old = im->schedule;
  im->schedule = schedule;
  int st = build_passes(im);
  if (st != DMG_OK) {
    im->schedule = old;
    build_passes(im);
    return st;
  }
  impl_free_device(im); /* passes point into the device tables: upload again */
  return DMG_OK;
}

int dmg_split_get_schedule(SplitPlan plan) { return plan ? (plan->impl->lines ? DMG_SCHEDULE_LINES : DMG_SCHEDULE_SPLIT) : -1; }

/* rebuild the passes after a change of one of the plan's choices; on failure
 * the old value is put back */
static int rebuild_with(struct dmg_split_impl *im, int *field, int value) {
  const int old = *field;
  *field = value;
  int st = build_passes(im);
  if (st != DMG_OK) {
    *field = old;
    build_passes(im);
    return st;
  }
  impl_free_device(im); /* passes point into the device tables: upload again */
  return DMG_OK;
}

int dmg_split_set_tile(SplitPlan plan, int values) {
  if (!plan) return dmg_error(DMG_ERR_ARG, "dmg_split_set_tile: NULL plan");
  struct dmg_split_impl *im = plan->impl;
  const int most = DMG_FFT_WIDE_TILE(im->esize);
  if (values != 0 && (values < 64 || values > most || (values & (values - 1))))
    return dmg_error(DMG_ERR_ARG, "dmg_split_set_tile: %d values per tile (0, or a power of two from 64 to %d)",
                     values, most);
  return rebuild_with(im, &im->tile_values, values);
}

int dmg_split_get_tile(SplitPlan plan) { return plan ? plan->impl->tile_values : -1; }

int dmg_split_set_radix(SplitPlan plan, int radix) {
  if (!plan) return dmg_error(DMG_ERR_ARG, "dmg_split_set_radix: NULL plan");
  if (radix != DMG_RADIX_FIXED && radix != DMG_RADIX_PLAN8 && radix != DMG_RADIX_PLAN4)
    return dmg_error(DMG_ERR_ARG, "dmg_split_set_radix: radix schedule %d", radix);
  return rebuild_with(plan->impl, &plan->impl->radix, radix);
}

int dmg_split_get_radix(SplitPlan plan) { return plan ? plan->impl->radix : -1; }

int dmg_split_launches(SplitPlan plan, int direction) {
  if (!plan) return 0;
  int k = direction == FFTW_FORWARD ? plan->impl->nfwd : plan->impl->ninv;
  if (k > 0 && plan->impl->arith == DMG_ARITH_DF) k += 1; /* the exponent pre-pass */
  return k > 0 ? k : 1;
}

double dmg_split_flops(SplitPlan plan) {
  if (!plan) return 0;
  double n = 1;
  for (int i = 0; i < plan->impl->ndim; ++i) n *= plan->impl->L[i];
  return n > 1 ? 5.0 * n * log2(n) : 0.0;
}

const char *dmg_split_describe(SplitPlan plan) { return plan ? plan->impl->desc : ""; }

int dmg_split_set_timing(SplitPlan plan, int on) {
  if (!plan) return dmg_error(DMG_ERR_ARG, "NULL plan");
  plan->impl->timing = on;
  if (on && !plan->impl->events) plan->impl->events = dmg_split_create_events(MAXPASS + 1);
  return DMG_OK;
}

/* Event k precedes pass k of the last timed run, event K follows the last. */
int dmg_split_pass_times(SplitPlan plan, int direction, float *ms, int max) {
  if (!plan) return dmg_error(DMG_ERR_ARG, "NULL plan");
  struct dmg_split_impl *im = plan->impl;
  if (!im->events || im->timed_dir != direction) return dmg_error(DMG_ERR_ARG, "no timed run in that direction");
  int K = im->timed_passes;
  for (int k = 0; k < K && k < max; ++k) {
    int st = dmg_split_event_elapsed(im->events, k, k + 1, &ms[k]);
    if (st != DMG_OK) return st;
  }
  return K;
}

int dmg_split_collect_times(SplitPlan plan) {
  if (!plan) return dmg_error(DMG_ERR_ARG, "NULL plan");
  struct dmg_split_impl *im = plan->impl;
  if (!im->events || im->timed_passes <= 0 || im->collected) return DMG_OK;
  float ms[MAXPASS];
  int K = dmg_split_pass_times(plan, im->timed_dir, ms, MAXPASS);
  if (K < 0) return K;
  /* stage-1 passes count as FFT_1 (with the fused start->A move and the
   * twiddle), stage-2 passes as FFT_2 (with the fused A->B move); passes of
   * the lines schedule as FFT_1 */
  pass_rec *list = im->timed_dir == FFTW_FORWARD ? im->fwd : im->inv;
  double all = 0;
  for (int k = 0; k < K; ++k) {
    double sec = ms[k] * 1e-3;
    all += sec;
    if (list[k].line || (list[k].p.t & 1)) plan->times[FFT_1] += sec;
    else plan->times[FFT_2] += sec;
  }
  plan->times[ALL] += all;
  im->collected = 1;
  return DMG_OK;
}

int dmg_split_run(SplitPlan plan, int direction, void *stream) {
  if (!plan) return dmg_error(DMG_ERR_ARG, "runSplitPlan: NULL plan");
  struct dmg_split_impl *im = plan->impl;
  if (direction != FFTW_FORWARD && direction != FFTW_BACKWARD)
    return dmg_error(DMG_ERR_ARG, "runSplitPlan: direction %d", direction);
  if (!im->dat || !im->work) return dmg_error(DMG_ERR_ARG, "runSplitPlan: NULL buffer");
  if (!im->dev_valid) {
    int st = impl_upload(im);
    if (st != DMG_OK) return st;
  }
  if (im->nfwd == 0) {
    /* nothing to transform (every length 1): move the data between layouts */
    if (direction == FFTW_FORWARD) return dmg_reshape_run(plan->start_to_A, im->dat, im->work, stream);
    return dmg_reshape_run(plan->A_to_start, im->work, im->dat, stream);
  }
  pass_rec *list = direction == FFTW_FORWARD ? im->fwd : im->inv;
  int cnt = direction == FFTW_FORWARD ? im->nfwd : im->ninv;
  int dt = arith_dtype(im);
  if (im->arith == DMG_ARITH_DF) {
    int st = launch_maxexp(im, &list[0], list[0].in_buf == BUF_DAT ? im->dat : im->work, stream);
    if (st != DMG_OK) return st;
  }
  if (im->timing) {
    if (im->timed_passes > 0 && !im->collected) dmg_split_collect_times(plan);
    im->timed_dir = direction;
    im->timed_passes = cnt;
    im->collected = 0;
  }
  for (int k = 0; k < cnt; ++k) {
    const void *src = list[k].in_buf == BUF_DAT ? im->dat : im->work;
    void *dst = list[k].out_buf == BUF_DAT ? im->dat : im->work;
    if (im->timing) dmg_split_record_event(im->events, k, stream);
    int st = dmg_fft_pass_launch(&list[k].p, dt, src, dst, stream);
    if (st != DMG_OK) return st;
  }
  if (im->timing) dmg_split_record_event(im->events, cnt, stream);
  return DMG_OK;
}

void runSplitPlan(SplitPlan plan, int direction) { dmg_split_run(plan, direction, dmg_current_stream()); }

int dmg_split_run_batch(SplitPlan plan, int direction, void *stream, int count, void *const *dats, void *const *works,
                        int *const *scales) {
  if (!plan) return dmg_error(DMG_ERR_ARG, "dmg_split_run_batch: NULL plan");
  struct dmg_split_impl *im = plan->impl;
  if (direction != FFTW_FORWARD && direction != FFTW_BACKWARD)
    return dmg_error(DMG_ERR_ARG, "dmg_split_run_batch: direction %d", direction);
  if (count < 1 || count > DMG_FFT_MAXBATCH)
    return dmg_error(DMG_ERR_ARG, "dmg_split_run_batch: %d jobs (1 to %d)", count, DMG_FFT_MAXBATCH);
  for (int j = 0; j < count; ++j)
    if (!dats[j] || !works[j] || (im->arith == DMG_ARITH_DF && !scales[j]))
      return dmg_error(DMG_ERR_ARG, "dmg_split_run_batch: NULL buffer for job %d", j);
  if (im->nfwd == 0) return dmg_error(DMG_ERR_UNSUPPORTED, "dmg_split_run_batch: the plan has no transform passes");
  if (!im->dev_valid) {
    int st = impl_upload(im);
    if (st != DMG_OK) return st;
  }
  pass_rec *list = direction == FFTW_FORWARD ? im->fwd : im->inv;
  int cnt = direction == FFTW_FORWARD ? im->nfwd : im->ninv;
  int dt = arith_dtype(im);
  if (im->arith == DMG_ARITH_DF) {
    int32_t L[DMG_FFT_MAXDIM], A[DMG_FFT_MAXDIM];
    for (int d = 0; d < DMG_FFT_MAXDIM; ++d) {
      L[d] = im->L[d];
      A[d] = im->A[d];
    }
    for (int j = 0; j < count; ++j) {
      const void *src = list[0].in_buf == BUF_DAT ? dats[j] : works[j];
      int st = dmg_fft_maxexp_launch(&list[0].p.in, im->ndim, A, L, src, scales[j], stream);
      if (st != DMG_OK) return st;
    }
  }
  struct dmg_fft_batch b;
  memset(&b, 0, sizeof(b));
  b.count = count;
  for (int k = 0; k < cnt; ++k) {
    for (int j = 0; j < count; ++j) {
      b.src[j] = list[k].in_buf == BUF_DAT ? dats[j] : works[j];
      b.dst[j] = list[k].out_buf == BUF_DAT ? dats[j] : works[j];
      b.scale_exp[j] = scales ? scales[j] : NULL;
    }
    int st = dmg_fft_pass_launch_batch(&list[k].p, dt, &b, stream);
    if (st != DMG_OK) return st;
  }
  return DMG_OK;
}

int dmg_split_batch_launches(SplitPlan plan, int direction, int count) {
  if (!plan) return 0;
  int k = direction == FFTW_FORWARD ? plan->impl->nfwd : plan->impl->ninv;
  if (plan->impl->arith == DMG_ARITH_DF) k += 2 * count; /* exponent pre-pass: a memset and a kernel per job */
  return k;
}

/* ---------------------------------------------------------------- grouped run */

_Static_assert(DMG_SPLIT_MAXGROUP == DMG_FFT_MAXGROUP, "a group is one launch per pass");

/* The k-th passes of several plans (any sizes, decompositions and pass
 * counts) in one launch each: plan i's pass k reads what its pass k-1 wrote
 * in the launch before, on the same stream.  Every plan runs its passes with
 * the runtime stages of its radix schedule, so it must have one
 * (DMG_RADIX_PLAN8 or DMG_RADIX_PLAN4); its results are then the bits of
 * dmg_split_run on the same plan.  own_buffers: the plans' dat and workspace
 * are the arrays (else the caller lists them). */
static int group_check(int count, SplitPlan const *plans, int direction, int own_buffers, const char *who) {
  if (direction != FFTW_FORWARD && direction != FFTW_BACKWARD)
    return dmg_error(DMG_ERR_ARG, "%s: direction %d", who, direction);
  if (count < 1 || count > DMG_FFT_MAXGROUP)
    return dmg_error(DMG_ERR_ARG, "%s: %d plans (1 to %d)", who, count, DMG_FFT_MAXGROUP);
  for (int i = 0; i < count; ++i) {
    if (!plans[i]) return dmg_error(DMG_ERR_ARG, "%s: NULL plan %d", who, i);
    const struct dmg_split_impl *im = plans[i]->impl;
    if (own_buffers && (!im->dat || !im->work)) return dmg_error(DMG_ERR_ARG, "%s: NULL buffer in plan %d", who, i);
    if (im->radix == DMG_RADIX_FIXED)
      return dmg_error(DMG_ERR_ARG, "%s: plan %d has the fixed radix schedules; set DMG_RADIX_PLAN8 or "
                                    "DMG_RADIX_PLAN4 on every plan of a group", who, i);
    if (im->nfwd == 0) return dmg_error(DMG_ERR_UNSUPPORTED, "%s: plan %d has no transform passes", who, i);
    if (arith_dtype(im) != arith_dtype(plans[0]->impl))
      return dmg_error(DMG_ERR_ARG, "%s: plan %d's arithmetic differs from plan 0's", who, i);
    for (int j = 0; j < i; ++j)
      if (plans[j] == plans[i]) return dmg_error(DMG_ERR_ARG, "%s: plan %d appears twice", who, i);
  }
  return DMG_OK;
}

/* The run over a checked group: plan i transforms njobs[i] arrays, listed
 * plan by plan in dats / works / scales (njobs NULL: one array per plan, the
 * plan's own dat and workspace, with its own exponent word). */
static int group_run(int count, SplitPlan const *plans, const int *njobs, void *const *dats, void *const *works,
                     int *const *scales, int direction, void *stream) {
  int st = DMG_OK, most = 0;
  int32_t L[DMG_FFT_MAXDIM], A[DMG_FFT_MAXDIM];
  for (int i = 0, at = 0; i < count; ++i) {
    struct dmg_split_impl *im = plans[i]->impl;
    if (!im->dev_valid && (st = impl_upload(im)) != DMG_OK) return st;
    const int cnt = direction == FFTW_FORWARD ? im->nfwd : im->ninv;
    if (cnt > most) most = cnt;
    const int nj = njobs ? njobs[i] : 1;
    if (im->arith == DMG_ARITH_DF) {
      const pass_rec *first = direction == FFTW_FORWARD ? &im->fwd[0] : &im->inv[0];
      for (int d = 0; d < DMG_FFT_MAXDIM; ++d) {
        L[d] = im->L[d];
        A[d] = im->A[d];
      }
      for (int j = 0; j < nj && st == DMG_OK; ++j) {
        const void *src = first->in_buf == BUF_DAT ? (njobs ? dats[at + j] : im->dat)
                                                   : (njobs ? works[at + j] : im->work);
        st = dmg_fft_maxexp_launch(&first->p.in, im->ndim, A, L, src, njobs ? scales[at + j] : im->d_scale, stream);
      }
      if (st != DMG_OK) return st;
    }
    at += nj;
  }
  /* the group's descriptor is about 16 KB: keep it off the stack */
  struct dmg_fft_group *g = (struct dmg_fft_group *)calloc(1, sizeof(struct dmg_fft_group));
  if (!g) return dmg_error(DMG_ERR_NOMEM, "split group: out of memory");
  const int dt = arith_dtype(plans[0]->impl);
  for (int k = 0; k < most && st == DMG_OK; ++k) {
    g->count = 0;
    for (int i = 0, at = 0; i < count; ++i) {
      struct dmg_split_impl *im = plans[i]->impl;
      const int cnt = direction == FFTW_FORWARD ? im->nfwd : im->ninv;
      const int nj = njobs ? njobs[i] : 1;
      if (k < cnt) {
        const pass_rec *r = direction == FFTW_FORWARD ? &im->fwd[k] : &im->inv[k];
        struct dmg_fft_group_job *job = &g->job[g->count++];
        memset(job, 0, sizeof(*job));
        job->p = r->p;
        job->bt.count = nj;
        for (int j = 0; j < nj; ++j) {
          void *dat = njobs ? dats[at + j] : im->dat, *work = njobs ? works[at + j] : im->work;
          job->bt.src[j] = r->in_buf == BUF_DAT ? dat : work;
          job->bt.dst[j] = r->out_buf == BUF_DAT ? dat : work;
          job->bt.scale_exp[j] = njobs ? scales[at + j] : r->p.scale_exp;
        }
      }
      at += nj;
    }
    st = dmg_fft_pass_launch_group(g, dt, stream);
  }
  free(g);
  return st;
}

int dmg_split_run_group(int count, SplitPlan const *plans, int direction, void *stream) {
  if (!plans) return dmg_error(DMG_ERR_ARG, "dmg_split_run_group: NULL plan list");
  int st = group_check(count, plans, direction, 1, "dmg_split_run_group");
  if (st != DMG_OK) return st;
  return group_run(count, plans, NULL, NULL, NULL, NULL, direction, stream);
}

int dmg_split_run_group_batch(int count, SplitPlan const *plans, const int *njobs, void *const *dats,
                              void *const *works, int *const *scales, int direction, void *stream) {
  if (!plans || !njobs || !dats || !works) return dmg_error(DMG_ERR_ARG, "dmg_split_run_group_batch: NULL list");
  int st = group_check(count, plans, direction, 0, "dmg_split_run_group_batch");
  if (st != DMG_OK) return st;
  for (int i = 0, at = 0; i < count; ++i) {
    if (njobs[i] < 1 || njobs[i] > DMG_FFT_MAXBATCH)
      return dmg_error(DMG_ERR_ARG, "dmg_split_run_group_batch: plan %d with %d arrays (1 to %d)", i, njobs[i],
                       DMG_FFT_MAXBATCH);
    for (int j = at; j < at + njobs[i]; ++j)
      if (!dats[j] || !works[j] || (plans[i]->impl->arith == DMG_ARITH_DF && (!scales || !scales[j])))
        return dmg_error(DMG_ERR_ARG, "dmg_split_run_group_batch: NULL buffer for array %d", j);
    at += njobs[i];
  }
  return group_run(count, plans, njobs, dats, works, scales, direction, stream);
}

int dmg_split_group_launches(int count, SplitPlan const *plans, int direction) {
  if (!plans || group_check(count, plans, direction, 1, "dmg_split_group_launches") != DMG_OK) return 0;
  int most = 0, pre = 0;
  for (int i = 0; i < count; ++i) {
    const struct dmg_split_impl *im = plans[i]->impl;
    const int cnt = direction == FFTW_FORWARD ? im->nfwd : im->ninv;
    if (cnt > most) most = cnt;
    if (im->arith == DMG_ARITH_DF) pre += 1; /* the exponent pre-pass, per plan */
  }
  return most + pre;
}



/* ---------------------------------------------------------------- no-allocation run */

/* runSplitPlan without touching the allocator: the intermediate passes live
 * in the library's fixed device scratch array instead of the upper half of
 * the workspace.  The plan's tables must already be on the device (one
 * dmg_split_run uploads them).  Calls that overlap on the GPU share the one
 * array and race. */
int dmg_split_run_noalloc(SplitPlan plan, int direction, void *stream) {
  if (!plan) return dmg_error(DMG_ERR_ARG, "dmg_split_run_noalloc: NULL plan");
  struct dmg_split_impl *im = plan->impl;
  if (direction != FFTW_FORWARD && direction != FFTW_BACKWARD)
    return dmg_error(DMG_ERR_ARG, "dmg_split_run_noalloc: direction %d", direction);
  if (!im->dat || !im->work) return dmg_error(DMG_ERR_ARG, "dmg_split_run_noalloc: NULL buffer");
  if (im->scratch_bytes > dmg_noalloc_scratch_bytes())
    return dmg_error(DMG_ERR_BOUNDS,
                     "dmg_split_run_noalloc: this plan needs %zu bytes of scratch (ranks x extent x element size), "
                     "more than the fixed %zu-byte array; use runSplitPlan with a workspace instead",
                     im->scratch_bytes, dmg_noalloc_scratch_bytes());
  if (im->nfwd == 0)
    return dmg_error(DMG_ERR_UNSUPPORTED, "dmg_split_run_noalloc: the plan has no transform passes");
  if (!im->dev_valid)
    return dmg_error(DMG_ERR_ARG,
                     "dmg_split_run_noalloc: the plan's tables are not on the device yet; run it once with "
                     "runSplitPlan or dmg_split_run, which uploads them");
  int cur = 0;
  int st = dmg_rt_get_device(&cur);
  if (st != DMG_OK) return st;
  if (cur != im->dev_id)
    return dmg_error(DMG_ERR_ARG,
                     "dmg_split_run_noalloc: the plan's tables are on device %d but device %d is current; make "
                     "device %d current for this call",
                     im->dev_id, cur, im->dev_id);
  void *scratch = NULL;
  st = dmg_noalloc_scratch(&scratch);
  if (st != DMG_OK) return st;
  pass_rec *list = direction == FFTW_FORWARD ? im->fwd_s : im->inv_s;
  int cnt = direction == FFTW_FORWARD ? im->nfwd : im->ninv;
  int dt = arith_dtype(im);
  if (im->arith == DMG_ARITH_DF) {
    st = launch_maxexp(im, &list[0], list[0].in_buf == BUF_DAT ? im->dat : im->work, stream);
    if (st != DMG_OK) return st;
  }
  for (int k = 0; k < cnt; ++k) {
    const void *src = list[k].in_buf == BUF_DAT ? im->dat : list[k].in_buf == BUF_WORK ? im->work : scratch;
    void *dst = list[k].out_buf == BUF_DAT ? im->dat : list[k].out_buf == BUF_WORK ? im->work : scratch;
    st = dmg_fft_pass_launch(&list[k].p, dt, src, dst, stream);
    if (st != DMG_OK) return st;
  }
  return DMG_OK;
}

/* ---------------------------------------------------------------- visitor */

void visitData(Decomp d, data_visitor vis, double *dat) {
  int nd = d->ndim;
  int pos[DMG_MAXAX], slot[DMG_MAXAX], gpos[DMG_MAXAX];
  long long total = 1;
  /* the rank the descriptor's fields describe (max_local, isLocal): the view rank when it was made */
  int view = myRank(d);
  for (int i = 0; i < nd; ++i) total *= (long long)d->dims[i]->max_local + 1;
  for (long long e = 0; e < total; ++e) {
    long long rem = e, off = 0;
    for (int i = nd - 1; i >= 0; --i) {
      int c = (int)(rem % (d->dims[i]->max_local + 1));
      rem /= d->dims[i]->max_local + 1;
      slot[i] = c;
      off += dmg_axis_stride(d->dims[i], view) * c;
    }
    /* the global coordinate whose local offset is this slot, if any */
    for (int i = 0; i < nd; ++i) {
      DimDecomp dd = d->dims[i]->decomp;
      gpos[i] = -1;
      for (int g = 0; g < dd->coord_size; ++g)
        if (isLocal(d->dims[i], g) && dd->type_offset(dd, g) == slot[i]) {
          gpos[i] = g;
          break;
        }
      pos[i] = gpos[i];
    }
    vis(nd, pos, dat + 2 * off);
  }
}

/* ---------------------------------------------------------------- autotuning */

SplitPlan autotuneParallelPlan(Decomp start, fftw_complex *dat, int length, fftw_complex workspace[]) {
  return dmg_autotune_split(start, dat, length, workspace, DMG_C128, 0);
}
