/*
 * Reshape planner: turns a (src, dest) pair of Decomps into per-axis device
 * address tables for the permutation kernel.
 *
 * Reference behaviour (reshape.c:351-449, typelist.c:74-119, reshape.c:461-492):
 * every participating rank builds one MPI datatype per peer by expanding the
 * dimensions in sortOrder; rank r sends the coordinates it holds to the rank
 * that holds them in dest, the receiver unpacks them in the same
 * lexicographic coordinate order.  When the rank maps form a proper grid and
 * all ranks agree on the expansion order, the k-th element of each message
 * is the same global coordinate on both sides, so the whole exchange is the
 * permutation
 *     dest[rank_d(g)][off_d(g)] = src[rank_s(g)][off_s(g)]   for every g held by both,
 * with rank(g) = sum_i rank_stride_i * rank_offset_i(g_i) and
 * off(g) = sum_i memory_stride_i * type_offset_i(g_i) (reshape.c:281-315).
 * Both are sums over axes, so each side reduces to one small table per axis,
 * built here by calling the DimDecomp plugins on the host.  The planner
 * checks the proper-grid and common-order conditions and refuses (with an
 * error) the decompositions where the reference's message matching would
 * differ from this permutation.
 */
#include <limits.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "dmg_internal.h"
#include "k1_params.h"

#define RK_ABSENT (-(1 << 27))

typedef struct {
  int ranked;                 /* memory strides differ between virtual ranks */
  int nranks;                 /* proc_used */
  int64_t pitch;              /* elements per virtual rank */
  int32_t *rk[DMG_MAXAX];     /* rank part rank_stride*pos, RK_ABSENT when not held */
  int64_t *to[DMG_MAXAX];     /* type offset (elements) */
  int64_t ustride[DMG_MAXAX]; /* uniform memory stride (elements) */
  int64_t *rstride;           /* ranked: [ndim][nranks] memory stride (elements) */
  int64_t max_extent;         /* largest rank extent */
} side_raw;

struct dmg_reshape_impl {
  int esize;  /* element bytes */
  int unit;   /* bytes moved per kernel unit before fusion */
  int m;      /* units per element */
  int ndim;   /* Decomp dimensions */
  int naxes;  /* kernel axes (ndim, plus one when m > 1) */
  int len[DMG_MAXAX];
  side_raw s, d;
  long long moved;  /* elements moved per run */
  /* device state */
  void *dev_buf;
  size_t dev_bytes;
  int dev_valid;
  struct dmg_k1_params kp;       /* unfused */
  struct dmg_k1_params kp_fused; /* fused along one axis */
  int fuse_v;                    /* fusion factor (1 = none) */
  char desc[256];
};

static void side_free(side_raw *s) {
  for (int a = 0; a < DMG_MAXAX; ++a) {
    free(s->rk[a]);
    free(s->to[a]);
  }
  free(s->rstride);
  memset(s, 0, sizeof(*s));
}

/* Checks that rank = sum rank_stride_i * pos_i inverts pos_i = (rank /
 * rank_stride_i) % proc_size_i for every data-holding position tuple, and
 * that no other rank below proc_used holds a copy of some tuple's data. */
int dmg_check_proper_grid(Decomp D, const char *side) {
  int nd = D->ndim;
  /* sufficient mixed-radix condition */
  int ok = 1;
  for (int i = 0; i < nd && ok; ++i) {
    AxisDecomp ai = D->dims[i];
    int psi = ai->decomp->proc_size;
    if (psi <= 1) continue;
    long long low = 0;
    for (int j = 0; j < nd; ++j) {
      if (j == i) continue;
      AxisDecomp aj = D->dims[j];
      int psj = aj->decomp->proc_size;
      if (psj <= 1) continue;
      if (aj->rank_stride <= ai->rank_stride) low += (long long)aj->rank_stride * (psj - 1);
      else if (aj->rank_stride % ((long long)ai->rank_stride * psi) != 0) ok = 0;
    }
    if (low >= ai->rank_stride) ok = 0;
  }
  if (!ok) {
    /* exact check over the data-holding tuples when there are few */
    long long ntup = 1;
    for (int i = 0; i < nd; ++i) {
      ntup *= D->dims[i]->decomp->proc_size;
      if (ntup > (1LL << 22)) break;
    }
    if (ntup > (1LL << 22)) {
      return dmg_error(DMG_ERR_UNSUPPORTED,
                       "makeReshapePlan: %s rank strides do not form a mixed-radix processor grid",
                       side);
    }
    int p[DMG_MAXAX] = {0};
    for (long long t = 0; t < ntup; ++t) {
      long long rem = t;
      int holds = 1;
      long long r = 0;
      for (int i = nd - 1; i >= 0; --i) {
        int ps = D->dims[i]->decomp->proc_size;
        p[i] = (int)(rem % ps);
        rem /= ps;
        holds &= D->dims[i]->pos_n_local[p[i]] > 0;
        r += (long long)D->dims[i]->rank_stride * p[i];
      }
      if (!holds) continue;
      for (int i = 0; i < nd; ++i) {
        if (dmg_axis_pos(D->dims[i], (int)r) != p[i]) {
          return dmg_error(DMG_ERR_UNSUPPORTED,
                           "makeReshapePlan: %s position tuple maps to rank %lld which sits "
                           "elsewhere in the grid (not a proper processor grid)",
                           side, r);
        }
      }
    }
  }
  /* no replicas: a data-holding rank must be the rank of its own tuple */
  for (int r = 0; r < D->proc_used; ++r) {
    if (!dmg_rank_holds(D, r)) continue;
    long long back = 0;
    for (int i = 0; i < nd; ++i) back += (long long)D->dims[i]->rank_stride * dmg_axis_pos(D->dims[i], r);
    if (back != r) {
      return dmg_error(DMG_ERR_UNSUPPORTED,
                       "makeReshapePlan: %s virtual rank %d holds a copy of rank %lld's data", side,
                       r, back);
    }
  }
  return DMG_OK;
}

static int side_build(side_raw *s, Decomp D, const char *side) {
  memset(s, 0, sizeof(*s));
  int nd = D->ndim;
  s->nranks = D->proc_used;
  s->pitch = extent64(D);
  s->max_extent = s->pitch;
  s->ranked = 0;
  for (int i = 0; i < nd; ++i)
    if (D->dims[i]->rank_memory_stride) s->ranked = 1;
  for (int i = 0; i < nd; ++i) {
    AxisDecomp a = D->dims[i];
    DimDecomp dd = a->decomp;
    int L = dd->coord_size;
    s->rk[i] = (int32_t *)malloc((size_t)L * sizeof(int32_t));
    s->to[i] = (int64_t *)malloc((size_t)L * sizeof(int64_t));
    if (!s->rk[i] || !s->to[i]) return dmg_error(DMG_ERR_NOMEM, "makeReshapePlan: out of memory");
    s->ustride[i] = a->memory_stride;
    for (int g = 0; g < L; ++g) {
      int p = dd->rank_offset(dd, g);
      if (p < 0 || p >= dd->proc_size) {
        s->rk[i][g] = RK_ABSENT;
        s->to[i][g] = 0;
        continue;
      }
      int off = dd->type_offset(dd, g);
      if (off < 0 || off > a->pos_max_local[p]) {
        return dmg_error(DMG_ERR_ARG, "makeReshapePlan: %s dim %d coordinate %d has local offset %d",
                         side, i, g, off);
      }
      s->rk[i][g] = a->rank_stride * p;
      s->to[i][g] = off;
    }
  }
  if (s->ranked) {
    int P = s->nranks;
    s->rstride = (int64_t *)malloc((size_t)nd * P * sizeof(int64_t));
    for (int i = 0; i < nd; ++i)
      for (int r = 0; r < P; ++r) s->rstride[(size_t)i * P + r] = dmg_axis_stride(D->dims[i], r);
  }
  return dmg_check_proper_grid(D, side);
}

/* Address (elements) of coordinate g on a side, -1 when the side does not hold it. */
static int64_t side_addr(const side_raw *s, int nd, const int *g) {
  int64_t R = 0;
  for (int i = 0; i < nd; ++i) {
    if (s->rk[i][g[i]] == RK_ABSENT) return -1;
    R += s->rk[i][g[i]];
  }
  int64_t a = R * s->pitch;
  for (int i = 0; i < nd; ++i) {
    int64_t st = s->ranked ? s->rstride[(size_t)i * s->nranks + R] : s->ustride[i];
    a += st * s->to[i][g[i]];
  }
  return a;
}

/* Fraction of unit steps along axis `ax` (addresses in kernel units),
 * measured through a held reference coordinate; -1 for a length-1 axis. */
static double axis_contiguity(const struct dmg_reshape_impl *im, const side_raw *s, int ax) {
  if (im->len[ax] <= 1) return -1.0;
  if (ax == im->ndim) return 1.0 + 1e-3; /* the unit axis inside one element */
  int g[DMG_MAXAX];
  for (int i = 0; i < im->ndim; ++i) {
    g[i] = 0;
    for (int k = 0; k < im->len[i]; ++k)
      if (s->rk[i][k] != RK_ABSENT) {
        g[i] = k;
        break;
      }
  }
  int hits = 0, total = 0;
  int64_t prev = -1;
  for (int k = 0; k < im->len[ax]; ++k) {
    g[ax] = k;
    int64_t a = side_addr(s, im->ndim, g);
    if (a >= 0 && prev >= 0) {
      total++;
      if (a - prev == 1) hits++;
    }
    prev = a;
  }
  if (total == 0) return 0.0;
  return (double)hits / (double)total;
}

static void plan_free_device(struct dmg_reshape_impl *im) {
  if (im->dev_buf) dmg_dev_free(im->dev_buf);
  im->dev_buf = NULL;
  im->dev_valid = 0;
}

/* Build and upload the device tables for both variants. */
static int plan_upload(struct dmg_reshape_impl *im) {
  plan_free_device(im);
  int na = im->naxes, nd = im->ndim, m = im->m;
  /* host staging: per side, per axis int64 table + int32 rank table;
   * ranked stride table; then the fused copies */
  size_t words = 0;
  for (int a = 0; a < na; ++a) words += (size_t)im->len[a] * 2 /* two sides */;
  size_t rkw = 0;
  for (int a = 0; a < na; ++a) rkw += (size_t)im->len[a] * 2;
  size_t rsw = 0;
  if (im->s.ranked) rsw += (size_t)na * im->s.nranks;
  if (im->d.ranked) rsw += (size_t)na * im->d.nranks;
  size_t fusedw = im->fuse_v > 1 ? words : 0;
  size_t nbytes = (words + rsw + fusedw) * sizeof(int64_t) + rkw * sizeof(int32_t) + 256;
  int64_t *h = (int64_t *)calloc(words + rsw + fusedw, sizeof(int64_t));
  int32_t *hrk = (int32_t *)calloc(rkw ? rkw : 1, sizeof(int32_t));
  if (!h || !hrk) {
    free(h);
    free(hrk);
    return dmg_error(DMG_ERR_NOMEM, "reshape plan: out of host memory");
  }
  void *dev = NULL;
  int st = dmg_dev_alloc(&dev, nbytes);
  if (st != DMG_OK) {
    free(h);
    free(hrk);
    return st;
  }
  int64_t *dtab = (int64_t *)dev;
  int32_t *drk = (int32_t *)(dtab + words + rsw + fusedw);
  size_t pos = 0, rpos = 0;
  const side_raw *sides[2] = {&im->s, &im->d};
  struct dmg_k1_side *ks[2] = {&im->kp.src, &im->kp.dst};
  int64_t *sep_host[2][DMG_MAXAX];
  for (int sd = 0; sd < 2; ++sd) {
    const side_raw *s = sides[sd];
    struct dmg_k1_side *k = ks[sd];
    memset(k, 0, sizeof(*k));
    k->ranked = s->ranked;
    k->nranks = s->nranks;
    k->pitch = s->pitch * m;
    for (int a = 0; a < na; ++a) {
      int L = im->len[a];
      int64_t *t = h + pos;
      int32_t *r = hrk + rpos;
      sep_host[sd][a] = t;
      for (int g = 0; g < L; ++g) {
        if (a == nd) { /* unit axis */
          t[g] = g;
          r[g] = 0;
          continue;
        }
        int32_t rk = s->rk[a][g];
        r[g] = rk;
        if (s->ranked) {
          t[g] = s->to[a][g];
        } else {
          t[g] = (rk == RK_ABSENT) ? DMG_ABSENT : ((int64_t)rk * s->pitch + s->ustride[a] * s->to[a][g]) * m;
        }
      }
      k->tab[a] = dtab + pos;
      k->rk[a] = drk + rpos;
      pos += L;
      rpos += L;
    }
    if (s->ranked) {
      int64_t *t = h + pos;
      int P = s->nranks;
      for (int a = 0; a < na; ++a)
        for (int R = 0; R < P; ++R) t[(size_t)a * P + R] = (a == nd) ? 1 : s->rstride[(size_t)a * P + R] * m;
      k->rstride = dtab + pos;
      pos += (size_t)na * P;
    }
  }
  if (im->fuse_v > 1) {
    int v = im->fuse_v, f = im->kp_fused.ax0;
    struct dmg_k1_side *kf[2] = {&im->kp_fused.src, &im->kp_fused.dst};
    for (int sd = 0; sd < 2; ++sd) {
      memset(kf[sd], 0, sizeof(*kf[sd]));
      for (int a = 0; a < na; ++a) {
        int L = im->len[a];
        int Lf = (a == f) ? L / v : L;
        int64_t *t = h + pos;
        for (int g = 0; g < Lf; ++g) {
          int64_t x = (a == f) ? sep_host[sd][a][(size_t)g * v] : sep_host[sd][a][g];
          t[g] = (x < 0) ? DMG_ABSENT : x / v;
        }
        kf[sd]->tab[a] = dtab + pos;
        pos += Lf;
      }
    }
  }
  st = dmg_dev_upload(dev, h, (words + rsw + fusedw) * sizeof(int64_t));
  if (st == DMG_OK && rkw) st = dmg_dev_upload(drk, hrk, rkw * sizeof(int32_t));
  free(h);
  free(hrk);
  if (st != DMG_OK) {
    dmg_dev_free(dev);
    return st;
  }
  im->dev_buf = dev;
  im->dev_bytes = nbytes;
  im->dev_valid = 1;
  return DMG_OK;
}

/* Can axis f fuse v consecutive units on both sides (separable only). */
static int can_fuse(const struct dmg_reshape_impl *im, int f, int v) {
  if (im->s.ranked || im->d.ranked) return 0;
  if (im->len[f] % v != 0) return 0;
  const side_raw *sides[2] = {&im->s, &im->d};
  for (int sd = 0; sd < 2; ++sd) {
    const side_raw *s = sides[sd];
    for (int a = 0; a < im->naxes; ++a) {
      for (int g = 0; g < im->len[a]; ++g) {
        int64_t x;
        if (a == im->ndim) x = g;
        else {
          if (s->rk[a][g] == RK_ABSENT) {
            if (a == f) return 0;
            continue;
          }
          x = ((int64_t)s->rk[a][g] * s->pitch + s->ustride[a] * s->to[a][g]) * im->m;
        }
        if (a == f) {
          int64_t base;
          if (a == im->ndim) base = (g / v) * v;
          else {
            int g0 = (g / v) * v;
            base = ((int64_t)s->rk[a][g0] * s->pitch + s->ustride[a] * s->to[a][g0]) * im->m;
          }
          if (x != base + (g % v)) return 0;
          if (base % v != 0) return 0;
        } else if (x % v != 0) {
          return 0;
        }
      }
    }
  }
  return 1;
}

/* Choose tile axes and extents for one parameter set. */
static void choose_tiles(struct dmg_k1_params *kp, const int *len, int na, int ax_s, int ax_d,
                         const double *dscore, int unit) {
  kp->naxes = na;
  for (int a = 0; a < DMG_MAXAX; ++a) kp->len[a] = a < na ? len[a] : 1;
  int tile_units = (unit >= 16) ? 1024 : 2048;
  if (ax_s != ax_d) {
    kp->ax0 = ax_s;
    kp->ax1 = ax_d;
    kp->load_fast = 0;
    kp->store_fast = 1;
    int e0max = (unit >= 16) ? 32 : 64;
    kp->e0 = len[ax_s] < e0max ? len[ax_s] : e0max;
    int e1max = tile_units / kp->e0;
    if (e1max > 64) e1max = 64;
    kp->e1 = len[ax_d] < e1max ? len[ax_d] : e1max;
  } else {
    /* same fast axis: the direct kernel moves 2048 units per tile without shared memory */
    tile_units = 2048;
    kp->ax0 = ax_s;
    kp->load_fast = 0;
    kp->store_fast = 0;
    kp->e0 = len[ax_s] < tile_units ? len[ax_s] : tile_units;
    /* second tile axis: best remaining dst contiguity, else the longest */
    int best = -1;
    for (int a = 0; a < na; ++a) {
      if (a == ax_s || len[a] <= 1) continue;
      if (best < 0 || dscore[a] > dscore[best] || (dscore[a] == dscore[best] && a > best)) best = a;
    }
    kp->ax1 = best;
    if (best >= 0) {
      int e1max = tile_units / kp->e0;
      if (e1max < 1) e1max = 1;
      kp->e1 = len[best] < e1max ? len[best] : e1max;
    } else {
      kp->e1 = 1;
    }
  }
  kp->nt0 = (len[kp->ax0] + kp->e0 - 1) / kp->e0;
  kp->nt1 = kp->ax1 >= 0 ? (len[kp->ax1] + kp->e1 - 1) / kp->e1 : 1;
  kp->nbatch = 0;
  /* batch axes ordered by dst contiguity, most contiguous first */
  int used[DMG_MAXAX] = {0};
  used[kp->ax0] = 1;
  if (kp->ax1 >= 0) used[kp->ax1] = 1;
  for (;;) {
    int best = -1;
    for (int a = 0; a < na; ++a) {
      if (used[a]) continue;
      if (best < 0 || dscore[a] > dscore[best] || (dscore[a] == dscore[best] && a > best)) best = a;
    }
    if (best < 0) break;
    used[best] = 1;
    kp->batch_ax[kp->nbatch++] = best;
  }
  kp->ntiles = (int64_t)kp->nt0 * kp->nt1;
  for (int b = 0; b < kp->nbatch; ++b) kp->ntiles *= len[kp->batch_ax[b]];
}

ReshapePlan makeReshapePlan(MPI_Comm comm, MPI_Datatype base, Decomp src, Decomp dest) {
  if (!dmg_comm_ok(comm) || !src || !dest) {
    dmg_error(DMG_ERR_ARG, "makeReshapePlan: NULL argument");
    return NULL;
  }
  if (compatible(src, dest) == NOT_COMPATIBLE) {
    raise_error(comm, "Decomp not compatible in makeReshapePlan");
    return NULL;
  }
  if (src->comm != comm) {
    raise_error(comm, "makeReshapePlan: communicator differs from the decompositions'");
    return NULL;
  }
  if (base < 1) {
    dmg_error(DMG_ERR_ARG, "makeReshapePlan: bad base type size %d", base);
    return NULL;
  }
  int nd = src->ndim;
  int unit = 1;
  while (unit < 16 && base % (unit * 2) == 0) unit *= 2;
  int m = base / unit;
  int na = nd + (m > 1 ? 1 : 0);
  if (na > DMG_MAXAX) {
    dmg_error(DMG_ERR_UNSUPPORTED, "makeReshapePlan: %d dimensions (at most %d)", nd,
              m > 1 ? DMG_MAXAX - 1 : DMG_MAXAX);
    return NULL;
  }
  /* every participating rank must expand the dimensions in one order */
  int *order0 = (int *)calloc((size_t)nd, sizeof(int));
  int *order = (int *)calloc((size_t)nd, sizeof(int));
  int have0 = 0;
  int maxp = src->proc_used > dest->proc_used ? src->proc_used : dest->proc_used;
  for (int r = 0; r < maxp; ++r) {
    int part = (r < src->proc_used && dmg_rank_holds(src, r)) ||
               (r < dest->proc_used && dmg_rank_holds(dest, r));
    if (!part) continue;
    dmg_sort_order(nd, order, src, r);
    if (!have0) {
      memcpy(order0, order, (size_t)nd * sizeof(int));
      have0 = 1;
    } else if (memcmp(order0, order, (size_t)nd * sizeof(int)) != 0) {
      free(order0);
      free(order);
      dmg_error(DMG_ERR_UNSUPPORTED,
                "makeReshapePlan: virtual ranks expand dimensions in different orders");
      return NULL;
    }
  }
  if (!have0) dmg_sort_order(nd, order0, src, comm->rank);
  free(order);

  struct dmg_reshape_impl *im = (struct dmg_reshape_impl *)calloc(1, sizeof(*im));
  ReshapePlan plan = (ReshapePlan)calloc(1, sizeof(struct reshape_plan));
  if (!im || !plan) {
    free(im);
    free(plan);
    free(order0);
    dmg_error(DMG_ERR_NOMEM, "makeReshapePlan: out of memory");
    return NULL;
  }
  plan->comm = comm;
  plan->src = src;
  plan->dest = dest;
  plan->order = order0;
  plan->impl = im;
  im->esize = base;
  im->unit = unit;
  im->m = m;
  im->ndim = nd;
  im->naxes = na;
  for (int i = 0; i < nd; ++i) im->len[i] = src->dims[i]->decomp->coord_size;
  if (m > 1) im->len[nd] = m;
  if (side_build(&im->s, src, "src") != DMG_OK || side_build(&im->d, dest, "dest") != DMG_OK) {
    freeReshapePlan(plan);
    return NULL;
  }
  /* elements moved: held on both sides, a product over axes */
  long long moved = 1;
  for (int i = 0; i < nd; ++i) {
    long long c = 0;
    for (int g = 0; g < im->len[i]; ++g) c += (im->s.rk[i][g] != RK_ABSENT && im->d.rk[i][g] != RK_ABSENT);
    moved *= c;
  }
  im->moved = moved;

  /* fastest axis of each side */
  double sscore[DMG_MAXAX] = {0}, dscore[DMG_MAXAX] = {0};
  int ax_s = na - 1, ax_d = na - 1;
  for (int a = 0; a < na; ++a) {
    sscore[a] = axis_contiguity(im, &im->s, a);
    dscore[a] = axis_contiguity(im, &im->d, a);
  }
  for (int a = 0; a < na; ++a) {
    if (sscore[a] > sscore[ax_s] || (sscore[a] == sscore[ax_s] && a > ax_s)) ax_s = a;
    if (dscore[a] > dscore[ax_d] || (dscore[a] == dscore[ax_d] && a > ax_d)) ax_d = a;
  }
  choose_tiles(&im->kp, im->len, na, ax_s, ax_d, dscore, unit);
  /* widen the unit along the common fastest axis when both sides allow */
  im->fuse_v = 1;
  if (ax_s == ax_d && !im->s.ranked && !im->d.ranked) {
    for (int v = 16 / unit; v >= 2; v /= 2) {
      if (can_fuse(im, ax_s, v)) {
        im->fuse_v = v;
        break;
      }
    }
  }
  if (im->fuse_v > 1) {
    int flen[DMG_MAXAX];
    memcpy(flen, im->len, sizeof(flen));
    flen[ax_s] /= im->fuse_v;
    choose_tiles(&im->kp_fused, flen, na, ax_s, ax_s, dscore, unit * im->fuse_v);
    im->kp_fused.ax0 = ax_s;
  }
  snprintf(im->desc, sizeof(im->desc),
           "src=%s dst=%s unit=%dB fuse=%d tile=ax%d:%d x ax%d:%d load_fast=%d store_fast=%d tiles=%lld",
           im->s.ranked ? "ranked" : "separable", im->d.ranked ? "ranked" : "separable", unit,
           im->fuse_v, im->kp.ax0, im->kp.e0, im->kp.ax1, im->kp.e1, im->kp.load_fast,
           im->kp.store_fast, (long long)im->kp.ntiles);
  return plan;
}

void freeReshapePlan(ReshapePlan plan) {
  if (!plan) return;
  struct dmg_reshape_impl *im = plan->impl;
  if (im) {
    plan_free_device(im);
    side_free(&im->s);
    side_free(&im->d);
    free(im);
  }
  free(plan->order);
  free(plan);
}

int dmg_reshape_set_pitch(ReshapePlan plan, long long src_pitch, long long dest_pitch) {
  if (!plan || !plan->impl) return dmg_error(DMG_ERR_ARG, "dmg_reshape_set_pitch: NULL plan");
  struct dmg_reshape_impl *im = plan->impl;
  if (src_pitch && src_pitch < im->s.max_extent)
    return dmg_error(DMG_ERR_BOUNDS, "src pitch %lld below extent %lld", src_pitch, (long long)im->s.max_extent);
  if (dest_pitch && dest_pitch < im->d.max_extent)
    return dmg_error(DMG_ERR_BOUNDS, "dest pitch %lld below extent %lld", dest_pitch, (long long)im->d.max_extent);
  int changed = 0;
  if (src_pitch && src_pitch != im->s.pitch) {
    im->s.pitch = src_pitch;
    changed = 1;
  }
  if (dest_pitch && dest_pitch != im->d.pitch) {
    im->d.pitch = dest_pitch;
    changed = 1;
  }
  if (changed) {
    plan_free_device(im);
    /* fusion depends on the pitch (address alignment) */
    if (im->fuse_v > 1 && !can_fuse(im, im->kp_fused.ax0, im->fuse_v)) im->fuse_v = 1;
  }
  return DMG_OK;
}

long long dmg_reshape_pitch(ReshapePlan plan, int which) {
  if (!plan || !plan->impl) return -1;
  return which == 0 ? plan->impl->s.pitch : plan->impl->d.pitch;
}

long long dmg_reshape_elements(ReshapePlan plan) { return plan && plan->impl ? plan->impl->moved : -1; }
long long dmg_reshape_bytes(ReshapePlan plan) {
  return plan && plan->impl ? 2LL * plan->impl->moved * plan->impl->esize : -1;
}
const char *dmg_reshape_describe(ReshapePlan plan) { return plan && plan->impl ? plan->impl->desc : ""; }
int dmg_reshape_launches(ReshapePlan plan) { return plan && plan->impl && plan->impl->moved > 0 ? 1 : 0; }

int dmg_reshape_run(ReshapePlan plan, const void *src, void *dest, void *stream) {
  if (!plan || !plan->impl) return dmg_error(DMG_ERR_ARG, "runReshapePlan: NULL plan");
  struct dmg_reshape_impl *im = plan->impl;
  if (im->moved == 0) return DMG_OK;
  if (!src || !dest) return dmg_error(DMG_ERR_ARG, "runReshapePlan: NULL buffer");
  if (src == dest) return dmg_error(DMG_ERR_ARG, "runReshapePlan: src and dest are the same buffer");
  if (!im->dev_valid) {
    int st = plan_upload(im);
    if (st != DMG_OK) return st;
  }
  int v = im->fuse_v;
  if (v > 1 && ((uintptr_t)src % (uintptr_t)(im->unit * v) == 0) &&
      ((uintptr_t)dest % (uintptr_t)(im->unit * v) == 0)) {
    /* the fused variant shares the rank/stride setup of the unfused one */
    im->kp_fused.src.ranked = im->kp_fused.dst.ranked = 0;
    return dmg_k1_launch(&im->kp_fused, im->unit * v, src, dest, stream);
  }
  if ((uintptr_t)src % (uintptr_t)im->unit || (uintptr_t)dest % (uintptr_t)im->unit)
    return dmg_error(DMG_ERR_ARG, "runReshapePlan: buffers not aligned to %d bytes", im->unit);
  return dmg_k1_launch(&im->kp, im->unit, src, dest, stream);
}

/* The kernel parameters and unit dmg_reshape_run would launch with for
 * these buffers (the fused form when both pointers allow it); an error when
 * the buffers do not fit the plan. */
static int launch_choice(struct dmg_reshape_impl *im, const void *src, const void *dest,
                         const struct dmg_k1_params **kp, int *unit) {
  int v = im->fuse_v;
  if (v > 1 && ((uintptr_t)src % (uintptr_t)(im->unit * v) == 0) &&
      ((uintptr_t)dest % (uintptr_t)(im->unit * v) == 0)) {
    im->kp_fused.src.ranked = im->kp_fused.dst.ranked = 0;
    *kp = &im->kp_fused;
    *unit = im->unit * v;
    return DMG_OK;
  }
  if ((uintptr_t)src % (uintptr_t)im->unit || (uintptr_t)dest % (uintptr_t)im->unit)
    return dmg_error(DMG_ERR_ARG, "dmg_reshape_run_group: buffers not aligned to %d bytes", im->unit);
  *kp = &im->kp;
  *unit = im->unit;
  return DMG_OK;
}

int dmg_reshape_run_group(int count, const ReshapePlan *plans, const void *const *srcs, void *const *dests,
                          void *stream) {
  if (count < 0 || (count > 0 && (!plans || !srcs || !dests)))
    return dmg_error(DMG_ERR_ARG, "dmg_reshape_run_group: %d jobs, NULL arrays", count);
  struct dmg_k1_group *g = (struct dmg_k1_group *)calloc(1, sizeof(struct dmg_k1_group));
  if (!g) return dmg_error(DMG_ERR_NOMEM, "dmg_reshape_run_group: out of host memory");
  int gunit = 0, st = DMG_OK;
  for (int j = 0; j <= count && st == DMG_OK; ++j) {
    const struct dmg_k1_params *kp = NULL;
    int unit = 0, direct = 0;
    if (j < count) {
      ReshapePlan pl = plans[j];
      if (!pl || !pl->impl) {
        st = dmg_error(DMG_ERR_ARG, "dmg_reshape_run_group: job %d has no plan", j);
        break;
      }
      struct dmg_reshape_impl *im = pl->impl;
      if (im->moved == 0) continue;
      if (!srcs[j] || !dests[j] || srcs[j] == dests[j]) {
        st = dmg_error(DMG_ERR_ARG, "dmg_reshape_run_group: job %d's buffers", j);
        break;
      }
      if (!im->dev_valid && (st = plan_upload(im)) != DMG_OK) break;
      if ((st = launch_choice(im, srcs[j], dests[j], &kp, &unit)) != DMG_OK) break;
      direct = kp->load_fast == kp->store_fast && kp->e0 * kp->e1 <= 2048;
    }
    /* close the open group when this job cannot join it (or at the end) */
    if (g->count > 0 && (j == count || !direct || unit != gunit || g->count == DMG_K1_MAXGROUP ||
                         kp->src.ranked != g->job[0].p.src.ranked || kp->dst.ranked != g->job[0].p.dst.ranked)) {
      st = g->count == 1 ? dmg_k1_launch(&g->job[0].p, gunit, g->job[0].src, g->job[0].dst, stream)
                         : dmg_k1_launch_group(g, gunit, stream);
      g->count = 0;
      g->total_tiles = 0;
      if (st != DMG_OK) break;
    }
    if (j == count) break;
    if (!direct) {
      st = dmg_k1_launch(kp, unit, srcs[j], dests[j], stream); /* the transposing kernel runs alone */
      continue;
    }
    struct dmg_k1_group_job *gj = &g->job[g->count++];
    gj->p = *kp;
    gj->src = srcs[j];
    gj->dst = dests[j];
    gj->first_tile = g->total_tiles;
    g->total_tiles += kp->ntiles;
    gunit = unit;
  }
  free(g);
  return st;
}

void runReshapePlan(MPI_Comm comm, ReshapePlan plan, void *src, void *dest) {
  (void)comm;
  dmg_reshape_run(plan, src, dest, dmg_current_stream());
}

int checkReshapePlanBounds(ReshapePlan plan, int type_size, int src_len, int dest_len) {
  if (!plan || !plan->impl) return 1;
  struct dmg_reshape_impl *im = plan->impl;
  if (type_size != im->esize) {
    fprintf(stderr, "checkReshapePlanBounds: type size %d differs from the plan's %d\n", type_size, im->esize);
    return 1;
  }
  if (im->s.max_extent > src_len) {
    fprintf(stderr, "checkReshapePlanBounds: src extent %lld beyond length %d\n", (long long)im->s.max_extent, src_len);
    return 1;
  }
  if (im->d.max_extent > dest_len) {
    fprintf(stderr, "checkReshapePlanBounds: dest extent %lld beyond length %d\n", (long long)im->d.max_extent, dest_len);
    return 1;
  }
  return 0;
}
