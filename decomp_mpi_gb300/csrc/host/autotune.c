/*
 * Split-plan autotuner.
 *
 * The reference searches every divisor tuple B (split_fft.c:214-231), for
 * each every processor grid for A and B (split_fft.c:130-159), builds each
 * candidate and keeps the one whose forward run is fastest
 * (split_fft.c:78-128), timing one run per candidate.  Here the same search
 * runs with the timing done by CUDA events on the GPU, the median of three
 * runs after one that uploads the candidate's tables.  By default the grids
 * come from makeProcessorGrid (the reference's GUESS_GRID variant,
 * split_fft.c:197-201), because on one GPU the grid only relabels which
 * virtual rank holds a block and the full grid search multiplies the
 * candidates by the grid count; full_grid_search = 1 walks every grid as
 * the reference does.
 *
 * Beyond the reference's search, the tuner chooses how the device runs the
 * plan: each candidate is timed in both pass schedules where its lengths
 * allow both, and the winner is then tried with half- and double-size tiles
 * and with the plan's own radix schedules in the runtime-length kernel (8s first and 4s
 * first) instead of the compile-time ones, keeping what is faster.
 *
 * Winners are cached per (dimensions, lengths, virtual ranks, element type,
 * grid search, start decomposition): a later call with the same key builds
 * the cached choice without timing anything.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "dmg_internal.h"
#include "split_fft.h"
#include "k1_params.h"
#include "fft_params.h"

SplitPlan dmg_build_plan_typed(int flags, int use_first, int use_second, Decomp start, int ndim, int A[], int B[],
                               int L[], int grid_a[], int grid_b[], void *dat, long long length, void *workspace,
                               int dtype);
void *dmg_split_create_events(int count);
void dmg_split_destroy_events(void *ev);
int dmg_split_record_event(void *ev, int idx, void *stream);
int dmg_split_event_elapsed(void *ev, int a, int b, float *ms);

#define TUNE_REPEATS 3

typedef struct {
  Decomp start;
  void *dat, *work;
  long long length;
  int dtype;
  int full;
  SplitPlan best;
  double best_ms;
  int best_grid_a[DMG_MAXAX], best_grid_b[DMG_MAXAX], best_full_grid;
  void *ev;
  int tried;
} tune_ctx;

/* ---------------------------------------------------------------- timing */

/* One untimed run uploads the tables, then the median of TUNE_REPEATS timed
 * runs (the reference times one run: SEARCH_TRIAL = SEARCH_REPEAT = 1). */
static int time_forward(tune_ctx *c, SplitPlan cand, float *ms) {
  void *s = dmg_current_stream();
  float t[TUNE_REPEATS];
  if (dmg_split_run(cand, FFTW_FORWARD, s) != DMG_OK) return DMG_ERR_CUDA;
  for (int i = 0; i < TUNE_REPEATS; ++i)
    if (dmg_split_record_event(c->ev, 0, s) != DMG_OK || dmg_split_run(cand, FFTW_FORWARD, s) != DMG_OK ||
        dmg_split_record_event(c->ev, 1, s) != DMG_OK || dmg_split_event_elapsed(c->ev, 0, 1, &t[i]) != DMG_OK)
      return DMG_ERR_CUDA;
  for (int i = 1; i < TUNE_REPEATS; ++i)
    for (int j = i; j > 0 && t[j] < t[j - 1]; --j) {
      float x = t[j];
      t[j] = t[j - 1];
      t[j - 1] = x;
    }
  *ms = t[TUNE_REPEATS / 2];
  return DMG_OK;
}

/* Times a candidate in its default pass schedule and, where the plan allows
 * it, in the other one (one pass per dimension, or the reference's two
 * stages), and keeps the faster schedule on the plan.  Returns 1 when the
 * candidate became the best so far (the context then owns it), else frees
 * it and returns 0. */
static int time_candidate(tune_ctx *c, SplitPlan cand) {
  if (!cand) return 0;
  float ms = 0;
  if (time_forward(c, cand, &ms) != DMG_OK) {
    freeSplitPlan(cand);
    return 0;
  }
  const int first = dmg_split_get_schedule(cand);
  const int other = first == DMG_SCHEDULE_LINES ? DMG_SCHEDULE_SPLIT : DMG_SCHEDULE_LINES;
  if (dmg_split_set_schedule(cand, other) == DMG_OK) {
    float ms2 = 0;
    if (time_forward(c, cand, &ms2) == DMG_OK && ms2 > 0 && ms2 < ms) ms = ms2;
    else dmg_split_set_schedule(cand, first);
  }
  c->tried++;
  if (ms > 0 && ms < c->best_ms) {
    if (c->best) freeSplitPlan(c->best);
    c->best = cand;
    c->best_ms = ms;
    return 1;
  }
  freeSplitPlan(cand);
  return 0;
}

/* The winner with half-size and double-size (wide-kernel) tiles and with the
 * runtime radix schedules: keeps each change that is faster. */
static void refine(tune_ctx *c) {
  SplitPlan b = c->best;
  if (!b) return;
  const int base = dmg_split_get_arith(b) == DMG_ARITH_FP64 ? DMG_FFT_TILE_TARGET_FP64
                                                            : DMG_FFT_TILE_TARGET(c->dtype == DMG_C128 ? 16 : 8);
  const int tiles[2] = {base / 2, 2 * base};
  for (int i = 0; i < 2; ++i) {
    const int keep = dmg_split_get_tile(b);
    if (dmg_split_set_tile(b, tiles[i]) != DMG_OK) continue;
    float ms = 0;
    c->tried++;
    if (time_forward(c, b, &ms) == DMG_OK && ms > 0 && ms < c->best_ms) c->best_ms = ms;
    else dmg_split_set_tile(b, keep);
  }
  const int radices[2] = {DMG_RADIX_PLAN8, DMG_RADIX_PLAN4};
  for (int i = 0; i < 2; ++i) {
    const int keep = dmg_split_get_radix(b);
    if (dmg_split_set_radix(b, radices[i]) != DMG_OK) continue;
    float ms = 0;
    c->tried++;
    if (time_forward(c, b, &ms) == DMG_OK && ms > 0 && ms < c->best_ms) c->best_ms = ms;
    else dmg_split_set_radix(b, keep);
  }
}

/* ---------------------------------------------------------------- search */

static void grids(tune_ctx *c, int nd, int *A, int *B, int *L, int use_first, int use_second, int dim_a, int *ga,
                  int dim_b, int *gb) {
  int P = c->start->comm->size;
  if (dim_a < nd) {
    int prev = 1;
    for (int i = 0; i < dim_a; ++i) prev *= ga[i];
    for (ga[dim_a] = 1; prev * ga[dim_a] <= P && ga[dim_a] <= A[dim_a]; ga[dim_a]++)
      grids(c, nd, A, B, L, use_first, use_second, dim_a + 1, ga, dim_b, gb);
    return;
  }
  if (dim_b < nd && !use_first) {
    int prev = 1;
    for (int i = 0; i < dim_b; ++i) prev *= gb[i];
    for (gb[dim_b] = 1; prev * gb[dim_b] <= P && gb[dim_b] <= B[dim_b]; gb[dim_b]++)
      grids(c, nd, A, B, L, use_first, use_second, dim_a, ga, dim_b + 1, gb);
    return;
  }
  SplitPlan cand = dmg_build_plan_typed(PREFER_STAGE1, use_first, use_second, c->start, nd, A, B, L, ga, gb,
                                        c->dat, c->length, c->work, c->dtype);
  if (time_candidate(c, cand)) {
    for (int i = 0; i < nd; ++i) {
      c->best_grid_a[i] = ga[i];
      c->best_grid_b[i] = gb[i];
    }
    c->best_full_grid = 1;
  }
}

static void factors(tune_ctx *c, int nd, int dim, int *B) {
  int L = c->start->dims[dim]->decomp->coord_size;
  for (B[dim] = 1; B[dim] <= L; B[dim]++) {
    if (L % B[dim]) continue;
    if (dim < nd - 1) {
      factors(c, nd, dim + 1, B);
      continue;
    }
    int A[DMG_MAXAX], Lv[DMG_MAXAX];
    int use_first = 1, use_second = 1;
    for (int i = 0; i < nd; ++i) {
      Lv[i] = c->start->dims[i]->decomp->coord_size;
      A[i] = Lv[i] / B[i];
      use_first = use_first && A[i] == 1;
      use_second = use_second && B[i] == 1;
    }
    if (use_second) continue; /* the reference rejects it (split_fft.c:188-195) */
    if (c->full) {
      int ga[DMG_MAXAX] = {0}, gb[DMG_MAXAX] = {0};
      grids(c, nd, A, B, Lv, use_first, use_second, 0, ga, 0, gb);
    } else {
      SplitPlan cand = dmg_makeParallelPlanTyped(c->start, B, c->dat, c->length, c->work, c->dtype);
      if (time_candidate(c, cand)) c->best_full_grid = 0;
    }
  }
}

/* ---------------------------------------------------------------- cache of winners */

typedef struct {
  int used;
  int ndim, L[DMG_MAXAX], nranks, dtype, full;
  uint64_t sig;
  /* the choice */
  int B[DMG_MAXAX], schedule, tile, radix;
  int full_grid, grid_a[DMG_MAXAX], grid_b[DMG_MAXAX];
} tune_entry;

#define TUNE_CACHE 64
static tune_entry g_cache[TUNE_CACHE];
static int g_cache_next;
static int g_last_tried;
static pthread_mutex_t g_cache_mu = PTHREAD_MUTEX_INITIALIZER;

/* FNV-1a over the start decomposition: per axis its plugin's maps over every
 * coordinate, the processor count, the rank stride and the memory strides of
 * every rank. */
static uint64_t fnv(uint64_t h, long long v) {
  for (int i = 0; i < 8; ++i) {
    h ^= (uint64_t)((v >> (8 * i)) & 0xFF);
    h *= 1099511628211ull;
  }
  return h;
}
static uint64_t start_signature(Decomp d) {
  uint64_t h = 14695981039346656037ull;
  const int P = d->comm->size;
  h = fnv(h, d->ndim);
  for (int i = 0; i < d->ndim; ++i) {
    AxisDecomp a = d->dims[i];
    DimDecomp dd = a->decomp;
    h = fnv(h, dd->coord_size);
    h = fnv(h, dd->proc_size);
    h = fnv(h, a->rank_stride);
    for (int g = 0; g < dd->coord_size; ++g) {
      h = fnv(h, dd->rank_offset(dd, g));
      h = fnv(h, dd->type_offset(dd, g));
    }
    for (int r = 0; r < P; ++r) h = fnv(h, dmg_axis_stride(a, r));
  }
  return h;
}

static tune_entry *cache_find(const tune_entry *key) {
  for (int i = 0; i < TUNE_CACHE; ++i) {
    tune_entry *e = &g_cache[i];
    if (!e->used || e->ndim != key->ndim || e->nranks != key->nranks || e->dtype != key->dtype ||
        e->full != key->full || e->sig != key->sig)
      continue;
    int same = 1;
    for (int d = 0; d < key->ndim; ++d) same = same && e->L[d] == key->L[d];
    if (same) return e;
  }
  return NULL;
}

/* Builds the cached choice; NULL when it no longer builds. */
static SplitPlan from_cache(const tune_entry *e, Decomp start, void *dat, long long length, void *work, int dtype) {
  int B[DMG_MAXAX], A[DMG_MAXAX], L[DMG_MAXAX], ga[DMG_MAXAX], gb[DMG_MAXAX];
  int use_first = 1, use_second = 1;
  for (int i = 0; i < e->ndim; ++i) {
    B[i] = e->B[i];
    L[i] = e->L[i];
    A[i] = L[i] / B[i];
    ga[i] = e->grid_a[i];
    gb[i] = e->grid_b[i];
    use_first = use_first && A[i] == 1;
    use_second = use_second && B[i] == 1;
  }
  SplitPlan p = e->full_grid ? dmg_build_plan_typed(PREFER_STAGE1, use_first, use_second, start, e->ndim, A, B, L, ga,
                                                    gb, dat, length, work, dtype)
                             : dmg_makeParallelPlanTyped(start, B, dat, length, work, dtype);
  if (!p) return NULL;
  if (dmg_split_set_schedule(p, e->schedule) != DMG_OK || dmg_split_set_tile(p, e->tile) != DMG_OK ||
      dmg_split_set_radix(p, e->radix) != DMG_OK) {
    freeSplitPlan(p);
    return NULL;
  }
  return p;
}

void dmg_autotune_cache_clear(void) {
  pthread_mutex_lock(&g_cache_mu);
  for (int i = 0; i < TUNE_CACHE; ++i) g_cache[i].used = 0;
  g_cache_next = 0;
  pthread_mutex_unlock(&g_cache_mu);
}

int dmg_autotune_cache_entries(void) {
  pthread_mutex_lock(&g_cache_mu);
  int n = 0;
  for (int i = 0; i < TUNE_CACHE; ++i) n += g_cache[i].used;
  pthread_mutex_unlock(&g_cache_mu);
  return n;
}

int dmg_autotune_last_timed(void) { return g_last_tried; }

SplitPlan dmg_autotune_split(Decomp start, void *dat, long long length, void *workspace, int dtype,
                             int full_grid_search) {
  if (!start || !dat || !workspace) {
    dmg_error(DMG_ERR_ARG, "autotune: NULL argument");
    return NULL;
  }
  tune_entry key;
  memset(&key, 0, sizeof(key));
  key.ndim = start->ndim;
  for (int i = 0; i < start->ndim; ++i) key.L[i] = start->dims[i]->decomp->coord_size;
  key.nranks = start->comm->size;
  key.dtype = dtype;
  key.full = full_grid_search;
  key.sig = start_signature(start);
  pthread_mutex_lock(&g_cache_mu);
  tune_entry *hit = cache_find(&key);
  tune_entry found;
  if (hit) found = *hit;
  pthread_mutex_unlock(&g_cache_mu);
  if (hit) {
    SplitPlan p = from_cache(&found, start, dat, length, workspace, dtype);
    if (p) {
      g_last_tried = 0;
      return p;
    }
  }

  tune_ctx c;
  memset(&c, 0, sizeof(c));
  c.start = start;
  c.dat = dat;
  c.work = workspace;
  c.length = length;
  c.dtype = dtype;
  c.full = full_grid_search;
  c.best_ms = 1e30;
  c.ev = dmg_split_create_events(2);
  int B[DMG_MAXAX] = {0};
  const int printing = dmg_set_error_printing(0);
  factors(&c, start->ndim, 0, B);
  refine(&c);
  dmg_set_error_printing(printing);
  dmg_split_destroy_events(c.ev);
  g_last_tried = c.tried;
  if (!c.best) {
    dmg_error(DMG_ERR_ARG, "autotune: no candidate plan could be built");
    return NULL;
  }
  dmg_clear_error();
  key.used = 1;
  for (int i = 0; i < start->ndim; ++i) {
    key.B[i] = key.L[i] / c.best->A_factors[i];
    key.grid_a[i] = c.best_grid_a[i];
    key.grid_b[i] = c.best_grid_b[i];
  }
  key.full_grid = c.best_full_grid;
  key.schedule = dmg_split_get_schedule(c.best);
  key.tile = dmg_split_get_tile(c.best);
  key.radix = dmg_split_get_radix(c.best);
  pthread_mutex_lock(&g_cache_mu);
  tune_entry *slot = cache_find(&key);
  if (!slot) {
    slot = &g_cache[g_cache_next];
    g_cache_next = (g_cache_next + 1) % TUNE_CACHE;
  }
  *slot = key;
  pthread_mutex_unlock(&g_cache_mu);
  return c.best;
}

SplitPlan dmg_autotuneParallelPlanTyped(Decomp start, void *dat, long long length, void *workspace, int dtype,
                                        int full_grid_search) {
  return dmg_autotune_split(start, dat, length, workspace, dtype, full_grid_search);
}
