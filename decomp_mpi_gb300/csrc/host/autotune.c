/*
 * Split-plan autotuner.
 *
 * The reference searches every divisor tuple B (split_fft.c:214-231), for
 * each every processor grid for A and B (split_fft.c:130-159), builds each
 * candidate and keeps the one whose forward run is fastest
 * (split_fft.c:78-128).  Here the same search runs with the timing done by
 * CUDA events on the GPU.  By default the grids come from makeProcessorGrid
 * (the reference's GUESS_GRID variant, split_fft.c:197-201), because on one
 * GPU the grid only relabels which virtual rank holds a block and the full
 * grid search multiplies the candidates by the grid count;
 * full_grid_search = 1 walks every grid as the reference does.  Each
 * candidate is timed in both pass schedules where its lengths allow both.
 */
#include <stdio.h>
#include <stdlib.h>
#include "dmg_internal.h"
#include "split_fft.h"
#include "k1_params.h"

SplitPlan dmg_build_plan_typed(int flags, int use_first, int use_second, Decomp start, int ndim, int A[], int B[],
                               int L[], int grid_a[], int grid_b[], void *dat, long long length, void *workspace,
                               int dtype);
void *dmg_split_create_events(int count);
void dmg_split_destroy_events(void *ev);
int dmg_split_record_event(void *ev, int idx, void *stream);
int dmg_split_event_elapsed(void *ev, int a, int b, float *ms);

typedef struct {
  Decomp start;
  void *dat, *work;
  long long length;
  int dtype;
  int full;
  SplitPlan best;
  double best_ms;
  void *ev;
  int tried;
} tune_ctx;

/* One untimed run uploads the tables, then one timed run (SEARCH_TRIAL =
 * SEARCH_REPEAT = 1 in the reference). */
static int time_forward(tune_ctx *c, SplitPlan cand, float *ms) {
  void *s = dmg_current_stream();
  if (dmg_split_run(cand, FFTW_FORWARD, s) != DMG_OK || dmg_split_record_event(c->ev, 0, s) != DMG_OK ||
      dmg_split_run(cand, FFTW_FORWARD, s) != DMG_OK || dmg_split_record_event(c->ev, 1, s) != DMG_OK ||
      dmg_split_event_elapsed(c->ev, 0, 1, ms) != DMG_OK)
    return DMG_ERR_CUDA;
  return DMG_OK;
}

/* Times a candidate in its default pass schedule and, where the plan allows
 * it, in the other one (one pass per dimension, or the reference's two
 * stages), and keeps the faster schedule on the plan. */
static void time_candidate(tune_ctx *c, SplitPlan cand) {
  if (!cand) return;
  float ms = 0;
  if (time_forward(c, cand, &ms) != DMG_OK) {
    freeSplitPlan(cand);
    return;
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
  } else {
    freeSplitPlan(cand);
  }
}

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
  time_candidate(c, cand);
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
      time_candidate(c, cand);
    }
  }
}

SplitPlan dmg_autotune_split(Decomp start, void *dat, long long length, void *workspace, int dtype,
                             int full_grid_search) {
  if (!start || !dat || !workspace) {
    dmg_error(DMG_ERR_ARG, "autotune: NULL argument");
    return NULL;
  }
  tune_ctx c = {start, dat, workspace, length, dtype, full_grid_search, NULL, 1e30, NULL, 0};
  c.ev = dmg_split_create_events(2);
  int B[DMG_MAXAX] = {0};
  const int printing = dmg_set_error_printing(0);
  factors(&c, start->ndim, 0, B);
  dmg_set_error_printing(printing);
  dmg_split_destroy_events(c.ev);
  if (!c.best) dmg_error(DMG_ERR_ARG, "autotune: no candidate plan could be built");
  else dmg_clear_error();
  return c.best;
}
