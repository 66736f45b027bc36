/*
 * Processor-grid search over the virtual communicator.
 *
 * The choice of grid fixes the A and B decompositions of a split plan and so
 * the output layout, so the search is kept step for step the same as the
 * reference's (processor_grid.c:24-97): a depth-first walk over grid sizes
 * per dimension whose product stays within the rank count, scoring a grid by
 * its load (product of ceil(tasks/grid)) and breaking ties on the ratio of
 * the largest to the smallest per-rank task count.
 */
#include <stdlib.h>
#include "dmg_internal.h"
#include "split_fft.h"

typedef struct {
  int *best;
  int load;
  double asym;
} grid_search;

static void walk(grid_search *gs, int ndim, int dim, int *grid, const int *tasks, int max_proc, int procs, int load,
                 int lo, int hi) {
  /* The reference's loop also stops once the previous iteration's product
   * exceeded max_proc; that is the same as stopping at the first grid size
   * whose product does. */
  for (int g = 1; g <= max_proc && g <= tasks[dim]; ++g) {
    int np = procs * g;
    if (np > max_proc) break;
    grid[dim] = g;
    int mn = tasks[dim] / g;
    int mx = (tasks[dim] + g - 1) / g;
    int nl = load * mx;
    if (lo < mn) mn = lo;
    if (hi > mx) mx = hi;
    if (dim < ndim - 1) {
      walk(gs, ndim, dim + 1, grid, tasks, max_proc, np, nl, mn, mx);
    } else {
      double ratio = (double)mx / (double)mn;
      if ((nl <= gs->load || gs->load == 0) && (gs->load == 0 || nl < gs->load || ratio < gs->asym)) {
        gs->load = nl;
        gs->asym = ratio;
        for (int i = 0; i < ndim; ++i) gs->best[i] = grid[i];
      }
    }
  }
}

int *makeProcessorGrid(MPI_Comm comm, int ndim, int tasks[]) {
  if (!dmg_comm_ok(comm) || ndim < 1) {
    dmg_error(DMG_ERR_ARG, "makeProcessorGrid: bad arguments");
    return NULL;
  }
  int *result = (int *)calloc((size_t)ndim, sizeof(int));
  int *grid = (int *)calloc((size_t)ndim, sizeof(int));
  grid_search gs;
  gs.best = result;
  gs.load = 1;
  gs.asym = 10000.0;
  int biggest = 1;
  for (int i = 0; i < ndim; ++i) {
    result[i] = 1;
    gs.load *= tasks[i];
    if (tasks[i] > biggest) biggest = tasks[i];
  }
  walk(&gs, ndim, 0, grid, tasks, comm->size, 1, 1, biggest, 0);
  free(grid);
  return result;
}
