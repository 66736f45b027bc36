/*
 * Global-order input and output of distributed arrays: the virtual-grid
 * counterpart of the reference's MPI-IO file view (reshape.c:137-172,
 * 494-521; fftw_bench.c:26-100).  The file format is the reference's: the
 * global array in C order, elements of `type` bytes, no header.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "dmg_internal.h"
#include "dmg_gb300.h"
#include "dmg_io.h"
#include "k1_params.h"
#include "single_decomp.h"

Decomp dmg_makeGlobalDecomp(MPI_Comm comm, int ndim, const int *L) {
  if (!comm || ndim < 1 || !L) {
    dmg_error(DMG_ERR_ARG, "dmg_makeGlobalDecomp: bad arguments");
    return NULL;
  }
  DimDecomp dims[DMG_MAXAX];
  if (ndim > DMG_MAXAX) {
    dmg_error(DMG_ERR_UNSUPPORTED, "dmg_makeGlobalDecomp: %d dimensions", ndim);
    return NULL;
  }
  for (int i = 0; i < ndim; ++i) {
    dims[i] = makeSingleDecomp(L[i], 0, 1);
    if (!dims[i]) {
      for (int j = 0; j < i; ++j) free(dims[j]);
      return NULL;
    }
  }
  Decomp g = makePackedDecomp(comm, ndim, dims);
  return g;
}

static Decomp global_of(Decomp d) {
  int L[DMG_MAXAX];
  for (int i = 0; i < d->ndim; ++i) L[i] = d->dims[i]->decomp->coord_size;
  return dmg_makeGlobalDecomp(d->comm, d->ndim, L);
}

/* one reshape between d and its global layout, run and waited for (the plan
 * and its device tables are freed before returning) */
static int move(Decomp d, MPI_Datatype type, const void *src, void *dst, int to_global, void *stream) {
  if (!d || !src || !dst || type <= 0) return dmg_error(DMG_ERR_ARG, "dmg_io: bad arguments");
  Decomp g = global_of(d);
  if (!g) return dmg_last_error_code() ? dmg_last_error_code() : DMG_ERR_NOMEM;
  ReshapePlan plan = to_global ? makeReshapePlan(d->comm, type, d, g) : makeReshapePlan(d->comm, type, g, d);
  if (!plan) {
    freeDecomp(g);
    return dmg_last_error_code() ? dmg_last_error_code() : dmg_error(DMG_ERR_UNSUPPORTED, "dmg_io: no plan");
  }
  int st = dmg_reshape_run(plan, src, dst, stream);
  if (st == DMG_OK) st = dmg_stream_sync(stream);
  freeReshapePlan(plan);
  freeDecomp(g);
  return st;
}

int dmg_io_gather(Decomp d, MPI_Datatype type, const void *src, void *global, void *stream) {
  return move(d, type, src, global, 1, stream);
}

int dmg_io_scatter(Decomp d, MPI_Datatype type, const void *global, void *dst, void *stream) {
  return move(d, type, global, dst, 0, stream);
}

static long long global_count(Decomp d) {
  long long n = 1;
  for (int i = 0; i < d->ndim; ++i) n *= d->dims[i]->decomp->coord_size;
  return n;
}

int dmg_io_write_file(const char *path, Decomp d, MPI_Datatype type, const void *src, void *stream) {
  if (!path || !d || !src || type <= 0) return dmg_error(DMG_ERR_ARG, "dmg_io_write_file: bad arguments");
  size_t bytes = (size_t)global_count(d) * (size_t)type;
  void *dev = NULL;
  int st = dmg_dev_alloc(&dev, bytes);
  if (st != DMG_OK) return st;
  char *host = (char *)malloc(bytes ? bytes : 1);
  if (!host) {
    dmg_dev_free(dev);
    return dmg_error(DMG_ERR_NOMEM, "dmg_io_write_file: %zu bytes of host memory", bytes);
  }
  st = dmg_io_gather(d, type, src, dev, stream);
  if (st == DMG_OK) st = dmg_copy_sync(host, dev, bytes, 1, stream);
  dmg_dev_free(dev);
  if (st == DMG_OK) {
    FILE *f = fopen(path, "wb");
    if (!f) {
      st = dmg_error(DMG_ERR_ARG, "dmg_io_write_file: cannot open %s", path);
    } else {
      if (fwrite(host, 1, bytes, f) != bytes) st = dmg_error(DMG_ERR_ARG, "dmg_io_write_file: short write to %s", path);
      if (fclose(f) != 0 && st == DMG_OK) st = dmg_error(DMG_ERR_ARG, "dmg_io_write_file: closing %s", path);
    }
  }
  free(host);
  return st;
}

int dmg_io_read_file(const char *path, Decomp d, MPI_Datatype type, void *dst, void *stream) {
  if (!path || !d || !dst || type <= 0) return dmg_error(DMG_ERR_ARG, "dmg_io_read_file: bad arguments");
  size_t bytes = (size_t)global_count(d) * (size_t)type;
  char *host = (char *)malloc(bytes ? bytes : 1);
  if (!host) return dmg_error(DMG_ERR_NOMEM, "dmg_io_read_file: %zu bytes of host memory", bytes);
  FILE *f = fopen(path, "rb");
  if (!f) {
    free(host);
    return dmg_error(DMG_ERR_ARG, "dmg_io_read_file: cannot open %s", path);
  }
  size_t got = fread(host, 1, bytes, f);
  fclose(f);
  if (got != bytes) {
    free(host);
    return dmg_error(DMG_ERR_BOUNDS, "dmg_io_read_file: %s holds %zu bytes, the array needs %zu", path, got, bytes);
  }
  void *dev = NULL;
  int st = dmg_dev_alloc(&dev, bytes);
  if (st == DMG_OK) st = dmg_copy_sync(dev, host, bytes, 0, stream);
  if (st == DMG_OK) st = dmg_io_scatter(d, type, dev, dst, stream);
  dmg_dev_free(dev);
  free(host);
  return st;
}

long long dmg_io_view(Decomp d, int rank, long long *file_off, long long *mem_off, long long max) {
  if (!d || rank < 0) {
    dmg_error(DMG_ERR_ARG, "dmg_io_view: bad arguments");
    return -1;
  }
  int nd = d->ndim;
  int pos[DMG_MAXAX], L[DMG_MAXAX], g[DMG_MAXAX];
  for (int i = 0; i < nd; ++i) {
    pos[i] = dmg_axis_pos(d->dims[i], rank);
    L[i] = d->dims[i]->decomp->coord_size;
    g[i] = 0;
    if (L[i] <= 0) return 0;
  }
  if (!dmg_rank_holds(d, rank)) return 0;
  long long count = 0, lin = 0;
  for (;;) {
    int local = 1;
    long long off = 0;
    for (int i = 0; i < nd && local; ++i) {
      DimDecomp dd = d->dims[i]->decomp;
      if (dd->rank_offset(dd, g[i]) != pos[i]) local = 0;
      else off += dmg_axis_stride(d->dims[i], rank) * (long long)dd->type_offset(dd, g[i]);
    }
    if (local) {
      if (count < max) {
        if (file_off) file_off[count] = lin;
        if (mem_off) mem_off[count] = off;
      }
      count++;
    }
    /* next global coordinate in C order */
    int i = nd - 1;
    while (i >= 0 && ++g[i] == L[i]) g[i--] = 0;
    if (i < 0) break;
    lin++;
  }
  return count;
}
