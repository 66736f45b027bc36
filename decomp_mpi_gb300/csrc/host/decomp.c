/*
 * AxisDecomp and Decomp over a virtual communicator.
 *
 * Semantics follow the reference (reshape.c:47-324): a virtual rank r sits at
 * position (r / rank_stride) % proc_size along each axis; it holds the global
 * coordinates whose rank_offset equals that position, at offset
 * sum(memory_stride * type_offset).  Because one process holds every rank,
 * each AxisDecomp keeps the local facts of every position along its axis and
 * the memory stride of every virtual rank; the reference's own fields are
 * filled for the communicator's view rank.
 */
#include <limits.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "dmg_internal.h"
#include "factor_reverse_decomp.h"

AxisDecomp makeAxisDecomp(MPI_Comm comm, DimDecomp d, int stride, int rank_stride) {
  if (!dmg_comm_ok(comm)) {
    dmg_error(DMG_ERR_ARG, "makeAxisDecomp: invalid communicator");
    return NULL;
  }
  if (!d) {
    dmg_error(DMG_ERR_ARG, "makeAxisDecomp: NULL DimDecomp");
    return NULL;
  }
  int size = comm->size;
  if (rank_stride < 1 || (long long)rank_stride * d->proc_size > size) {
    raise_error(comm, "Illegal rank_stride");
    return NULL;
  }
  if (d->proc_size < 1 || d->coord_size < 1) {
    dmg_error(DMG_ERR_ARG, "makeAxisDecomp: DimDecomp with proc_size=%d coord_size=%d",
              d->proc_size, d->coord_size);
    return NULL;
  }
  AxisDecomp a = (AxisDecomp)calloc(1, sizeof(struct axis_decomp));
  if (!a) {
    dmg_error(DMG_ERR_NOMEM, "makeAxisDecomp: out of memory");
    return NULL;
  }
  int ps = d->proc_size;
  a->decomp = d;
  a->comm = comm;
  a->memory_stride = stride;
  a->rank_stride = rank_stride;
  a->rank_memory_stride = NULL;
  a->pos_n_local = (int *)calloc((size_t)ps, sizeof(int));
  a->pos_max_local = (int *)calloc((size_t)ps, sizeof(int));
  a->pos_index = (Index *)calloc((size_t)ps + 1, sizeof(Index));
  if (!a->pos_n_local || !a->pos_max_local || !a->pos_index) {
    freeAxisDecomp(a);
    dmg_error(DMG_ERR_NOMEM, "makeAxisDecomp: out of memory");
    return NULL;
  }
  for (int p = 0; p < ps; ++p) a->pos_index[p] = makeIndex();
  /* One pass over the axis: each coordinate goes to the position its
   * rank_offset names; a position outside [0, proc_size) holds nothing. */
  for (int g = 0; g < d->coord_size; ++g) {
    int p = d->rank_offset(d, g);
    if (p < 0 || p >= ps) continue;
    int off = d->type_offset(d, g);
    a->pos_n_local[p]++;
    if (off > a->pos_max_local[p]) a->pos_max_local[p] = off;
    addIndex(a->pos_index[p], off);
  }
  int view = comm->rank;
  a->my_rank_in_dimension = (view / rank_stride) % ps;
  a->n_local = a->pos_n_local[a->my_rank_in_dimension];
  a->max_local = a->pos_max_local[a->my_rank_in_dimension];
  a->index = a->pos_index[a->my_rank_in_dimension];
  return a;
}

void freeAxisDecomp(AxisDecomp a) {
  if (!a) return;
  if (a->pos_index) {
    for (int p = 0; a->decomp && p < a->decomp->proc_size; ++p) freeIndex(a->pos_index[p]);
    free(a->pos_index);
  }
  free(a->pos_n_local);
  free(a->pos_max_local);
  free(a->rank_memory_stride);
  freeDimDecomp(a->decomp);
  free(a);
}

void describeAxisDecomp(FILE *out, AxisDecomp a) {
  fprintf(out, "AxisDecomp: mem_stride=%d rank_stride=%d ", a->memory_stride, a->rank_stride);
  describeDimDecomp(out, a->decomp);
}

int isLocal(AxisDecomp a, int global) {
  return a->my_rank_in_dimension == a->decomp->rank_offset(a->decomp, global);
}

Index *makeIndexList(AxisDecomp mine, DimDecomp remote) {
  if (mine->decomp->coord_size != remote->coord_size) {
    raise_error(mine->comm, "non-conformant sizes in makeIndexList %d!=%d",
                mine->decomp->coord_size, remote->coord_size);
    return NULL;
  }
  int n = remote->proc_size;
  Index *list = (Index *)calloc((size_t)n + 1, sizeof(Index));
  for (int p = 0; p < n; ++p) list[p] = makeIndex();
  for (int g = 0; g < mine->decomp->coord_size; ++g) {
    if (!isLocal(mine, g)) continue;
    int p = remote->rank_offset(remote, g);
    if (p < 0 || p >= n) continue;
    addIndex(list[p], mine->decomp->type_offset(mine->decomp, g));
  }
  return list;
}

Index makeGlobalIndex(AxisDecomp mine) {
  Index ix = makeIndex();
  for (int g = 0; g < mine->decomp->coord_size; ++g)
    if (isLocal(mine, g)) addIndex(ix, g);
  return ix;
}

Decomp makeDecomp(int ndim, AxisDecomp dims[]) {
  if (ndim < 1 || !dims) {
    dmg_error(DMG_ERR_ARG, "makeDecomp: ndim=%d", ndim);
    return NULL;
  }
  for (int i = 0; i < ndim; ++i) {
    if (!dims[i]) {
      dmg_error(DMG_ERR_ARG, "makeDecomp: axis %d is NULL", i);
      return NULL;
    }
  }
  MPI_Comm comm = dims[0]->comm;
  /* every axis must share one communicator (the reference compares
   * dims[0] with dims[1] ndim-1 times, reshape.c:186-191) */
  for (int i = 1; i < ndim; ++i) {
    if (dims[i]->comm != comm) {
      raise_error(comm, "Different communicators in Decomp");
      return NULL;
    }
  }
  long long maxrank = 0;
  for (int i = 0; i < ndim; ++i)
    maxrank += (long long)dims[i]->rank_stride * (dims[i]->decomp->proc_size - 1);
  if (maxrank >= comm->size) {
    raise_error(comm, "Maximum processor rank out of range max=%lld size=%d", maxrank, comm->size);
    return NULL;
  }
  for (int i = 0; i < ndim; ++i) {
    for (int j = i + 1; j < ndim; ++j) {
      if (dims[i]->decomp->proc_size > 1 && dims[j]->decomp->proc_size > 1 &&
          dims[i]->rank_stride > 1 && dims[j]->rank_stride > 1 &&
          dims[i]->rank_stride == dims[j]->rank_stride) {
        raise_error(comm, "duplicate rank strides dim=%d rank_stride=%d, dim=%d rank_stride=%d", i,
                    dims[i]->rank_stride, j, dims[j]->rank_stride);
        return NULL;
      }
    }
  }
  Decomp d = (Decomp)calloc(1, sizeof(struct decomp));
  if (!d) return NULL;
  d->ndim = ndim;
  d->comm = comm;
  d->proc_used = (int)maxrank + 1;
  d->dims = (AxisDecomp *)calloc((size_t)ndim, sizeof(AxisDecomp));
  memcpy(d->dims, dims, (size_t)ndim * sizeof(AxisDecomp));
  return d;
}

Decomp makePackedDecomp(MPI_Comm comm, int ndim, DimDecomp dims[]) {
  if (!dmg_comm_ok(comm) || ndim < 1 || !dims) {
    dmg_error(DMG_ERR_ARG, "makePackedDecomp: bad arguments");
    return NULL;
  }
  AxisDecomp *axes = (AxisDecomp *)calloc((size_t)ndim, sizeof(AxisDecomp));
  int rank_stride = 1;
  int ok = 1;
  /* last dimension fastest; rank strides are the running product of
   * proc_size (reference reshape.c:228-236) */
  for (int i = ndim - 1; i >= 0 && ok; --i) {
    if (!dims[i]) {
      dmg_error(DMG_ERR_ARG, "makePackedDecomp: DimDecomp %d is NULL", i);
      ok = 0;
      break;
    }
    axes[i] = makeAxisDecomp(comm, dims[i], 1, rank_stride);
    if (!axes[i]) {
      ok = 0;
      break;
    }
    rank_stride *= dims[i]->proc_size;
  }
  if (ok) {
    /* memory strides per virtual rank: the product of (max_local+1) of the
     * later dimensions at that rank's positions */
    int P = comm->size;
    long long *st = (long long *)calloc((size_t)P * ndim, sizeof(long long));
    for (int r = 0; r < P; ++r) {
      long long s = 1;
      for (int i = ndim - 1; i >= 0; --i) {
        st[(size_t)i * P + r] = s;
        s *= (long long)axes[i]->pos_max_local[dmg_axis_pos(axes[i], r)] + 1;
      }
    }
    int view = comm->rank;
    for (int i = 0; i < ndim && ok; ++i) {
      long long *row = st + (size_t)i * P;
      int uniform = 1;
      for (int r = 1; r < P; ++r) uniform &= (row[r] == row[0]);
      if (row[view] > INT_MAX) {
        dmg_error(DMG_ERR_UNSUPPORTED, "makePackedDecomp: stride %lld exceeds int", row[view]);
        ok = 0;
        break;
      }
      axes[i]->memory_stride = (int)row[view];
      if (!uniform) {
        axes[i]->rank_memory_stride = (long long *)malloc((size_t)P * sizeof(long long));
        memcpy(axes[i]->rank_memory_stride, row, (size_t)P * sizeof(long long));
      }
    }
    free(st);
  }
  Decomp d = ok ? makeDecomp(ndim, axes) : NULL;
  if (!d) {
    for (int i = 0; i < ndim; ++i) {
      if (axes[i]) freeAxisDecomp(axes[i]);
      else if (!ok && dims[i]) {
        /* axes not yet built still own nothing; the caller's DimDecomp is
         * consumed as in the reference */
        freeDimDecomp(dims[i]);
      }
    }
  }
  free(axes);
  return d;
}

void freeDecomp(Decomp d) {
  if (!d) return;
  for (int i = 0; i < d->ndim; ++i) freeAxisDecomp(d->dims[i]);
  free(d->dims);
  free(d);
}

void describeDecomp(FILE *out, Decomp d) {
  fprintf(out, "Decomp ndim=%d procs_used=%d\n", d->ndim, d->proc_used);
  for (int i = 0; i < d->ndim; ++i) {
    describeAxisDecomp(out, d->dims[i]);
    fprintf(out, "\n");
  }
}
void describeDeomp(FILE *out, Decomp d) { describeDecomp(out, d); }

int dmg_rank_holds(Decomp d, int r) {
  for (int i = 0; i < d->ndim; ++i) {
    AxisDecomp a = d->dims[i];
    if (a->pos_n_local[dmg_axis_pos(a, r)] == 0) return 0;
  }
  return 1;
}

long long rankExtent64(Decomp d, int r) {
  long long e = 1;
  for (int i = 0; i < d->ndim; ++i) {
    AxisDecomp a = d->dims[i];
    e += dmg_axis_stride(a, r) * a->pos_max_local[dmg_axis_pos(a, r)];
  }
  return e;
}

long long extent64(Decomp d) {
  long long best = 1;
  for (int r = 0; r < d->proc_used; ++r) {
    long long e = rankExtent64(d, r);
    if (e > best) best = e;
  }
  return best;
}

int extent(Decomp d) {
  long long e = extent64(d);
  if (e > INT_MAX) {
    dmg_error(DMG_ERR_UNSUPPORTED, "extent %lld does not fit in int; use extent64", e);
    return -1;
  }
  return (int)e;
}

int compatible(Decomp a, Decomp b) {
  if (a->ndim != b->ndim) return NOT_COMPATIBLE;
  if (a->comm != b->comm) return NOT_COMPATIBLE;
  for (int i = 0; i < a->ndim; ++i)
    if (sizeDimDecomp(a->dims[i]->decomp) != sizeDimDecomp(b->dims[i]->decomp)) return NOT_COMPATIBLE;
  return COMPATIBLE;
}

int myRank(Decomp d) {
  int r = 0;
  for (int i = 0; i < d->ndim; ++i) r += d->dims[i]->my_rank_in_dimension * d->dims[i]->rank_stride;
  return r;
}

int isCoordLocal(Decomp d, int dim, int pos) { return isLocal(d->dims[dim], pos); }

int areCoordsLocal(Decomp d, int *pos) {
  for (int i = 0; i < d->ndim; ++i)
    if (!isLocal(d->dims[i], pos[i])) return 0;
  return 1;
}

int getOffset(Decomp d, int *pos) {
  int off = 0;
  for (int i = 0; i < d->ndim; ++i) {
    DimDecomp dd = d->dims[i]->decomp;
    off += d->dims[i]->memory_stride * dd->type_offset(dd, pos[i]);
  }
  return off;
}

int ownerRank(Decomp d, int *pos) {
  long long r = 0;
  for (int i = 0; i < d->ndim; ++i) {
    DimDecomp dd = d->dims[i]->decomp;
    int p = dd->rank_offset(dd, pos[i]);
    if (p < 0 || p >= dd->proc_size) return -1;
    r += (long long)d->dims[i]->rank_stride * p;
  }
  if (r >= d->proc_used) return -1;
  for (int i = 0; i < d->ndim; ++i) {
    DimDecomp dd = d->dims[i]->decomp;
    if (dmg_axis_pos(d->dims[i], (int)r) != dd->rank_offset(dd, pos[i])) return -1;
  }
  return (int)r;
}

long long globalOffset64(Decomp d, int *pos, long long pitch) {
  int r = ownerRank(d, pos);
  if (r < 0) return -1;
  long long off = (long long)r * pitch;
  for (int i = 0; i < d->ndim; ++i) {
    DimDecomp dd = d->dims[i]->decomp;
    off += dmg_axis_stride(d->dims[i], r) * dd->type_offset(dd, pos[i]);
  }
  return off;
}

void dmg_sort_order(int ndim, int *order, Decomp src, int r) {
  for (int i = 0; i < ndim; ++i) order[i] = ndim - 1 - i;
  for (int i = 0; i < ndim - 1; ++i) {
    for (int j = i + 1; j < ndim; ++j) {
      if (dmg_axis_stride(src->dims[order[j]], r) < dmg_axis_stride(src->dims[order[i]], r)) {
        int t = order[i];
        order[i] = order[j];
        order[j] = t;
      }
    }
  }
}

AxisDecomp makeFactorReverseAxisDecomp(int A, int B, AxisDecomp orig) {
  DimDecomp fr = makeFactorReverseDecomp(A, B, orig->decomp);
  if (!fr) {
    dmg_error(DMG_ERR_ARG, "makeFactorReverseAxisDecomp: A*B=%d*%d != %d", A, B,
              orig->decomp->coord_size);
    return NULL;
  }
  AxisDecomp a = makeAxisDecomp(orig->comm, fr, orig->memory_stride, orig->rank_stride);
  if (a && orig->rank_memory_stride) {
    size_t n = (size_t)orig->comm->size;
    a->rank_memory_stride = (long long *)malloc(n * sizeof(long long));
    memcpy(a->rank_memory_stride, orig->rank_memory_stride, n * sizeof(long long));
  }
  return a;
}
