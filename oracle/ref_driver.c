/*
 * TEST INFRASTRUCTURE (oracle).  Drives the reference library, compiled
 * unmodified from its own sources against the project's MPI and FFTW shims,
 * with one thread per MPI rank.  Built into oracle/_ref/libref.so by
 * oracle/Makefile; used only to pin the oracle restatement and to generate
 * the golden fixtures under tests/golden/.
 *
 * Every buffer argument is a virtual-grid array: rank r's local buffer
 * starts at element r * pitch.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <mpi.h>
#include "reshape.h"
#include "block_decomp.h"
#include "interleave_decomp.h"
#include "rotate_decomp.h"
#include "factor_reverse_decomp.h"
#include "single_decomp.h"
#include "local_decomp.h"
#include "split_fft.h"
#include "processor_grid.h"
#include "spec.h"

static DimDecomp build_dim(const spec_dim *d) {
  DimDecomp n, r;
  switch (d->kind) {
    case SK_BLOCK: return makeBlockDecomp(d->v[0], d->v[1]);
    case SK_BLOCKF: return makeBlockDecompWithFactor(d->v[0], d->v[1], d->v[2]);
    case SK_LOCAL: return makeLocalDecomp(d->v[0]);
    case SK_SINGLE: return makeSingleDecomp(d->v[0], d->v[1], d->v[2]);
    case SK_ROTATE:
      n = build_dim(d->nested);
      r = makeRotatedDecomp(d->v[0], n);
      freeDimDecomp(n);
      return r;
    case SK_INTERLEAVE:
      n = build_dim(d->nested);
      r = makeInterleaveDecomp(n, d->v[0]);
      return r; /* the reference's interleave destroy frees no nested decomp */
    case SK_FREV:
      n = build_dim(d->nested);
      r = makeFactorReverseDecomp(d->v[0], d->v[1], n);
      freeDimDecomp(n);
      return r;
  }
  return NULL;
}

static Decomp build_decomp(const char *spec) {
  spec_decomp sd;
  if (spec_parse(spec, &sd) != 0) {
    fprintf(stderr, "ref_driver: bad spec %s\n", spec);
    MPI_Abort(MPI_COMM_WORLD, 1);
  }
  Decomp d;
  if (sd.packed) {
    DimDecomp dims[SPEC_MAXD];
    for (int i = 0; i < sd.ndim; ++i) dims[i] = build_dim(sd.dims[i]);
    d = makePackedDecomp(MPI_COMM_WORLD, sd.ndim, dims);
  } else {
    AxisDecomp axes[SPEC_MAXD];
    for (int i = 0; i < sd.ndim; ++i)
      axes[i] = makeAxisDecomp(MPI_COMM_WORLD, build_dim(sd.dims[i]), sd.stride[i], sd.rank_stride[i]);
    d = makeDecomp(sd.ndim, axes);
  }
  spec_free(&sd);
  return d;
}

/* ---- reshape ---- */

typedef struct {
  const char *src_spec, *dst_spec;
  int esize;
  long long src_pitch, dst_pitch;
  const char *src;
  char *dst;
  int *extents; /* [P][2] */
  int *proc_used; /* [2] */
} reshape_job;

static void reshape_rank(int r, void *arg) {
  reshape_job *j = (reshape_job *)arg;
  Decomp s = build_decomp(j->src_spec);
  Decomp d = build_decomp(j->dst_spec);
  MPI_Datatype base;
  MPI_Type_contiguous(j->esize, MPI_CHAR, &base);
  MPI_Type_commit(&base);
  if (j->extents) {
    j->extents[2 * r] = extent(s);
    j->extents[2 * r + 1] = extent(d);
  }
  if (j->proc_used && r == 0) {
    j->proc_used[0] = s->proc_used;
    j->proc_used[1] = d->proc_used;
  }
  ReshapePlan plan = makeReshapePlan(MPI_COMM_WORLD, base, s, d);
  if (j->src && j->dst) {
    runReshapePlan(MPI_COMM_WORLD, plan, (void *)(j->src + (size_t)r * j->src_pitch * j->esize),
                   j->dst + (size_t)r * j->dst_pitch * j->esize);
  }
  MPI_Barrier(MPI_COMM_WORLD);
  freeReshapePlan(plan);
  MPI_Type_free(&base);
}

/* Run the reference reshape on P thread-ranks.  extents (optional, [P][2])
 * receives each rank's extent(src), extent(dst).  Returns 0 on success. */
int ref_reshape(int P, const char *src_spec, const char *dst_spec, int esize, long long src_pitch,
                long long dst_pitch, const void *src_all, void *dst_all, int *extents, int *proc_used, char *err,
                int errlen) {
  reshape_job j = {src_spec, dst_spec, esize, src_pitch, dst_pitch, (const char *)src_all, (char *)dst_all,
                   extents, proc_used};
  int rc = shim_run(P, reshape_rank, &j);
  if (rc && err) snprintf(err, errlen, "%s", shim_error());
  return rc;
}

/* ---- processor grid ---- */

int ref_processor_grid(int P, int ndim, const int *tasks, int *grid_out) {
  shim_set_self(0, P);
  int t[16];
  for (int i = 0; i < ndim; ++i) t[i] = tasks[i];
  int *g = makeProcessorGrid(MPI_COMM_WORLD, ndim, t);
  for (int i = 0; i < ndim; ++i) grid_out[i] = g[i];
  free(g);
  return 0;
}

/* ---- split FFT ---- */

typedef struct {
  const char *start_spec;
  int mode; /* 0: makeSplitPlan(slab=0), 1: makeSplitPlan(slab=1), 2: makeParallelPlan(B) */
  const int *B;
  long long dat_pitch, work_len;
  double *dat, *work;
  int *info;           /* per rank: [extent, A0..A(n-1), ok] */
  long long *slot_map; /* per rank, work_len entries: global slot index of each B-layout slot, -1 none */
  int direction_back;  /* also run the (reference) backward transform */
} split_job;

#define INFO_W 8

static void split_rank(int r, void *arg) {
  split_job *j = (split_job *)arg;
  Decomp start = build_decomp(j->start_spec);
  fftw_complex *dat = (fftw_complex *)(j->dat + 2 * (size_t)r * j->dat_pitch);
  fftw_complex *work = (fftw_complex *)(j->work + 2 * (size_t)r * j->work_len);
  SplitPlan plan = NULL;
  if (j->mode == 2) plan = makeParallelPlan(start, (int *)j->B, dat, (int)j->work_len, work);
  else plan = makeSplitPlan(j->mode, start, dat, (int)j->work_len, work);
  int *info = j->info + (size_t)r * INFO_W;
  if (!plan) {
    info[INFO_W - 1] = 0;
    MPI_Barrier(MPI_COMM_WORLD);
    return;
  }
  info[0] = plan->extent;
  for (int i = 0; i < start->ndim && i < INFO_W - 2; ++i) info[1 + i] = plan->A_factors[i];
  info[INFO_W - 1] = 1;
  MPI_Barrier(MPI_COMM_WORLD);
  runSplitPlan(plan, FFTW_FORWARD);
  MPI_Barrier(MPI_COMM_WORLD);
  if (j->slot_map) {
    /* where each global slot of the output decomposition lives on this rank */
    Decomp B = plan->B ? plan->B : plan->A;
    long long *map = j->slot_map + (size_t)r * j->work_len;
    for (long long k = 0; k < j->work_len; ++k) map[k] = -1;
    int nd = B->ndim;
    int L[16], c[16];
    long long total = 1;
    for (int i = 0; i < nd; ++i) {
      L[i] = B->dims[i]->decomp->coord_size;
      total *= L[i];
    }
    if (r < B->proc_used) {
      for (long long g = 0; g < total; ++g) {
        long long rem = g;
        for (int i = nd - 1; i >= 0; --i) {
          c[i] = (int)(rem % L[i]);
          rem /= L[i];
        }
        if (!areCoordsLocal(B, c)) continue;
        int off = getOffset(B, c);
        if (off >= 0 && off < j->work_len) map[off] = g;
      }
    }
  }
  if (j->direction_back) runSplitPlan(plan, FFTW_BACKWARD);
  MPI_Barrier(MPI_COMM_WORLD);
}

int ref_split(int P, const char *start_spec, int mode, const int *B, long long dat_pitch, long long work_len,
              double *dat_all, double *work_all, int *info, long long *slot_map, int run_back, char *err,
              int errlen) {
  split_job j = {start_spec, mode, B, dat_pitch, work_len, dat_all, work_all, info, slot_map, run_back};
  int rc = shim_run(P, split_rank, &j);
  if (rc && err) snprintf(err, errlen, "%s", shim_error());
  return rc;
}

/* ---- timing of the benchmark step (calibration of the CPU port against the reference itself) ---- */

#include <time.h>

typedef struct {
  const char *s0, *s1, *s2; /* block, rotate, factor_reverse */
  long long p0, p1, p2, work_len;
  double *a0, *a1, *a2, *work;
  int warmup, steps;
  double seconds; /* rank 0: wall time of the timed steps */
} step_job;

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec + 1e-9 * t.tv_nsec;
}

static void step_rank(int r, void *arg) {
  step_job *j = (step_job *)arg;
  Decomp d0 = build_decomp(j->s0), d1 = build_decomp(j->s1), d2 = build_decomp(j->s2);
  MPI_Datatype base;
  MPI_Type_contiguous(16, MPI_CHAR, &base);
  MPI_Type_commit(&base);
  ReshapePlan r01 = makeReshapePlan(MPI_COMM_WORLD, base, d0, d1);
  ReshapePlan r12 = makeReshapePlan(MPI_COMM_WORLD, base, d1, d2);
  double *a0 = j->a0 + 2 * (size_t)r * j->p0, *a1 = j->a1 + 2 * (size_t)r * j->p1;
  fftw_complex *a2 = (fftw_complex *)(j->a2 + 2 * (size_t)r * j->p2);
  fftw_complex *work = (fftw_complex *)(j->work + 2 * (size_t)r * j->work_len);
  SplitPlan plan = makeSplitPlan(0, d2, a2, (int)j->work_len, work);
  double t0 = 0;
  for (int s = 0; s < j->warmup + j->steps; ++s) {
    if (s == j->warmup) {
      MPI_Barrier(MPI_COMM_WORLD);
      t0 = now_s();
    }
    runReshapePlan(MPI_COMM_WORLD, r01, a0, a1);
    runReshapePlan(MPI_COMM_WORLD, r12, a1, a2);
    if (plan) {
      runSplitPlan(plan, FFTW_FORWARD);
      runSplitPlan(plan, FFTW_BACKWARD);
    }
  }
  MPI_Barrier(MPI_COMM_WORLD);
  if (r == 0) j->seconds = now_s() - t0;
  freeReshapePlan(r01);
  freeReshapePlan(r12);
  MPI_Type_free(&base);
}

/* The benchmark step (two reshapes, the split FFT forward and backward) with
 * the reference's own code on P thread-ranks: `steps` timed steps after
 * `warmup`; returns their wall time in *seconds.  The arrays are whole
 * virtual-grid arrays (rank r at r * pitch complex values). */
int ref_time_step(int P, const char *s0, const char *s1, const char *s2, long long p0, long long p1, long long p2,
                  long long work_len, double *a0, double *a1, double *a2, double *work, int warmup, int steps,
                  double *seconds, char *err, int errlen) {
  step_job j = {s0, s1, s2, p0, p1, p2, work_len, a0, a1, a2, work, warmup, steps, 0.0};
  int rc = shim_run(P, step_rank, &j);
  if (rc && err) snprintf(err, errlen, "%s", shim_error());
  *seconds = j.seconds;
  return rc;
}
