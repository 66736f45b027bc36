/*
 * TEST INFRASTRUCTURE.  Runs the reference's own reshape and split FFT
 * (its sources compiled unmodified against the project's MPI and FFTW shims,
 * oracle/_ref/libref.so) with the caller-defined block-cyclic plugin of
 * block_cyclic.c on dimension 0, one thread per virtual rank, to make the
 * golden fixture of tests/test_plugin_gpu.py (tests/golden/make_plugin_golden.py
 * compiles this file against the reference's headers).
 *
 * Decompositions on a g0 x g1 grid of L0 x L1 x L2 complex128 values:
 *   src   block(L0, g0) | block(L1, g1) | local(L2)
 *   dest  block_cyclic(L0, b, g0) | block(L1, g1) | local(L2)
 * The reshape moves src to dest; the split FFT (makeSplitPlan, forward)
 * transforms dest.  Every array is a virtual-grid array: rank r at r * pitch.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <mpi.h>
#include "reshape.h"
#include "block_decomp.h"
#include "local_decomp.h"
#include "split_fft.h"

DimDecomp make_block_cyclic(int len, int block, int procs);

typedef struct {
  int g0, g1, L0, L1, L2, b;
  long long src_pitch, dst_pitch, work_len;
  const double *src;
  double *dst, *work;
  long long *slot_map;
  int *extents; /* [P][3]: extent(src), extent(dest), split plan extent */
} plugin_job;

static Decomp build(const plugin_job *j, int cyclic) {
  DimDecomp d[3];
  d[0] = cyclic ? make_block_cyclic(j->L0, j->b, j->g0) : makeBlockDecomp(j->L0, j->g0);
  d[1] = makeBlockDecomp(j->L1, j->g1);
  d[2] = makeLocalDecomp(j->L2);
  return makePackedDecomp(MPI_COMM_WORLD, 3, d);
}

static void plugin_rank(int r, void *arg) {
  plugin_job *j = (plugin_job *)arg;
  Decomp s = build(j, 0), d = build(j, 1);
  if (j->extents) {
    j->extents[3 * r] = extent(s);
    j->extents[3 * r + 1] = extent(d);
  }
  if (j->src) {
    MPI_Datatype base;
    MPI_Type_contiguous(16, MPI_CHAR, &base);
    MPI_Type_commit(&base);
    ReshapePlan plan = makeReshapePlan(MPI_COMM_WORLD, base, s, d);
    runReshapePlan(MPI_COMM_WORLD, plan, (void *)(j->src + 2 * (size_t)r * j->src_pitch),
                   j->dst + 2 * (size_t)r * j->dst_pitch);
    MPI_Barrier(MPI_COMM_WORLD);
    freeReshapePlan(plan);
    MPI_Type_free(&base);
  }
  if (!j->src || !j->work) {
    MPI_Barrier(MPI_COMM_WORLD);
    return;
  }
  fftw_complex *dat = (fftw_complex *)(j->dst + 2 * (size_t)r * j->dst_pitch);
  fftw_complex *work = (fftw_complex *)(j->work + 2 * (size_t)r * j->work_len);
  SplitPlan sp = makeSplitPlan(0, d, dat, (int)j->work_len, work);
  if (j->extents) j->extents[3 * r + 2] = sp ? sp->extent : -1;
  MPI_Barrier(MPI_COMM_WORLD);
  if (sp) {
    runSplitPlan(sp, FFTW_FORWARD);
    MPI_Barrier(MPI_COMM_WORLD);
    /* the global slot each local slot of the output decomposition holds */
    Decomp B = sp->B ? sp->B : sp->A;
    long long *map = j->slot_map + (size_t)r * j->work_len;
    for (long long k = 0; k < j->work_len; ++k) map[k] = -1;
    int L[3] = {j->L0, j->L1, j->L2}, c[3];
    if (r < B->proc_used)
      for (long long g = 0; g < (long long)L[0] * L[1] * L[2]; ++g) {
        c[0] = (int)(g / ((long long)L[1] * L[2]));
        c[1] = (int)((g / L[2]) % L[1]);
        c[2] = (int)(g % L[2]);
        if (!areCoordsLocal(B, c)) continue;
        int off = getOffset(B, c);
        if (off >= 0 && off < j->work_len) map[off] = g;
      }
  }
  MPI_Barrier(MPI_COMM_WORLD);
}

/* extents (optional, [P][3]); with src, dst, work and slot_map the reshape and
 * the forward split FFT */
int plugin_ref_run(int g0, int g1, int L0, int L1, int L2, int b, long long src_pitch, long long dst_pitch,
                   long long work_len, const double *src, double *dst, double *work, long long *slot_map,
                   int *extents, char *err, int errlen) {
  plugin_job j = {g0, g1, L0, L1, L2, b, src_pitch, dst_pitch, work_len, src, dst, work, slot_map, extents};
  int rc = shim_run(g0 * g1, plugin_rank, &j);
  if (rc && err) snprintf(err, errlen, "%s", shim_error());
  return rc;
}
