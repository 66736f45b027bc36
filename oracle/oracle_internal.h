/*
 * TEST INFRASTRUCTURE (oracle).  Decomposition model shared by the oracle's
 * reshape and split-FFT restatements.
 */
#ifndef ORACLE_INTERNAL_H
#define ORACLE_INTERNAL_H
#include "spec.h"

typedef struct {
  int P;          /* communicator size */
  int ndim;
  int proc_used;  /* 1 + sum rank_stride*(proc_size-1) (reshape.c:181-200) */
  spec_decomp sd;
  int L[SPEC_MAXD], ps[SPEC_MAXD], rs[SPEC_MAXD];
  int *pos_max[SPEC_MAXD]; /* [ps] largest local offset per position (0 when none) */
  int *pos_n[SPEC_MAXD];   /* [ps] local points per position */
  long long *stride[SPEC_MAXD]; /* [P] memory stride of each rank */
} odecomp;

int o_coord_size(const spec_dim *d);
int o_proc_size(const spec_dim *d);
int o_rank_offset(const spec_dim *d, int g);
int o_type_offset(const spec_dim *d, int g);

/* Build from a spec over P ranks; returns 0 on success. */
int od_build(odecomp *od, int P, const char *spec);
void od_free(odecomp *od);
static inline int od_pos(const odecomp *od, int i, int r) { return (r / od->rs[i]) % od->ps[i]; }
static inline int od_local(const odecomp *od, int i, int r, int g) {
  return od_pos(od, i, r) == o_rank_offset(od->sd.dims[i], g);
}
long long od_extent(const odecomp *od, int r);
long long od_max_extent(const odecomp *od);
/* sortOrder restated (reshape.c:330-350) with rank r's src strides */
void od_sort_order(const odecomp *src, int r, int *order);

/* Reshape plan: per rank send and receive typemaps (element offsets). */
typedef struct {
  int peer;
  long long n;
  long long *off;
} omsg;
typedef struct {
  int nmsg, cap;
  omsg *m;
} omsglist;
typedef struct {
  int P;
  int esize;
  omsglist *sends, *recvs; /* [P] */
  int src_used, dst_used;
} oplan;

int oplan_build(oplan *pl, const odecomp *src, const odecomp *dst, int esize);
/* Execute with pack/unpack through a message buffer; 0 on success. */
int oplan_run(const oplan *pl, const char *src, long long src_pitch, char *dst, long long dst_pitch, int nthreads);
/* Same with optional per-rank element offsets of each rank's buffer. */
int oplan_run_based(const oplan *pl, const char *src, long long src_pitch, const long long *src_base, char *dst,
                    long long dst_pitch, const long long *dst_base, int nthreads);
void oplan_free(oplan *pl);

#endif
