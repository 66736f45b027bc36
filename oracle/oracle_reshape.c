/*
 * TEST INFRASTRUCTURE (oracle).  CPU restatement of the reference's
 * decompositions and reshape.  The product never links this file.
 *
 * Each function follows the reference step it names.  The reshape keeps the
 * reference's message structure: every rank builds, for every peer, the
 * ordered list of element offsets its MPI datatype would describe, and a
 * run packs each sender's list into a message buffer and unpacks it through
 * the receiver's list, as MPI's datatype engine does.
 */
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"
#include "oracle_internal.h"

/* ---- per-axis maps ---- */

int o_coord_size(const spec_dim *d) {
  switch (d->kind) {
    case SK_BLOCK:
    case SK_BLOCKF:
    case SK_LOCAL:
    case SK_SINGLE: return d->v[0];
    case SK_ROTATE:
    case SK_FREV: return o_coord_size(d->nested);
    case SK_INTERLEAVE: return o_coord_size(d->nested) * d->v[0]; /* interleave_decomp.c:44-46 */
  }
  return 0;
}

int o_proc_size(const spec_dim *d) {
  switch (d->kind) {
    case SK_BLOCK: return d->v[1];
    case SK_BLOCKF: return d->v[2];
    case SK_LOCAL: return 1;
    case SK_SINGLE: return d->v[2];
    default: return o_proc_size(d->nested);
  }
}

/* block size: factor * ceil((len/factor)/procs) (block_decomp.c:50) */
static int o_blocksize(const spec_dim *d) {
  int len = d->v[0], f = d->kind == SK_BLOCKF ? d->v[1] : 1, p = d->kind == SK_BLOCKF ? d->v[2] : d->v[1];
  return f * (((len / f) + p - 1) / p);
}

/* decorator coordinate maps */
static int o_inner_coord(const spec_dim *d, int g) {
  if (d->kind == SK_ROTATE) { /* rotate_decomp.c:28-33 */
    int len = o_coord_size(d);
    return (g + len + d->v[0]) % len;
  }
  /* factor_reverse: z + B*y with y = g % A, z = g / A (factor_reverse_decomp.c:27-34) */
  return g / d->v[0] + d->v[1] * (g % d->v[0]);
}

int o_rank_offset(const spec_dim *d, int g) {
  switch (d->kind) {
    case SK_BLOCK:
    case SK_BLOCKF: return g / o_blocksize(d); /* block_decomp.c:6-9 */
    case SK_LOCAL: return 0;                   /* local_decomp.c:6-8 */
    case SK_SINGLE: return d->v[1];            /* single_decomp.c:6-9 */
    case SK_INTERLEAVE: {                      /* interleave_decomp.c:6-12 */
      int A = o_coord_size(d->nested);
      return o_rank_offset(d->nested, g % A);
    }
    default: return o_rank_offset(d->nested, o_inner_coord(d, g));
  }
}

int o_type_offset(const spec_dim *d, int g) {
  switch (d->kind) {
    case SK_BLOCK:
    case SK_BLOCKF: return g % o_blocksize(d); /* block_decomp.c:10-13 */
    case SK_LOCAL:
    case SK_SINGLE: return g;
    case SK_INTERLEAVE: { /* interleave_decomp.c:13-20 */
      int A = o_coord_size(d->nested);
      return g / A + d->v[0] * o_type_offset(d->nested, g % A);
    }
    default: return o_type_offset(d->nested, o_inner_coord(d, g));
  }
}

/* ---- decompositions ---- */

int od_build(odecomp *od, int P, const char *spec) {
  memset(od, 0, sizeof(*od));
  if (spec_parse(spec, &od->sd) != 0) return -1;
  od->P = P;
  od->ndim = od->sd.ndim;
  int rank_stride = 1;
  /* makePackedDecomp assigns rank strides from the last dim (reshape.c:228-236) */
  for (int i = od->ndim - 1; i >= 0; --i) {
    const spec_dim *d = od->sd.dims[i];
    od->L[i] = o_coord_size(d);
    od->ps[i] = o_proc_size(d);
    if (od->sd.packed) {
      od->rs[i] = rank_stride;
      rank_stride *= od->ps[i];
    } else {
      od->rs[i] = od->sd.rank_stride[i];
    }
  }
  long long maxr = 0;
  for (int i = 0; i < od->ndim; ++i) {
    if (od->rs[i] < 1 || (long long)od->rs[i] * od->ps[i] > P) return -2; /* reshape.c:60-62 */
    maxr += (long long)od->rs[i] * (od->ps[i] - 1);
    od->pos_max[i] = (int *)calloc(od->ps[i], sizeof(int));
    od->pos_n[i] = (int *)calloc(od->ps[i], sizeof(int));
    /* makeAxisDecomp's scan (reshape.c:72-87), for every position at once */
    for (int g = 0; g < od->L[i]; ++g) {
      int p = o_rank_offset(od->sd.dims[i], g);
      if (p < 0 || p >= od->ps[i]) continue;
      int off = o_type_offset(od->sd.dims[i], g);
      od->pos_n[i][p]++;
      if (off > od->pos_max[i][p]) od->pos_max[i][p] = off;
    }
  }
  if (maxr >= P) return -3; /* reshape.c:197-200 */
  od->proc_used = (int)maxr + 1;
  for (int i = 0; i < od->ndim; ++i) od->stride[i] = (long long *)calloc(P, sizeof(long long));
  for (int r = 0; r < P; ++r) {
    long long s = 1;
    for (int i = od->ndim - 1; i >= 0; --i) {
      if (od->sd.packed) {
        od->stride[i][r] = s; /* reshape.c:233-234 */
        s *= od->pos_max[i][od_pos(od, i, r)] + 1;
      } else {
        od->stride[i][r] = od->sd.stride[i];
      }
    }
  }
  return 0;
}

void od_free(odecomp *od) {
  for (int i = 0; i < od->ndim; ++i) {
    free(od->pos_max[i]);
    free(od->pos_n[i]);
    free(od->stride[i]);
  }
  spec_free(&od->sd);
  memset(od, 0, sizeof(*od));
}

long long od_extent(const odecomp *od, int r) { /* reshape.c:317-324 */
  long long e = 1;
  for (int i = 0; i < od->ndim; ++i) e += od->stride[i][r] * od->pos_max[i][od_pos(od, i, r)];
  return e;
}

long long od_max_extent(const odecomp *od) {
  long long m = 1;
  for (int r = 0; r < od->proc_used; ++r) {
    long long e = od_extent(od, r);
    if (e > m) m = e;
  }
  return m;
}

void od_sort_order(const odecomp *src, int r, int *order) {
  int n = src->ndim;
  for (int i = 0; i < n; ++i) order[i] = n - 1 - i;
  for (int i = 0; i < n - 1; ++i)
    for (int j = i + 1; j < n; ++j)
      if (src->stride[order[j]][r] < src->stride[order[i]][r]) {
        int t = order[j];
        order[j] = order[i];
        order[i] = t;
      }
}

/* ---- reshape plan ---- */

static void ml_add(omsglist *l, int peer, long long n, long long *off) {
  if (l->nmsg == l->cap) {
    l->cap = l->cap ? 2 * l->cap : 8;
    l->m = (omsg *)realloc(l->m, l->cap * sizeof(omsg));
  }
  l->m[l->nmsg].peer = peer;
  l->m[l->nmsg].n = n;
  l->m[l->nmsg].off = off;
  l->nmsg++;
}

static void ml_free(omsglist *l) {
  for (int k = 0; k < l->nmsg; ++k) free(l->m[k].off);
  free(l->m);
  memset(l, 0, sizeof(*l));
}

/* expandList (typelist.c:108-119) for rank r along dim i: each entry splits
 * into one entry per remote position whose index list is non-empty
 * (makeIndexList, reshape.c:104-136); the new typemap is, for each local
 * offset o of the list in coordinate order, a copy of the old typemap
 * displaced by o * stride (expandEntry, typelist.c:74-106).  Entries whose
 * new rank reaches max_proc are dropped (typelist.c:93-99). */
static omsglist expand(const omsglist *in, const odecomp *mine, const odecomp *remote, int i, int r,
                       int max_proc) {
  omsglist out = {0, 0, NULL};
  int rps = remote->ps[i];
  long long *cnt = (long long *)calloc(rps, sizeof(long long));
  int L = mine->L[i];
  int *rpos = (int *)malloc(L * sizeof(int));
  int *loff = (int *)malloc(L * sizeof(int));
  for (int g = 0; g < L; ++g) {
    rpos[g] = -1;
    if (!od_local(mine, i, r, g)) continue;
    int p = o_rank_offset(remote->sd.dims[i], g);
    if (p < 0 || p >= rps) continue;
    rpos[g] = p;
    loff[g] = o_type_offset(mine->sd.dims[i], g);
    cnt[p]++;
  }
  long long st = mine->stride[i][r];
  for (int e = 0; e < in->nmsg; ++e) {
    const omsg *m = &in->m[e];
    for (int p = 0; p < rps; ++p) {
      if (cnt[p] == 0) continue;
      int nr = m->peer + p * remote->rs[i];
      if (nr >= max_proc) continue;
      long long n = cnt[p] * m->n;
      long long *off = (long long *)malloc((n ? n : 1) * sizeof(long long));
      long long k = 0;
      for (int g = 0; g < L; ++g) {
        if (rpos[g] != p) continue;
        long long base = (long long)loff[g] * st;
        for (long long x = 0; x < m->n; ++x) off[k++] = base + m->off[x];
      }
      ml_add(&out, nr, n, off);
    }
  }
  free(cnt);
  free(rpos);
  free(loff);
  return out;
}

static omsglist build_list(const odecomp *mine, const odecomp *remote, const odecomp *src, int r, int max_proc) {
  omsglist l = {0, 0, NULL};
  long long *z = (long long *)malloc(sizeof(long long));
  z[0] = 0;
  ml_add(&l, 0, 1, z); /* (rank 0, base type) seed, reshape.c:376-387 */
  int order[SPEC_MAXD];
  od_sort_order(src, r, order);
  for (int j = 0; j < mine->ndim; ++j) {
    omsglist nl = expand(&l, mine, remote, order[j], r, max_proc);
    ml_free(&l);
    l = nl;
  }
  return l;
}

int oplan_build(oplan *pl, const odecomp *src, const odecomp *dst, int esize) {
  memset(pl, 0, sizeof(*pl));
  if (src->ndim != dst->ndim || src->P != dst->P) return -1;
  for (int i = 0; i < src->ndim; ++i)
    if (src->L[i] != dst->L[i]) return -1; /* compatible(), reshape.c:258-279 */
  int P = src->P;
  pl->P = P;
  pl->esize = esize;
  pl->src_used = src->proc_used;
  pl->dst_used = dst->proc_used;
  pl->sends = (omsglist *)calloc(P, sizeof(omsglist));
  pl->recvs = (omsglist *)calloc(P, sizeof(omsglist));
  for (int r = 0; r < P; ++r) {
    if (r < src->proc_used) pl->sends[r] = build_list(src, dst, src, r, dst->proc_used);
    if (r < dst->proc_used) pl->recvs[r] = build_list(dst, src, src, r, src->proc_used);
  }
  return 0;
}

void oplan_free(oplan *pl) {
  for (int r = 0; r < pl->P; ++r) {
    ml_free(&pl->sends[r]);
    ml_free(&pl->recvs[r]);
  }
  free(pl->sends);
  free(pl->recvs);
  memset(pl, 0, sizeof(*pl));
}

/* The k-th message from r to q matches the k-th receive q posts from r
 * (MPI non-overtaking order). */
static const omsg *find_send(const oplan *pl, int r, int q, int kth) {
  const omsglist *l = &pl->sends[r];
  for (int e = 0; e < l->nmsg; ++e)
    if (l->m[e].peer == q && kth-- == 0) return &l->m[e];
  return NULL;
}

typedef struct {
  const oplan *pl;
  const char *src;
  long long sp;
  char *dst;
  long long dp;
  const long long *sbase, *dbase; /* optional per-rank element offsets replacing r*pitch */
  int next;
  int err;
  pthread_mutex_t mu;
} run_ctx;

static void *run_worker(void *arg) {
  run_ctx *c = (run_ctx *)arg;
  const oplan *pl = c->pl;
  const int es = pl->esize;
  char *buf = NULL;
  long long bufcap = 0;
  for (;;) {
    pthread_mutex_lock(&c->mu);
    int q = c->next++;
    pthread_mutex_unlock(&c->mu);
    if (q >= pl->P) break;
    const omsglist *rl = &pl->recvs[q];
    for (int e = 0; e < rl->nmsg; ++e) {
      const omsg *rm = &rl->m[e];
      int kth = 0;
      for (int e2 = 0; e2 < e; ++e2) kth += rl->m[e2].peer == rm->peer;
      const omsg *sm = find_send(pl, rm->peer, q, kth);
      if (!sm || sm->n > rm->n) {
        c->err = 1;
        continue;
      }
      /* pack (sender typemap) then unpack (receiver typemap) */
      if (sm->n * es > bufcap) {
        bufcap = sm->n * es;
        buf = (char *)realloc(buf, bufcap);
      }
      long long so = c->sbase ? c->sbase[rm->peer] : (long long)rm->peer * c->sp;
      long long dq = c->dbase ? c->dbase[q] : (long long)q * c->dp;
      const char *sbase = c->src + (size_t)so * es;
      for (long long k = 0; k < sm->n; ++k) memcpy(buf + k * es, sbase + sm->off[k] * es, es);
      char *dbase = c->dst + (size_t)dq * es;
      for (long long k = 0; k < sm->n; ++k) memcpy(dbase + rm->off[k] * es, buf + k * es, es);
    }
  }
  free(buf);
  return NULL;
}

int oplan_run(const oplan *pl, const char *src, long long src_pitch, char *dst, long long dst_pitch, int nthreads) {
  return oplan_run_based(pl, src, src_pitch, NULL, dst, dst_pitch, NULL, nthreads);
}

int oplan_run_based(const oplan *pl, const char *src, long long src_pitch, const long long *src_base, char *dst,
                    long long dst_pitch, const long long *dst_base, int nthreads) {
  /* every send must have a matching receive */
  for (int r = 0; r < pl->P; ++r) {
    const omsglist *sl = &pl->sends[r];
    for (int e = 0; e < sl->nmsg; ++e) {
      int q = sl->m[e].peer, kth = 0, have = 0;
      for (int e2 = 0; e2 < e; ++e2) kth += sl->m[e2].peer == q;
      const omsglist *rl = &pl->recvs[q];
      for (int e2 = 0; e2 < rl->nmsg; ++e2) have += rl->m[e2].peer == r;
      if (kth >= have) return 2;
    }
  }
  run_ctx c;
  c.pl = pl;
  c.src = src;
  c.sp = src_pitch;
  c.dst = dst;
  c.dp = dst_pitch;
  c.sbase = src_base;
  c.dbase = dst_base;
  c.next = 0;
  c.err = 0;
  pthread_mutex_init(&c.mu, NULL);
  if (nthreads < 1) nthreads = 1;
  if (nthreads > pl->P) nthreads = pl->P;
  pthread_t th[256];
  if (nthreads > 256) nthreads = 256;
  for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, run_worker, &c);
  run_worker(&c);
  for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
  pthread_mutex_destroy(&c.mu);
  return c.err;
}

/* ---- exported ---- */

int oracle_decomp_info(int P, const char *spec, long long *extents, int *proc_used) {
  odecomp od;
  int rc = od_build(&od, P, spec);
  if (rc) {
    od_free(&od);
    return rc;
  }
  for (int r = 0; r < P; ++r) extents[r] = od_extent(&od, r);
  *proc_used = od.proc_used;
  od_free(&od);
  return 0;
}

int oracle_global_offsets(int P, const char *spec, long long pitch, long long *out) {
  odecomp od;
  int rc = od_build(&od, P, spec);
  if (rc) {
    od_free(&od);
    return rc;
  }
  long long total = 1;
  for (int i = 0; i < od.ndim; ++i) total *= od.L[i];
  int c[SPEC_MAXD];
  for (long long g = 0; g < total; ++g) {
    long long rem = g;
    for (int i = od.ndim - 1; i >= 0; --i) {
      c[i] = (int)(rem % od.L[i]);
      rem /= od.L[i];
    }
    long long R = 0;
    int ok = 1;
    for (int i = 0; i < od.ndim && ok; ++i) {
      int p = o_rank_offset(od.sd.dims[i], c[i]);
      if (p < 0 || p >= od.ps[i]) ok = 0;
      R += (long long)od.rs[i] * p;
    }
    if (ok) {
      for (int i = 0; i < od.ndim && ok; ++i) ok = od_local(&od, i, (int)R, c[i]);
    }
    if (!ok) {
      out[g] = -1;
      continue;
    }
    long long off = R * pitch;
    for (int i = 0; i < od.ndim; ++i) off += od.stride[i][R] * o_type_offset(od.sd.dims[i], c[i]);
    out[g] = off;
  }
  od_free(&od);
  return 0;
}

typedef struct {
  odecomp s, d;
  oplan pl;
} oracle_reshape_handle;

void *oracle_reshape_plan(int P, const char *src_spec, const char *dst_spec, int esize) {
  oracle_reshape_handle *h = (oracle_reshape_handle *)calloc(1, sizeof(*h));
  if (od_build(&h->s, P, src_spec) || od_build(&h->d, P, dst_spec) || oplan_build(&h->pl, &h->s, &h->d, esize)) {
    od_free(&h->s);
    od_free(&h->d);
    free(h);
    return NULL;
  }
  return h;
}

int oracle_reshape_exec(void *hv, const void *src, long long src_pitch, void *dst, long long dst_pitch,
                        int nthreads) {
  oracle_reshape_handle *h = (oracle_reshape_handle *)hv;
  return oplan_run(&h->pl, (const char *)src, src_pitch, (char *)dst, dst_pitch, nthreads);
}

void oracle_reshape_free(void *hv) {
  oracle_reshape_handle *h = (oracle_reshape_handle *)hv;
  if (!h) return;
  oplan_free(&h->pl);
  od_free(&h->s);
  od_free(&h->d);
  free(h);
}

int oracle_reshape(int P, const char *src_spec, const char *dst_spec, int esize, long long src_pitch,
                   long long dst_pitch, const void *src, void *dst, int nthreads) {
  void *h = oracle_reshape_plan(P, src_spec, dst_spec, esize);
  if (!h) return -1;
  int rc = oracle_reshape_exec(h, src, src_pitch, dst, dst_pitch, nthreads);
  oracle_reshape_free(h);
  return rc;
}
