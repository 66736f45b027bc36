/*
 * TEST INFRASTRUCTURE (oracle).  CPU restatement of the reference's split
 * (two-stage) parallel FFT: factor choice, processor-grid search, the A and
 * B decompositions, and the forward pipeline of runSplitPlan with each MPI
 * rank on a worker thread.  The FFTW stages run on the oracle's FP64 FFT
 * (cfft.c).  The inverse runs the mathematically inverse sequence (the
 * reference's backward path is mis-ordered, split_fft.c:683-743).
 */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "cfft.h"
#include "oracle.h"
#include "oracle_internal.h"

/* ---- processor grid (processor_grid.c:24-97) ---- */

typedef struct {
  int *length;
  int procs;
  int load;
  double asym;
} grid_best;

static void search_grid(grid_best *best, int ndim, int mydim, int *grid, const int *tasks, int max_proc, int proc,
                        int load, int min, int max) {
  int newproc = proc;
  for (grid[mydim] = 1; grid[mydim] <= max_proc && grid[mydim] <= tasks[mydim] && newproc <= max_proc;
       grid[mydim]++) {
    newproc = proc * grid[mydim];
    if (newproc > max_proc) continue;
    int mymin = tasks[mydim] / grid[mydim];
    int mymax = (tasks[mydim] + grid[mydim] - 1) / grid[mydim];
    int newload = load * mymax;
    if (min < mymin) mymin = min;
    if (max > mymax) mymax = max;
    if (mydim < ndim - 1) {
      search_grid(best, ndim, mydim + 1, grid, tasks, max_proc, newproc, newload, mymin, mymax);
    } else {
      double ratio = (double)mymax / (double)mymin;
      if (newload <= best->load || best->load == 0) {
        if (best->load == 0 || newload < best->load || ratio < best->asym) {
          best->procs = newproc;
          best->load = newload;
          best->asym = ratio;
          for (int i = 0; i < ndim; ++i) best->length[i] = grid[i];
        }
      }
    }
  }
}

/* makeProcessorGrid (processor_grid.c:73-97): the search above from one task per rank upward */
int oracle_processor_grid(int P, int ndim, const int *tasks, int *out) {
  grid_best b;
  b.length = (int *)calloc(ndim, sizeof(int));
  b.procs = 1;
  b.load = 1;
  b.asym = 10000.0;
  int mx = 1;
  for (int i = 0; i < ndim; ++i) {
    b.length[i] = 1;
    b.load *= tasks[i];
    if (tasks[i] > mx) mx = tasks[i];
  }
  int *grid = (int *)calloc(ndim, sizeof(int));
  search_grid(&b, ndim, 0, grid, tasks, P, 1, 1, mx, 0);
  for (int i = 0; i < ndim; ++i) out[i] = b.length[i];
  free(grid);
  free(b.length);
  return 0;
}

/* ---- factors (split_fft.c:573-607, 747-776) ---- */

static void choose_B(const odecomp *st, int mode, const int *Bin, int *B) {
  int nd = st->ndim;
  for (int i = 0; i < nd; ++i) {
    int LL = st->L[i];
    if (mode == 2) {
      B[i] = Bin[i];
      continue;
    }
    int AA = 1, BB = LL;
    if (mode == 1) {
      if (i == nd - 1) {
        BB = 1;
        AA = LL;
      }
    } else {
      for (int qq = 1; qq < LL; ++qq) {
        if (LL % qq == 0) {
          int pp = LL / qq;
          if (qq > AA && qq <= pp) {
            AA = qq;
            BB = pp;
          }
        }
      }
    }
    B[i] = BB;
  }
}

int oracle_split_factors(int P, const char *start_spec, int mode, const int *Bin, int *A, int *B, int *grid_a,
                         int *grid_b, char *a_spec, char *b_spec, int speclen) {
  odecomp st;
  if (od_build(&st, P, start_spec)) {
    od_free(&st);
    return -1;
  }
  int nd = st.ndim;
  choose_B(&st, mode, Bin, B);
  for (int i = 0; i < nd; ++i) {
    if (B[i] < 1 || st.L[i] % B[i]) {
      od_free(&st);
      return -2;
    }
    A[i] = st.L[i] / B[i];
  }
  oracle_processor_grid(P, nd, A, grid_a);
  oracle_processor_grid(P, nd, B, grid_b);
  /* A: interleave(block(A_i, grid_a_i), B_i) packed (split_fft.c:36-61);
   * B: block(A_i*B_i, factor A_i, grid_b_i) packed (split_fft.c:63-77) */
  int pa = snprintf(a_spec, speclen, "packed:");
  int pb = snprintf(b_spec, speclen, "packed:");
  for (int i = 0; i < nd; ++i) {
    pa += snprintf(a_spec + pa, speclen - pa, "%sinterleave(block(%d,%d),%d)", i ? "|" : "", A[i], grid_a[i], B[i]);
    pb += snprintf(b_spec + pb, speclen - pb, "%sblockf(%d,%d,%d)", i ? "|" : "", A[i] * B[i], A[i], grid_b[i]);
  }
  od_free(&st);
  return 0;
}

/* ---- pipeline ---- */

typedef struct {
  int P, nd;
  int use_first, use_second;
  int A[SPEC_MAXD], B[SPEC_MAXD];
  odecomp st, da, db;
  long long *ext;       /* [P] per-rank extent: max(extent(A), extent(B)) (split_fft.c:286-303) */
  double **tw[SPEC_MAXD]; /* [dim][rank] twiddle table over local offsets, NULL when none */
  int have_tw;
  oplan s2a, a2b, b2a, a2s;
} splitplan;

/* exp(-2 pi i y*l/L) with the exact quarter turns of split_fft.c:373-399 */
static void twiddle_value(int y, int l, int L, double *re, double *im) {
  double angle = -(2.0 * M_PI) * ((double)(y * l) / (double)L);
  double c = cos(angle), s = sin(angle);
  int rem = (y * l) % L;
  if (rem == 0) {
    c = 1.0;
    s = 0.0;
  } else if (4 * rem == L) {
    c = 0.0;
    s = -1.0;
  } else if (2 * rem == L) {
    c = -1.0;
    s = 0.0;
  } else if (4 * rem == 3 * L) {
    c = -0.0;
    s = 1.0;
  }
  *re = c;
  *im = s;
}

/* buildParallelPlan (split_fft.c:249-569): factors, grids, the A and B decompositions, their extents
 * against the workspace (split_fft.c:304-308), and the twiddle tables */
static int sp_build(splitplan *sp, int P, const char *start_spec, int mode, const int *Bin, long long work_len) {
  memset(sp, 0, sizeof(*sp));
  if (od_build(&sp->st, P, start_spec)) return -1;
  int nd = sp->st.ndim;
  sp->P = P;
  sp->nd = nd;
  int ga[SPEC_MAXD], gb[SPEC_MAXD];
  char as[1024], bs[1024];
  if (oracle_split_factors(P, start_spec, mode, Bin, sp->A, sp->B, ga, gb, as, bs, sizeof(as))) return -2;
  sp->use_first = sp->use_second = 1;
  for (int i = 0; i < nd; ++i) {
    sp->use_first &= sp->A[i] == 1;
    sp->use_second &= sp->B[i] == 1;
  }
  if (od_build(&sp->da, P, as)) return -3;
  if (!sp->use_first && od_build(&sp->db, P, bs)) return -4;
  sp->ext = (long long *)calloc(P, sizeof(long long));
  for (int r = 0; r < P; ++r) {
    long long e = od_extent(&sp->da, r);
    if (!sp->use_first) {
      long long eb = od_extent(&sp->db, r);
      if (eb > e) e = eb;
    }
    if (2 * e > work_len) return -5; /* split_fft.c:304-308 */
    sp->ext[r] = e;
  }
  oplan_build(&sp->s2a, &sp->st, &sp->da, 16);
  oplan_build(&sp->a2s, &sp->da, &sp->st, 16);
  if (!sp->use_first) {
    oplan_build(&sp->a2b, &sp->da, &sp->db, 16);
    oplan_build(&sp->b2a, &sp->db, &sp->da, 16);
  }
  if (!(sp->use_first || sp->use_second)) {
    int non_trivial = 0;
    for (int i = 0; i < nd; ++i) {
      sp->tw[i] = (double **)calloc(P, sizeof(double *));
      for (int r = 0; r < P; ++r) {
        int ml = sp->da.pos_max[i][od_pos(&sp->da, i, r)];
        double *t = (double *)calloc(2 * (size_t)(ml + 1), sizeof(double));
        int any = 0;
        for (int g = 0; g < sp->st.L[i]; ++g) {
          if (!od_local(&sp->da, i, r, g)) continue;
          any = 1;
          int local = o_type_offset(sp->da.sd.dims[i], g);
          double re, im;
          twiddle_value(g % sp->A[i], g / sp->A[i], sp->st.L[i], &re, &im);
          if (re != 1.0 && im != 0.0) non_trivial = 1;
          t[2 * local] = re;
          t[2 * local + 1] = im;
        }
        if (any) sp->tw[i][r] = t;
        else free(t);
      }
    }
    sp->have_tw = non_trivial;
  }
  return 0;
}

/* freeSplitPlan (split_fft.c:789-858) */
static void sp_free(splitplan *sp) {
  for (int i = 0; i < sp->nd; ++i) {
    if (!sp->tw[i]) continue;
    for (int r = 0; r < sp->P; ++r) free(sp->tw[i][r]);
    free(sp->tw[i]);
  }
  free(sp->ext);
  oplan_free(&sp->s2a);
  oplan_free(&sp->a2s);
  if (!sp->use_first) {
    oplan_free(&sp->a2b);
    oplan_free(&sp->b2a);
  }
  od_free(&sp->st);
  od_free(&sp->da);
  if (!sp->use_first) od_free(&sp->db);
}

/* dim_scale restated (dimscale.c:7-49): recurse over local slots
 * 0..max_local of each dim, multiply the factors, skip zero factors (unused
 * slots), conjugate on sign == 1. */
static void dim_scale(const splitplan *sp, int r, int dim, double fr, double fi, double *data, long long offset,
                      int sign) {
  const odecomp *d = &sp->da;
  int count = d->pos_max[dim][od_pos(d, dim, r)] + 1;
  long long ms = d->stride[dim][r];
  const double *f = sp->tw[dim] ? sp->tw[dim][r] : NULL;
  for (int pos = 0; pos < count; ++pos) {
    long long no = offset + pos * ms;
    double nr = fr, ni = fi;
    if (f) {
      nr = fr * f[2 * pos] - fi * f[2 * pos + 1];
      ni = fr * f[2 * pos + 1] + fi * f[2 * pos];
    }
    if (nr == 0.0 && ni == 0.0) continue;
    if (dim == d->ndim - 1) {
      if (sign == 1) ni = -ni;
      double *v = data + 2 * no;
      double vr = v[0], vi = v[1];
      v[0] = nr * vr - ni * vi;
      v[1] = nr * vi + ni * vr;
    } else {
      dim_scale(sp, r, dim + 1, nr, ni, data, no, sign);
    }
  }
}

/* One FFT stage on rank r (split_fft.c:427-541): transform the dims whose
 * factor F[i] > 1 with the layout's strides, loop over the rest. */
static void stage_fft(const odecomp *lay, int r, const int *F, const double *in, double *out, int sign) {
  cfft_dim tr[SPEC_MAXD], lp[SPEC_MAXD];
  int nt = 0, nl = 0;
  for (int i = 0; i < lay->ndim; ++i) {
    long long st = lay->stride[i][r];
    if (F[i] > 1) {
      tr[nt].n = F[i];
      tr[nt].is = tr[nt].os = (int)st;
      nt++;
    }
    int count = lay->pos_n[i][od_pos(lay, i, r)] / F[i];
    if (count > 1) {
      lp[nl].n = count;
      lp[nl].is = lp[nl].os = (int)(st * F[i]);
      nl++;
    }
  }
  if (nt == 0) return;
  if (nl == 0) {
    lp[0].n = 1;
    lp[0].is = lp[0].os = 0;
    nl = 1;
  }
  cfft_guru(nt, tr, nl, lp, in, out, sign);
}

typedef struct {
  const splitplan *sp;
  int stage;
  int sign;
  double *work;
  long long work_len;
  int next;
  pthread_mutex_t mu;
} stage_ctx;

/* one virtual rank's batched FFTs of a stage (the fftw_execute calls of runSplitPlan, split_fft.c:638-690) */
static void *stage_worker(void *arg) {
  stage_ctx *c = (stage_ctx *)arg;
  const splitplan *sp = c->sp;
  for (;;) {
    pthread_mutex_lock(&c->mu);
    int r = c->next++;
    pthread_mutex_unlock(&c->mu);
    if (r >= sp->P) break;
    double *lo = c->work + 2 * (size_t)r * c->work_len;
    double *hi = lo + 2 * (size_t)sp->ext[r];
    switch (c->stage) {
      case 0: /* forward stage 1: hi -> lo on A layout */
        if (r < sp->da.proc_used && !sp->use_second) stage_fft(&sp->da, r, sp->B, hi, lo, -1);
        break;
      case 1: /* twiddle on lo (A layout) */
        if (sp->have_tw) dim_scale(sp, r, 0, 1.0, 0.0, lo, 0, c->sign);
        break;
      case 2: /* forward stage 2: hi -> lo on B layout */
        if (!sp->use_first && r < sp->db.proc_used) stage_fft(&sp->db, r, sp->A, hi, lo, -1);
        break;
      case 3: /* inverse stage 2: lo -> hi on B layout */
        if (!sp->use_first && r < sp->db.proc_used) stage_fft(&sp->db, r, sp->A, lo, hi, +1);
        break;
      case 4: /* inverse stage 1: lo -> hi on A layout */
        if (r < sp->da.proc_used && !sp->use_second) stage_fft(&sp->da, r, sp->B, lo, hi, +1);
        break;
    }
  }
  return NULL;
}

/* a stage over every rank, ranks spread over worker threads as the reference spreads them over processes */
static void run_stage(const splitplan *sp, int stage, int sign, double *work, long long work_len, int nthreads) {
  stage_ctx c = {sp, stage, sign, work, work_len, 0};
  pthread_mutex_init(&c.mu, NULL);
  if (nthreads < 1) nthreads = 1;
  if (nthreads > sp->P) nthreads = sp->P;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, stage_worker, &c);
  stage_worker(&c);
  for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
  pthread_mutex_destroy(&c.mu);
}

/* runSplitPlan (split_fft.c:622-744): forward = reshape start->A, stage-A FFTs, twiddle, reshape A->B,
 * stage-B FFTs; the inverse runs those steps backwards with conjugate twiddles */
static int sp_run(const splitplan *sp, long long dat_pitch, long long work_len, double *dat, double *work, int dir,
                  int nthreads) {
  int P = sp->P;
  long long *lo = (long long *)malloc(P * sizeof(long long));
  long long *hi = (long long *)malloc(P * sizeof(long long));
  for (int r = 0; r < P; ++r) {
    lo[r] = (long long)r * work_len;
    hi[r] = lo[r] + sp->ext[r];
  }
  int rc = 0;
  if (dir < 0) {
    rc |= oplan_run_based(&sp->s2a, (const char *)dat, dat_pitch, NULL, (char *)work, 0, hi, nthreads);
    run_stage(sp, 0, -1, work, work_len, nthreads);
    run_stage(sp, 1, -1, work, work_len, nthreads);
    if (!sp->use_first) {
      rc |= oplan_run_based(&sp->a2b, (const char *)work, 0, lo, (char *)work, 0, hi, nthreads);
      run_stage(sp, 2, -1, work, work_len, nthreads);
    }
  } else {
    if (!sp->use_first) {
      run_stage(sp, 3, +1, work, work_len, nthreads);
      rc |= oplan_run_based(&sp->b2a, (const char *)work, 0, hi, (char *)work, 0, lo, nthreads);
    }
    run_stage(sp, 1, +1, work, work_len, nthreads);
    run_stage(sp, 4, +1, work, work_len, nthreads);
    rc |= oplan_run_based(&sp->a2s, (const char *)work, 0, hi, (char *)dat, dat_pitch, NULL, nthreads);
  }
  free(lo);
  free(hi);
  return rc;
}

/* handle-based API so that planning stays out of timed regions */
void *oracle_split_plan(int P, const char *start_spec, int mode, const int *Bin, long long work_len) {
  splitplan *sp = (splitplan *)calloc(1, sizeof(splitplan));
  if (sp_build(sp, P, start_spec, mode, Bin, work_len)) {
    free(sp); /* partial plans are leaked on purpose: test-only code */
    return NULL;
  }
  return sp;
}

int oracle_split_exec(void *h, long long dat_pitch, long long work_len, double *dat, double *work, int direction,
                      int nthreads) {
  return sp_run((const splitplan *)h, dat_pitch, work_len, dat, work, direction, nthreads);
}

long long oracle_split_extent(void *h, int r) { return ((splitplan *)h)->ext[r]; }

void oracle_split_free(void *h) {
  if (!h) return;
  sp_free((splitplan *)h);
  free(h);
}

int oracle_split_fft(int P, const char *start_spec, int mode, const int *Bin, long long dat_pitch,
                     long long work_len, double *dat, double *work, int direction, int nthreads) {
  void *h = oracle_split_plan(P, start_spec, mode, Bin, work_len);
  if (!h) return -1;
  int rc = oracle_split_exec(h, dat_pitch, work_len, dat, work, direction, nthreads);
  oracle_split_free(h);
  return rc;
}
