/*
 * Request server for reshape + split-FFT jobs (include/dmg_serve.h).
 *
 * One scheduler thread owns the device work.  Each loop it (1) retires the
 * batches whose completion event has fired, returning their arena space,
 * and (2) fills every idle stream slot with the oldest queued job that fits
 * the arena (a few younger jobs may pass a head that does not fit yet)
 * plus the queued jobs of the same side and type that also fit, up to the
 * batch limit; with mixing on, queued jobs of other sides up to the mixing
 * limit (and the same type) join a head of such a side too.  A batch runs
 * on its slot's stream: per job the host-to-device copy, the block -> rotate
 * reshapes of all jobs in shared launches, then the forward split FFT of all
 * jobs as shared launches (one launch per pass for jobs of one side; the
 * k-th passes of every side in one launch for a mixed batch), the spectrum
 * copies, the inverse as shared launches and the output copies, and an
 * event.  Plans and their device tables are cached per (side, type); the
 * plans of sides that may mix run the runtime radix schedule PLAN8, which
 * the grouped pass launch needs.
 */
#define _POSIX_C_SOURCE 200809L
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "block_decomp.h"
#include "dmg_gb300.h"
#include "dmg_internal.h"
#include "arena.h"
#include "dmg_serve.h"
#include "fft_params.h"
#include "local_decomp.h"
#include "rotate_decomp.h"

#define ALIGN DMG_ARENA_ALIGN
#define BYPASS 8 /* younger jobs that may start ahead of a head that does not fit */

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ---------------------------------------------------------------- plans */

typedef struct {
  int side, dtype, es;
  Decomp dblk, drot;
  ReshapePlan r01;
  SplitPlan sp;
  long long pitch_blk, pitch_rot, ext, len;
  long long bytes_in, bytes_dat, bytes_work;
} plan_entry;

typedef struct job_rec {
  long long id;
  dmg_job j;
  double t_submit, t_start, t_done;
  int batch, status;
  plan_entry *pe;
  long long off_in, off_dat, off_work, off_scale;
  struct job_rec *next;
} job_rec;

typedef struct {
  void *stream, *event;
  int busy, njobs;
  job_rec *jobs[DMG_FFT_MAXBATCH];
} slot;

struct dmg_server {
  int grid, P, nslots, max_batch, dev;
  int arith[2]; /* arithmetic of complex128 and complex64 plans (DMG_ARITH_*; -1: the plan's default) */
  int mix_side; /* jobs of sides up to this may share launches with other sides (0: none) */
  MPI_Comm comm;
  char *base;
  arena ar;
  slot *slots;
  plan_entry **plans;
  int nplans, cap_plans;
  job_rec *q_head, *q_tail;
  int nqueued, running;
  job_rec **done;
  int ndone, cap_done;
  long long next_id, submitted, completed;
  pthread_mutex_t mu;
  pthread_cond_t cv, cv_done;
  pthread_t th;
  int started, stop;
};

static void plan_free(plan_entry *pe) {
  if (!pe) return;
  if (pe->sp) freeSplitPlan(pe->sp);
  if (pe->r01) freeReshapePlan(pe->r01);
  if (pe->drot) freeDecomp(pe->drot);
  if (pe->dblk) freeDecomp(pe->dblk);
  free(pe);
}

/* block(L,g) | block(L,g) | local(L), and the rotated copy rotate(L/3,.) | rotate(1,.) | local */
static Decomp cube_decomp(MPI_Comm comm, int L, int g, int rotated) {
  DimDecomp d[3];
  for (int i = 0; i < 2; ++i) {
    DimDecomp b = makeBlockDecomp(L, g);
    if (rotated) {
      d[i] = makeRotatedDecomp(i == 0 ? L / 3 : 1, b);
      freeDimDecomp(b);
    } else {
      d[i] = b;
    }
  }
  d[2] = makeLocalDecomp(L);
  return makePackedDecomp(comm, 3, d);
}

static plan_entry *plan_make(struct dmg_server *s, int side, int dtype) {
  plan_entry *pe = (plan_entry *)calloc(1, sizeof(plan_entry));
  if (!pe) return NULL;
  pe->side = side;
  pe->dtype = dtype;
  pe->es = dtype == DMG_C128 ? 16 : 8;
  pe->dblk = cube_decomp(s->comm, side, s->grid, 0);
  pe->drot = cube_decomp(s->comm, side, s->grid, 1);
  if (!pe->dblk || !pe->drot) goto fail;
  pe->r01 = makeReshapePlan(s->comm, pe->es, pe->dblk, pe->drot);
  if (!pe->r01) goto fail;
  pe->pitch_blk = extent64(pe->dblk);
  pe->pitch_rot = extent64(pe->drot);
  {
    /* the workspace the reference asks for: twice the larger stage extent per rank */
    SplitPlan probe = dmg_makeSplitPlanTyped(0, pe->drot, (void *)(uintptr_t)ALIGN, 1ll << 40,
                                             (void *)(uintptr_t)(2 * ALIGN), dtype);
    if (!probe) goto fail;
    pe->ext = dmg_split_extent64(probe);
    freeSplitPlan(probe);
  }
  pe->len = 2 * pe->ext;
  pe->sp = dmg_makeSplitPlanTyped(0, pe->drot, (void *)(uintptr_t)ALIGN, pe->len, (void *)(uintptr_t)(2 * ALIGN),
                                  dtype);
  if (!pe->sp) goto fail;
  if (s->arith[dtype == DMG_C128 ? 0 : 1] >= 0 &&
      dmg_split_set_arith(pe->sp, s->arith[dtype == DMG_C128 ? 0 : 1]) != DMG_OK)
    goto fail;
  if (side <= s->mix_side && dmg_split_set_radix(pe->sp, DMG_RADIX_PLAN8) != DMG_OK) goto fail;
  pe->bytes_in = (long long)s->P * pe->pitch_blk * pe->es;
  pe->bytes_dat = (long long)s->P * pe->pitch_rot * pe->es;
  pe->bytes_work = (long long)s->P * pe->len * pe->es;
  return pe;
fail:
  plan_free(pe);
  return NULL;
}

static plan_entry *plan_get(struct dmg_server *s, int side, int dtype) {
  for (int i = 0; i < s->nplans; ++i)
    if (s->plans[i]->side == side && s->plans[i]->dtype == dtype) return s->plans[i];
  plan_entry *pe = plan_make(s, side, dtype);
  if (!pe) return NULL;
  if (s->nplans == s->cap_plans) {
    int nc = s->cap_plans ? 2 * s->cap_plans : 8;
    plan_entry **np = (plan_entry **)realloc(s->plans, (size_t)nc * sizeof(plan_entry *));
    if (!np) {
      plan_free(pe);
      return NULL;
    }
    s->plans = np;
    s->cap_plans = nc;
  }
  s->plans[s->nplans++] = pe;
  return pe;
}

static long long job_bytes(const plan_entry *pe) {
  return round_up(pe->bytes_in) + round_up(pe->bytes_dat) + round_up(pe->bytes_work) + ALIGN;
}

/* ---------------------------------------------------------------- scheduling (mutex held) */

static int job_alloc(struct dmg_server *s, job_rec *jr) {
  const plan_entry *pe = jr->pe;
  jr->off_in = arena_alloc(&s->ar, pe->bytes_in);
  jr->off_dat = jr->off_in >= 0 ? arena_alloc(&s->ar, pe->bytes_dat) : -1;
  jr->off_work = jr->off_dat >= 0 ? arena_alloc(&s->ar, pe->bytes_work) : -1;
  jr->off_scale = jr->off_work >= 0 ? arena_alloc(&s->ar, ALIGN) : -1;
  if (jr->off_scale >= 0) return 1;
  if (jr->off_work >= 0) arena_free(&s->ar, jr->off_work, pe->bytes_work);
  if (jr->off_dat >= 0) arena_free(&s->ar, jr->off_dat, pe->bytes_dat);
  if (jr->off_in >= 0) arena_free(&s->ar, jr->off_in, pe->bytes_in);
  return 0;
}

static void job_release(struct dmg_server *s, job_rec *jr) {
  const plan_entry *pe = jr->pe;
  arena_free(&s->ar, jr->off_scale, ALIGN);
  arena_free(&s->ar, jr->off_work, pe->bytes_work);
  arena_free(&s->ar, jr->off_dat, pe->bytes_dat);
  arena_free(&s->ar, jr->off_in, pe->bytes_in);
}

static void q_remove(struct dmg_server *s, job_rec *prev, job_rec *jr) {
  if (prev) prev->next = jr->next;
  else s->q_head = jr->next;
  if (s->q_tail == jr) s->q_tail = prev;
  jr->next = NULL;
  s->nqueued--;
}

static void push_done(struct dmg_server *s, job_rec *jr) {
  if (s->ndone == s->cap_done) {
    int nc = s->cap_done ? 2 * s->cap_done : 64;
    job_rec **nd = (job_rec **)realloc(s->done, (size_t)nc * sizeof(job_rec *));
    if (!nd) {
      free(jr); /* the record is lost; the job still counts as completed */
      return;
    }
    s->done = nd;
    s->cap_done = nc;
  }
  s->done[s->ndone++] = jr;
}

/* Enqueue a batch on a slot's stream.  The slot's jobs are in plan order
 * (the jobs of one plan next to each other). */
static int launch_batch(struct dmg_server *s, slot *sl) {
  job_rec **jobs = sl->jobs;
  const int k = sl->njobs;
  void *st = sl->stream;
  void *dats[DMG_FFT_MAXBATCH], *works[DMG_FFT_MAXBATCH];
  int *scales[DMG_FFT_MAXBATCH];
  int rc = DMG_OK;
  ReshapePlan plans[DMG_FFT_MAXBATCH];
  const void *ins[DMG_FFT_MAXBATCH];
  SplitPlan splits[DMG_FFT_MAXBATCH];
  int njobs[DMG_FFT_MAXBATCH], nplans = 0;
  for (int i = 0; i < k && rc == DMG_OK; ++i) {
    const plan_entry *pe = jobs[i]->pe;
    char *in = s->base + jobs[i]->off_in;
    dats[i] = s->base + jobs[i]->off_dat;
    works[i] = s->base + jobs[i]->off_work;
    scales[i] = (int *)(s->base + jobs[i]->off_scale);
    plans[i] = pe->r01;
    ins[i] = in;
    if (i == 0 || pe != jobs[i - 1]->pe) {
      splits[nplans] = pe->sp;
      njobs[nplans++] = 0;
    }
    njobs[nplans - 1]++;
    rc = dmg_rt_copy_async(in, jobs[i]->j.input, (size_t)pe->bytes_in, 0, st);
  }
  /* every job's block -> rotate reshape in shared launches */
  if (rc == DMG_OK) rc = dmg_reshape_run_group(k, plans, ins, dats, st);
  for (int dir = 0; dir < 2 && rc == DMG_OK; ++dir) {
    const int direction = dir == 0 ? FFTW_FORWARD : FFTW_BACKWARD;
    rc = nplans == 1 ? dmg_split_run_batch(splits[0], direction, st, k, dats, works, scales)
                     : dmg_split_run_group_batch(nplans, splits, njobs, dats, works, scales, direction, st);
    for (int i = 0; i < k && rc == DMG_OK; ++i) {
      const plan_entry *pe = jobs[i]->pe;
      if (dir == 0 && jobs[i]->j.spectrum)
        rc = dmg_rt_copy2d_async(jobs[i]->j.spectrum, (size_t)(pe->ext * pe->es), works[i],
                                 (size_t)(pe->len * pe->es), (size_t)(pe->ext * pe->es), (size_t)s->P, 1, st);
      if (dir == 1 && jobs[i]->j.output)
        rc = dmg_rt_copy_async(jobs[i]->j.output, dats[i], (size_t)pe->bytes_dat, 1, st);
    }
  }
  int rr = dmg_rt_event_record(sl->event, st);
  return rc != DMG_OK ? rc : rr;
}

static int mixes(const struct dmg_server *s, const plan_entry *a, const plan_entry *b) {
  return a == b || (a->dtype == b->dtype && a->side <= s->mix_side && b->side <= s->mix_side);
}

/* Fill idle slots; returns how many batches started. */
static int admit(struct dmg_server *s) {
  int started = 0;
  for (int si = 0; si < s->nslots && s->q_head; ++si) {
    slot *sl = &s->slots[si];
    if (sl->busy) continue;
    /* the oldest job that fits, looking past at most BYPASS younger ones */
    job_rec *prev = NULL, *jr = s->q_head, *head = NULL, *head_prev = NULL;
    for (int look = 0; jr && look <= BYPASS; ++look) {
      if (job_alloc(s, jr)) {
        head = jr;
        head_prev = prev;
        break;
      }
      prev = jr;
      jr = jr->next;
    }
    if (!head) break;
    q_remove(s, head_prev, head);
    sl->njobs = 0;
    sl->jobs[sl->njobs++] = head;
    /* queued jobs of the same plan (or, with mixing, of another side that
     * may mix) that also fit join the batch */
    prev = NULL;
    jr = s->q_head;
    while (jr && sl->njobs < s->max_batch) {
      job_rec *nx = jr->next;
      if (mixes(s, head->pe, jr->pe) && job_alloc(s, jr)) {
        q_remove(s, prev, jr);
        sl->jobs[sl->njobs++] = jr;
      } else {
        prev = jr;
      }
      jr = nx;
    }
    /* plan order: each plan's jobs next to each other, plans in order of first arrival */
    for (int i = 1; i < sl->njobs; ++i) {
      int last = i - 1;
      while (last >= 0 && sl->jobs[last]->pe != sl->jobs[i]->pe) --last;
      if (last < 0 || last == i - 1) continue;
      job_rec *t = sl->jobs[i];
      memmove(&sl->jobs[last + 2], &sl->jobs[last + 1], (size_t)(i - last - 1) * sizeof(job_rec *));
      sl->jobs[last + 1] = t;
    }
    const double t = now_s();
    for (int i = 0; i < sl->njobs; ++i) {
      sl->jobs[i]->t_start = t;
      sl->jobs[i]->batch = sl->njobs;
    }
    int rc = launch_batch(s, sl);
    sl->busy = 1;
    s->running += sl->njobs;
    for (int i = 0; i < sl->njobs; ++i) sl->jobs[i]->status = rc;
    started++;
  }
  return started;
}

/* Retire finished batches; returns how many. */
static int retire(struct dmg_server *s) {
  int n = 0;
  for (int si = 0; si < s->nslots; ++si) {
    slot *sl = &s->slots[si];
    if (!sl->busy) continue;
    int d = dmg_rt_event_done(sl->event);
    if (d == 0) continue;
    const double t = now_s();
    for (int i = 0; i < sl->njobs; ++i) {
      job_rec *jr = sl->jobs[i];
      jr->t_done = t;
      if (d < 0 && jr->status == DMG_OK) jr->status = -d;
      job_release(s, jr);
      push_done(s, jr);
      s->completed++;
    }
    s->running -= sl->njobs;
    sl->njobs = 0;
    sl->busy = 0;
    n++;
  }
  if (n) pthread_cond_broadcast(&s->cv_done);
  return n;
}

static void *worker(void *arg) {
  struct dmg_server *s = (struct dmg_server *)arg;
  dmg_rt_set_device(s->dev);
  pthread_mutex_lock(&s->mu);
  for (;;) {
    int progress = retire(s);
    progress += admit(s);
    if (s->stop && !s->nqueued && !s->running) break;
    if (!progress) {
      /* wait for a submit, or poll the running batches again shortly */
      struct timespec ts;
      clock_gettime(CLOCK_REALTIME, &ts);
      ts.tv_nsec += s->running ? 20000 : 2000000;
      if (ts.tv_nsec >= 1000000000) {
        ts.tv_sec += 1;
        ts.tv_nsec -= 1000000000;
      }
      pthread_cond_timedwait(&s->cv, &s->mu, &ts);
    }
  }
  pthread_mutex_unlock(&s->mu);
  return NULL;
}

/* ---------------------------------------------------------------- public API */

DmgServer dmg_server_create(int grid, long long arena_bytes, int slots, int max_batch) {
  if (grid < 1 || arena_bytes < ALIGN || slots < 1 || max_batch < 1 || max_batch > DMG_FFT_MAXBATCH) {
    dmg_error(DMG_ERR_ARG, "dmg_server_create: grid %d, arena %lld, slots %d, batch %d", grid, arena_bytes, slots,
              max_batch);
    return NULL;
  }
  struct dmg_server *s = (struct dmg_server *)calloc(1, sizeof(*s));
  if (!s) return NULL;
  s->grid = grid;
  s->P = grid * grid;
  s->arith[0] = s->arith[1] = -1;
  s->nslots = slots;
  s->max_batch = max_batch;
  if (dmg_rt_get_device(&s->dev) != DMG_OK) goto fail;
  s->comm = dmg_comm_create(s->P);
  if (!s->comm) goto fail;
  void *base = NULL;
  if (dmg_dev_alloc(&base, (size_t)arena_bytes) != DMG_OK) goto fail;
  s->base = (char *)base;
  /* the capacity is what the free list can hand out: a larger job never fits */
  if (arena_init(&s->ar, arena_bytes) != DMG_OK) goto fail;
  s->slots = (slot *)calloc((size_t)slots, sizeof(slot));
  if (!s->slots) goto fail;
  for (int i = 0; i < slots; ++i)
    if (dmg_rt_stream_create(&s->slots[i].stream) != DMG_OK || dmg_rt_event_create(&s->slots[i].event) != DMG_OK)
      goto fail;
  pthread_mutex_init(&s->mu, NULL);
  pthread_cond_init(&s->cv, NULL);
  pthread_cond_init(&s->cv_done, NULL);
  if (pthread_create(&s->th, NULL, worker, s) != 0) {
    dmg_error(DMG_ERR_ARG, "dmg_server_create: no scheduler thread");
    goto fail;
  }
  s->started = 1;
  return s;
fail:
  dmg_server_destroy(s);
  return NULL;
}

int dmg_server_set_arith(DmgServer s, int dtype, int arith) {
  if (!s || (dtype != DMG_C128 && dtype != DMG_C64))
    return dmg_error(DMG_ERR_ARG, "dmg_server_set_arith: server %p, element type %d", (void *)s, dtype);
  if (dtype == DMG_C128 ? (arith != DMG_ARITH_FP64 && arith != DMG_ARITH_DF)
                        : (arith != DMG_ARITH_FP32 && arith != DMG_ARITH_TC16))
    return dmg_error(DMG_ERR_ARG, "dmg_server_set_arith: arithmetic %d does not apply to element type %d", arith,
                     dtype);
  pthread_mutex_lock(&s->mu);
  int st = DMG_OK;
  if (s->running || s->nqueued) {
    st = dmg_error(DMG_ERR_ARG, "dmg_server_set_arith: jobs are queued or running; drain the server first");
  } else {
    s->arith[dtype == DMG_C128 ? 0 : 1] = arith;
    for (int i = 0; i < s->nplans && st == DMG_OK; ++i)
      if (s->plans[i]->dtype == dtype) st = dmg_split_set_arith(s->plans[i]->sp, arith);
  }
  pthread_mutex_unlock(&s->mu);
  return st;
}

int dmg_server_set_mixing(DmgServer s, int max_side) {
  if (!s || max_side < 0) return dmg_error(DMG_ERR_ARG, "dmg_server_set_mixing: server %p, side %d", (void *)s, max_side);
  pthread_mutex_lock(&s->mu);
  int st = DMG_OK;
  if (s->running || s->nqueued) {
    st = dmg_error(DMG_ERR_ARG, "dmg_server_set_mixing: jobs are queued or running; drain the server first");
  } else {
    s->mix_side = max_side;
    for (int i = 0; i < s->nplans && st == DMG_OK; ++i)
      st = dmg_split_set_radix(s->plans[i]->sp, s->plans[i]->side <= max_side ? DMG_RADIX_PLAN8 : DMG_RADIX_FIXED);
  }
  pthread_mutex_unlock(&s->mu);
  return st;
}

int dmg_server_job_sizes(DmgServer s, int side, int dtype, long long *input, long long *spectrum,
                         long long *output) {
  if (!s || side < 1 || (dtype != DMG_C128 && dtype != DMG_C64))
    return dmg_error(DMG_ERR_ARG, "dmg_server_job_sizes: side %d dtype %d", side, dtype);
  pthread_mutex_lock(&s->mu);
  plan_entry *pe = plan_get(s, side, dtype);
  pthread_mutex_unlock(&s->mu);
  if (!pe) return dmg_last_error_code() ? dmg_last_error_code() : DMG_ERR_ARG;
  if (input) *input = (long long)s->P * pe->pitch_blk;
  if (spectrum) *spectrum = (long long)s->P * pe->ext;
  if (output) *output = (long long)s->P * pe->pitch_rot;
  return DMG_OK;
}

long long dmg_server_submit(DmgServer s, const dmg_job *job) {
  if (!s || !job || !job->input || job->side < 1 || (job->dtype != DMG_C128 && job->dtype != DMG_C64))
    return -dmg_error(DMG_ERR_ARG, "dmg_server_submit: bad job (side %d, dtype %d)", job ? job->side : 0,
                      job ? job->dtype : -1);
  job_rec *jr = (job_rec *)calloc(1, sizeof(job_rec));
  if (!jr) return -dmg_error(DMG_ERR_NOMEM, "dmg_server_submit: out of memory");
  jr->j = *job;
  jr->t_submit = now_s();
  pthread_mutex_lock(&s->mu);
  jr->pe = plan_get(s, job->side, job->dtype);
  if (!jr->pe || job_bytes(jr->pe) > s->ar.size) {
    const int no_plan = !jr->pe;
    pthread_mutex_unlock(&s->mu);
    free(jr);
    if (no_plan) return -(dmg_last_error_code() ? dmg_last_error_code() : DMG_ERR_ARG);
    return -dmg_error(DMG_ERR_NOMEM, "dmg_server_submit: a %d^3 job needs more than the whole arena", job->side);
  }
  jr->id = s->next_id++;
  if (s->q_tail) s->q_tail->next = jr;
  else s->q_head = jr;
  s->q_tail = jr;
  s->nqueued++;
  s->submitted++;
  long long id = jr->id;
  pthread_cond_signal(&s->cv);
  pthread_mutex_unlock(&s->mu);
  return id;
}

int dmg_server_poll(DmgServer s, dmg_job_done *done, int max) {
  if (!s || max < 0 || (!done && max > 0)) return -dmg_error(DMG_ERR_ARG, "dmg_server_poll: bad arguments");
  pthread_mutex_lock(&s->mu);
  int n = s->ndone < max ? s->ndone : max;
  for (int i = 0; i < n; ++i) {
    job_rec *jr = s->done[i];
    done[i].id = jr->id;
    done[i].t_submit = jr->t_submit;
    done[i].t_start = jr->t_start;
    done[i].t_done = jr->t_done;
    done[i].batch = jr->batch;
    done[i].status = jr->status;
    free(jr);
  }
  memmove(s->done, s->done + n, (size_t)(s->ndone - n) * sizeof(job_rec *));
  s->ndone -= n;
  pthread_mutex_unlock(&s->mu);
  return n;
}

int dmg_server_drain(DmgServer s) {
  if (!s) return dmg_error(DMG_ERR_ARG, "dmg_server_drain: NULL server");
  pthread_mutex_lock(&s->mu);
  while (s->completed < s->submitted) pthread_cond_wait(&s->cv_done, &s->mu);
  pthread_mutex_unlock(&s->mu);
  return DMG_OK;
}

int dmg_server_status(DmgServer s, int *queued, int *running, long long *arena_used) {
  if (!s) return dmg_error(DMG_ERR_ARG, "dmg_server_status: NULL server");
  pthread_mutex_lock(&s->mu);
  if (queued) *queued = s->nqueued;
  if (running) *running = s->running;
  if (arena_used) *arena_used = s->ar.used;
  pthread_mutex_unlock(&s->mu);
  return DMG_OK;
}

void dmg_server_destroy(DmgServer s) {
  if (!s) return;
  if (s->started) {
    pthread_mutex_lock(&s->mu);
    s->stop = 1;
    pthread_cond_signal(&s->cv);
    pthread_mutex_unlock(&s->mu);
    pthread_join(s->th, NULL);
    pthread_mutex_destroy(&s->mu);
    pthread_cond_destroy(&s->cv);
    pthread_cond_destroy(&s->cv_done);
  }
  for (int i = 0; i < s->ndone; ++i) free(s->done[i]);
  free(s->done);
  for (int i = 0; i < s->nplans; ++i) plan_free(s->plans[i]);
  free(s->plans);
  if (s->slots) {
    for (int i = 0; i < s->nslots; ++i) {
      dmg_rt_event_destroy(s->slots[i].event);
      dmg_rt_stream_destroy(s->slots[i].stream);
    }
    free(s->slots);
  }
  arena_release(&s->ar);
  if (s->base) dmg_dev_free(s->base);
  if (s->comm) dmg_comm_free(s->comm);
  free(s);
}
