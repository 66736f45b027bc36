/*
 * TEST INFRASTRUCTURE (oracle).  Thread-per-rank MPI subset for running the
 * reference's C sources in one process.  See mpi.h for what is covered.
 *
 * Datatypes are kept flattened: the ordered list of (byte displacement,
 * byte length) blocks of the typemap, plus lb and extent.  Sends are eager:
 * MPI_Isend packs the typemap into a message that goes to the receiver's
 * mailbox; MPI_Waitall unpacks matching messages in arrival order per
 * (source, tag), which is MPI's non-overtaking rule.
 */
#define _GNU_SOURCE
#include "mpi.h"
#include <errno.h>
#include <pthread.h>
#include <setjmp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ---------------- datatypes ---------------- */

typedef struct {
  MPI_Aint lb, extent;
  long size;
  long nblk, cap;
  long *disp, *len;
} dtype;

#define MAXTYPES (1 << 20)
static dtype *g_types[MAXTYPES];
static int g_free_slots[MAXTYPES];
static int g_nfree = 0, g_next = 16;
static pthread_mutex_t g_type_mu = PTHREAD_MUTEX_INITIALIZER;

static void blk_push(dtype *t, long d, long l) {
  if (l <= 0) return;
  if (t->nblk > 0 && t->disp[t->nblk - 1] + t->len[t->nblk - 1] == d) {
    t->len[t->nblk - 1] += l;
    return;
  }
  if (t->nblk == t->cap) {
    t->cap = t->cap ? t->cap * 2 : 8;
    t->disp = (long *)realloc(t->disp, t->cap * sizeof(long));
    t->len = (long *)realloc(t->len, t->cap * sizeof(long));
  }
  t->disp[t->nblk] = d;
  t->len[t->nblk] = l;
  t->nblk++;
}

static dtype *new_dtype(void) { return (dtype *)calloc(1, sizeof(dtype)); }

static int reg_type(dtype *t) {
  pthread_mutex_lock(&g_type_mu);
  int h;
  if (g_nfree > 0) h = g_free_slots[--g_nfree];
  else h = g_next++;
  if (h >= MAXTYPES) {
    pthread_mutex_unlock(&g_type_mu);
    fprintf(stderr, "mpi shim: too many datatypes\n");
    abort();
  }
  g_types[h] = t;
  pthread_mutex_unlock(&g_type_mu);
  return h;
}

static void init_basic(void);
static dtype *get_type(MPI_Datatype h) {
  static pthread_once_t once = PTHREAD_ONCE_INIT;
  pthread_once(&once, init_basic);
  if (h <= 0 || h >= MAXTYPES) return NULL;
  return g_types[h];
}

static void init_basic(void) {
  static const int sizes[7] = {0, 1, 1, 4, 4, 8, 8};
  for (int h = 1; h <= 6; ++h) {
    dtype *t = new_dtype();
    t->lb = 0;
    t->extent = sizes[h];
    t->size = sizes[h];
    blk_push(t, 0, sizes[h]);
    g_types[h] = t;
  }
}

static void free_dtype(dtype *t) {
  if (!t) return;
  free(t->disp);
  free(t->len);
  free(t);
}

int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *nt) {
  dtype *o = get_type(old);
  if (!o || count < 0) return MPI_ERR_OTHER;
  dtype *t = new_dtype();
  for (int c = 0; c < count; ++c)
    for (long b = 0; b < o->nblk; ++b) blk_push(t, o->disp[b] + (long)c * o->extent, o->len[b]);
  t->size = o->size * count;
  t->lb = o->lb;
  t->extent = o->extent * count;
  *nt = reg_type(t);
  return MPI_SUCCESS;
}

int MPI_Type_indexed(int count, const int blocklens[], const int displs[], MPI_Datatype old, MPI_Datatype *nt) {
  dtype *o = get_type(old);
  if (!o || count < 0) return MPI_ERR_OTHER;
  dtype *t = new_dtype();
  int first = 1;
  MPI_Aint lo = 0, hi = 0;
  for (int j = 0; j < count; ++j) {
    for (int k = 0; k < blocklens[j]; ++k) {
      long shift = ((long)displs[j] + k) * o->extent;
      for (long b = 0; b < o->nblk; ++b) blk_push(t, o->disp[b] + shift, o->len[b]);
      MPI_Aint l = shift + o->lb, u = shift + o->lb + o->extent;
      if (first || l < lo) lo = l;
      if (first || u > hi) hi = u;
      first = 0;
    }
    t->size += o->size * blocklens[j];
  }
  t->lb = lo;
  t->extent = hi - lo;
  *nt = reg_type(t);
  return MPI_SUCCESS;
}

int MPI_Type_create_resized(MPI_Datatype old, MPI_Aint lb, MPI_Aint extent, MPI_Datatype *nt) {
  dtype *o = get_type(old);
  if (!o) return MPI_ERR_OTHER;
  dtype *t = new_dtype();
  for (long b = 0; b < o->nblk; ++b) blk_push(t, o->disp[b], o->len[b]);
  t->size = o->size;
  t->lb = lb;
  t->extent = extent;
  *nt = reg_type(t);
  return MPI_SUCCESS;
}

int MPI_Type_dup(MPI_Datatype old, MPI_Datatype *nt) {
  dtype *o = get_type(old);
  if (!o) return MPI_ERR_OTHER;
  return MPI_Type_create_resized(old, o->lb, o->extent, nt);
}

int MPI_Type_commit(MPI_Datatype *t) { return get_type(*t) ? MPI_SUCCESS : MPI_ERR_OTHER; }

int MPI_Type_free(MPI_Datatype *t) {
  int h = *t;
  if (h <= 6) {
    *t = 0;
    return MPI_SUCCESS;
  }
  pthread_mutex_lock(&g_type_mu);
  if (h > 0 && h < MAXTYPES && g_types[h]) {
    free_dtype(g_types[h]);
    g_types[h] = NULL;
    g_free_slots[g_nfree++] = h;
  }
  pthread_mutex_unlock(&g_type_mu);
  *t = 0;
  return MPI_SUCCESS;
}

int MPI_Type_size(MPI_Datatype h, int *size) {
  dtype *t = get_type(h);
  if (!t) return MPI_ERR_OTHER;
  *size = (int)t->size;
  return MPI_SUCCESS;
}

int MPI_Type_get_extent(MPI_Datatype h, MPI_Aint *lb, MPI_Aint *extent) {
  dtype *t = get_type(h);
  if (!t) return MPI_ERR_OTHER;
  *lb = t->lb;
  *extent = t->extent;
  return MPI_SUCCESS;
}

int MPI_Type_get_true_extent(MPI_Datatype h, MPI_Aint *lb, MPI_Aint *extent) {
  dtype *t = get_type(h);
  if (!t) return MPI_ERR_OTHER;
  if (t->nblk == 0) {
    *lb = 0;
    *extent = 0;
    return MPI_SUCCESS;
  }
  long lo = t->disp[0], hi = t->disp[0] + t->len[0];
  for (long b = 1; b < t->nblk; ++b) {
    if (t->disp[b] < lo) lo = t->disp[b];
    if (t->disp[b] + t->len[b] > hi) hi = t->disp[b] + t->len[b];
  }
  *lb = lo;
  *extent = hi - lo;
  return MPI_SUCCESS;
}

/* ---------------- ranks, errors ---------------- */

static __thread int t_rank = 0;
static __thread int t_in_run = 0;
static __thread jmp_buf t_jmp;
static int g_size = 1;
static volatile int g_abort = 0;
static char g_errmsg[512];
static pthread_mutex_t g_err_mu = PTHREAD_MUTEX_INITIALIZER;

static void set_error(const char *msg) {
  pthread_mutex_lock(&g_err_mu);
  if (!g_abort) snprintf(g_errmsg, sizeof(g_errmsg), "%s", msg);
  g_abort = 1;
  pthread_mutex_unlock(&g_err_mu);
}

static void bail(const char *msg) {
  set_error(msg);
  if (t_in_run) longjmp(t_jmp, 1);
  fprintf(stderr, "mpi shim: %s\n", msg);
  abort();
}

const char *shim_error(void) { return g_errmsg; }
void shim_set_self(int rank, int size) {
  t_rank = rank;
  g_size = size;
}

int MPI_Init(int *argc, char ***argv) {
  (void)argc;
  (void)argv;
  return MPI_SUCCESS;
}
int MPI_Init_thread(int *argc, char ***argv, int required, int *provided) {
  (void)argc;
  (void)argv;
  *provided = required;
  return MPI_SUCCESS;
}
int MPI_Finalize(void) { return MPI_SUCCESS; }

int MPI_Comm_rank(MPI_Comm comm, int *rank) {
  *rank = (comm == MPI_COMM_SELF) ? 0 : t_rank;
  return MPI_SUCCESS;
}
int MPI_Comm_size(MPI_Comm comm, int *size) {
  *size = (comm == MPI_COMM_SELF) ? 1 : g_size;
  return MPI_SUCCESS;
}
int MPI_Abort(MPI_Comm comm, int code) {
  (void)comm;
  char m[64];
  snprintf(m, sizeof(m), "MPI_Abort(%d) on rank %d", code, t_rank);
  bail(m);
  return MPI_ERR_OTHER;
}
double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}
int MPI_Error_string(int code, char *s, int *len) {
  *len = snprintf(s, MPI_MAX_ERROR_STRING, "shim error %d", code);
  return MPI_SUCCESS;
}

/* timed wait that gives up on abort or after a long timeout */
static int timed_wait(pthread_cond_t *cv, pthread_mutex_t *mu, double *waited) {
  struct timespec ts;
  clock_gettime(CLOCK_REALTIME, &ts);
  ts.tv_nsec += 100 * 1000 * 1000;
  if (ts.tv_nsec >= 1000000000) {
    ts.tv_sec += 1;
    ts.tv_nsec -= 1000000000;
  }
  pthread_cond_timedwait(cv, mu, &ts);
  *waited += 0.1;
  return g_abort || *waited > 300.0;
}

/* ---------------- barrier / allreduce ---------------- */

static pthread_mutex_t g_bar_mu = PTHREAD_MUTEX_INITIALIZER;
static pthread_cond_t g_bar_cv = PTHREAD_COND_INITIALIZER;
static int g_bar_count = 0;
static long g_bar_gen = 0;

static void barrier_world(void) {
  if (g_size == 1) return;
  pthread_mutex_lock(&g_bar_mu);
  long gen = g_bar_gen;
  if (++g_bar_count == g_size) {
    g_bar_count = 0;
    g_bar_gen++;
    pthread_cond_broadcast(&g_bar_cv);
  } else {
    double w = 0;
    while (gen == g_bar_gen) {
      if (timed_wait(&g_bar_cv, &g_bar_mu, &w)) {
        pthread_mutex_unlock(&g_bar_mu);
        bail("barrier timed out or aborted");
      }
    }
  }
  pthread_mutex_unlock(&g_bar_mu);
}

int MPI_Barrier(MPI_Comm comm) {
  if (comm != MPI_COMM_SELF) barrier_world();
  return MPI_SUCCESS;
}

#define AR_MAX 64
static double g_ar_d[1024][AR_MAX];
static long long g_ar_i[1024][AR_MAX];

int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm) {
  int isd = (type == MPI_DOUBLE);
  if ((!isd && type != MPI_INT) || count > AR_MAX || g_size > 1024) bail("unsupported MPI_Allreduce");
  if (comm == MPI_COMM_SELF || g_size == 1) {
    memcpy(recvbuf, sendbuf, (size_t)count * (isd ? sizeof(double) : sizeof(int)));
    return MPI_SUCCESS;
  }
  for (int k = 0; k < count; ++k) {
    if (isd) g_ar_d[t_rank][k] = ((const double *)sendbuf)[k];
    else g_ar_i[t_rank][k] = ((const int *)sendbuf)[k];
  }
  barrier_world();
  for (int k = 0; k < count; ++k) {
    double ad = g_ar_d[0][k];
    long long ai = g_ar_i[0][k];
    for (int r = 1; r < g_size; ++r) {
      double vd = g_ar_d[r][k];
      long long vi = g_ar_i[r][k];
      if (op == MPI_MAX) {
        if (vd > ad) ad = vd;
        if (vi > ai) ai = vi;
      } else if (op == MPI_MIN) {
        if (vd < ad) ad = vd;
        if (vi < ai) ai = vi;
      } else {
        ad += vd;
        ai += vi;
      }
    }
    if (isd) ((double *)recvbuf)[k] = ad;
    else ((int *)recvbuf)[k] = (int)ai;
  }
  barrier_world();
  return MPI_SUCCESS;
}

/* ---------------- point to point ---------------- */

typedef struct msg {
  int src, tag;
  long bytes;
  char *data;
  struct msg *next;
} msg;

typedef struct {
  pthread_mutex_t mu;
  pthread_cond_t cv;
  msg *head, *tail;
} mailbox;

static mailbox g_box[1024];

typedef struct {
  int is_recv;
  void *buf;
  int count;
  MPI_Datatype type;
  int peer, tag;
  int done;
} req;

static __thread req *t_reqs = NULL;
static __thread int t_nreq = 0, t_capreq = 0;

static int new_req(void) {
  if (t_nreq == t_capreq) {
    t_capreq = t_capreq ? 2 * t_capreq : 64;
    t_reqs = (req *)realloc(t_reqs, (size_t)t_capreq * sizeof(req));
  }
  memset(&t_reqs[t_nreq], 0, sizeof(req));
  return t_nreq++;
}

int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm, MPI_Request *r) {
  (void)comm;
  dtype *t = get_type(type);
  if (!t) bail("MPI_Isend: bad datatype");
  if (dest < 0 || dest >= g_size) bail("MPI_Isend: bad destination rank");
  msg *m = (msg *)calloc(1, sizeof(msg));
  m->src = t_rank;
  m->tag = tag;
  m->bytes = t->size * count;
  m->data = (char *)malloc(m->bytes ? m->bytes : 1);
  long pos = 0;
  for (int c = 0; c < count; ++c) {
    const char *base = (const char *)buf + (long)c * t->extent;
    for (long b = 0; b < t->nblk; ++b) {
      memcpy(m->data + pos, base + t->disp[b], t->len[b]);
      pos += t->len[b];
    }
  }
  mailbox *bx = &g_box[dest];
  pthread_mutex_lock(&bx->mu);
  if (bx->tail) bx->tail->next = m;
  else bx->head = m;
  bx->tail = m;
  pthread_cond_broadcast(&bx->cv);
  pthread_mutex_unlock(&bx->mu);
  int h = new_req();
  t_reqs[h].done = 1;
  *r = h + 1;
  return MPI_SUCCESS;
}

int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Request *r) {
  (void)comm;
  int h = new_req();
  req *q = &t_reqs[h];
  q->is_recv = 1;
  q->buf = buf;
  q->count = count;
  q->type = type;
  q->peer = source;
  q->tag = tag;
  *r = h + 1;
  return MPI_SUCCESS;
}

static void complete_recv(req *q) {
  dtype *t = get_type(q->type);
  if (!t) bail("MPI_Irecv: bad datatype");
  mailbox *bx = &g_box[t_rank];
  pthread_mutex_lock(&bx->mu);
  double w = 0;
  for (;;) {
    msg *prev = NULL, *m = bx->head;
    while (m && !(m->src == q->peer && m->tag == q->tag)) {
      prev = m;
      m = m->next;
    }
    if (m) {
      if (prev) prev->next = m->next;
      else bx->head = m->next;
      if (bx->tail == m) bx->tail = prev;
      pthread_mutex_unlock(&bx->mu);
      long want = t->size * q->count;
      if (m->bytes > want) bail("MPI_Waitall: message truncated");
      long pos = 0;
      for (int c = 0; c < q->count && pos < m->bytes; ++c) {
        char *base = (char *)q->buf + (long)c * t->extent;
        for (long b = 0; b < t->nblk && pos < m->bytes; ++b) {
          memcpy(base + t->disp[b], m->data + pos, t->len[b]);
          pos += t->len[b];
        }
      }
      free(m->data);
      free(m);
      q->done = 1;
      return;
    }
    if (timed_wait(&bx->cv, &bx->mu, &w)) {
      pthread_mutex_unlock(&bx->mu);
      bail("MPI_Waitall: receive timed out or aborted");
    }
  }
}

int MPI_Waitall(int count, MPI_Request reqs[], MPI_Status statuses[]) {
  (void)statuses;
  for (int i = 0; i < count; ++i) {
    int h = reqs[i] - 1;
    if (h < 0 || h >= t_nreq) bail("MPI_Waitall: bad request");
    if (!t_reqs[h].done && t_reqs[h].is_recv) complete_recv(&t_reqs[h]);
  }
  /* all of this thread's requests are complete: recycle the table */
  int pending = 0;
  for (int i = 0; i < t_nreq; ++i) pending |= !t_reqs[i].done;
  if (!pending) t_nreq = 0;
  return MPI_SUCCESS;
}

/* ---------------- driver ---------------- */

typedef struct {
  int rank;
  void (*fn)(int, void *);
  void *arg;
} thr_arg;

static void *thr_main(void *p) {
  thr_arg *a = (thr_arg *)p;
  t_rank = a->rank;
  t_in_run = 1;
  t_nreq = 0;
  if (setjmp(t_jmp) == 0) a->fn(a->rank, a->arg);
  t_in_run = 0;
  free(t_reqs);
  t_reqs = NULL;
  t_nreq = t_capreq = 0;
  return NULL;
}

int shim_run(int nranks, void (*fn)(int, void *), void *arg) {
  if (nranks < 1 || nranks > 1024) return -1;
  g_size = nranks;
  g_abort = 0;
  g_errmsg[0] = 0;
  g_bar_count = 0;
  for (int r = 0; r < nranks; ++r) {
    pthread_mutex_init(&g_box[r].mu, NULL);
    pthread_cond_init(&g_box[r].cv, NULL);
    g_box[r].head = g_box[r].tail = NULL;
  }
  pthread_t *th = (pthread_t *)calloc((size_t)nranks, sizeof(pthread_t));
  thr_arg *ta = (thr_arg *)calloc((size_t)nranks, sizeof(thr_arg));
  pthread_attr_t attr;
  pthread_attr_init(&attr);
  pthread_attr_setstacksize(&attr, 64u << 20);
  for (int r = 0; r < nranks; ++r) {
    ta[r].rank = r;
    ta[r].fn = fn;
    ta[r].arg = arg;
    pthread_create(&th[r], &attr, thr_main, &ta[r]);
  }
  for (int r = 0; r < nranks; ++r) pthread_join(th[r], NULL);
  pthread_attr_destroy(&attr);
  int leftover = 0;
  for (int r = 0; r < nranks; ++r) {
    msg *m = g_box[r].head;
    while (m) {
      msg *n = m->next;
      free(m->data);
      free(m);
      m = n;
      leftover++;
    }
    g_box[r].head = g_box[r].tail = NULL;
  }
  free(th);
  free(ta);
  if (leftover && !g_abort) set_error("messages left unreceived");
  return g_abort ? 1 : 0;
}
