/* Virtual communicators and the per-thread error state. */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "dmg_internal.h"

static _Thread_local char g_err_msg[512];
static _Thread_local int g_err_code = DMG_OK;
static _Thread_local int g_err_print = 1;

int dmg_error(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err_msg, sizeof(g_err_msg), fmt, ap);
  va_end(ap);
  g_err_code = code;
  if (g_err_print) fprintf(stderr, "decomp_gb300 error: %s\n", g_err_msg);
  return code;
}

const char *dmg_last_error(void) { return g_err_msg; }
int dmg_last_error_code(void) { return g_err_code; }
void dmg_clear_error(void) {
  g_err_code = DMG_OK;
  g_err_msg[0] = 0;
}
int dmg_set_error_printing(int on) {
  const int prev = g_err_print;
  g_err_print = on;
  return prev;
}

/* The reference prints "<rank>: Error in reshape:<msg>" and aborts with
 * code 555 (reshape.c:12-21).  Here the message becomes the thread's last
 * error and control returns to the caller, which then fails its call. */
void raise_error(MPI_Comm comm, char *msg, ...) {
  char body[400];
  va_list ap;
  va_start(ap, msg);
  vsnprintf(body, sizeof(body), msg, ap);
  va_end(ap);
  int me = 0;
  if (dmg_comm_ok(comm)) me = comm->rank;
  dmg_error(DMG_ERR_ARG, "%d: Error in reshape:%s", me, body);
}

int dmg_comm_ok(MPI_Comm comm) { return comm != NULL && comm->magic == DMG_VCOMM_MAGIC; }

MPI_Comm dmg_comm_create(int nranks) {
  if (nranks < 1) {
    dmg_error(DMG_ERR_ARG, "dmg_comm_create: nranks=%d must be >= 1", nranks);
    return NULL;
  }
  MPI_Comm c = (MPI_Comm)calloc(1, sizeof(struct dmg_vcomm));
  if (!c) {
    dmg_error(DMG_ERR_NOMEM, "dmg_comm_create: out of memory");
    return NULL;
  }
  c->magic = DMG_VCOMM_MAGIC;
  c->size = nranks;
  c->rank = 0;
  return c;
}

void dmg_comm_free(MPI_Comm comm) {
  if (!dmg_comm_ok(comm)) return;
  comm->magic = 0;
  free(comm);
}

int dmg_comm_set_rank(MPI_Comm comm, int rank) {
  if (!dmg_comm_ok(comm) || rank < 0 || rank >= comm->size) {
    dmg_error(DMG_ERR_ARG, "dmg_comm_set_rank: rank %d out of range", rank);
    return MPI_ERR_ARG;
  }
  comm->rank = rank;
  return MPI_SUCCESS;
}
