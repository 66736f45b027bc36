/*
 * TEST INFRASTRUCTURE (oracle).  A single-process MPI subset, written for
 * this project, that lets the reference's C sources compile and run
 * unmodified: every MPI rank is a thread of one process.
 *
 * Covered: communicator rank/size, derived datatypes (contiguous, indexed,
 * resized, dup, commit, free, size, extent, true extent), eager
 * Isend/Irecv/Waitall, Barrier, Allreduce (MAX/MIN/SUM on int/double), Wtime,
 * Abort.  MPI-IO is not provided.
 */
#ifndef ORACLE_SHIM_MPI_H
#define ORACLE_SHIM_MPI_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef int MPI_Op;
typedef int MPI_Info;
typedef long MPI_Aint;
typedef struct {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
} MPI_Status;

#define MPI_COMM_WORLD ((MPI_Comm)1)
#define MPI_COMM_SELF ((MPI_Comm)2)
#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15
#define MPI_MAX_ERROR_STRING 256
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_INFO_NULL ((MPI_Info)0)
#define MPI_THREAD_SINGLE 0
#define MPI_THREAD_FUNNELED 1
#define MPI_MAX ((MPI_Op)1)
#define MPI_MIN ((MPI_Op)2)
#define MPI_SUM ((MPI_Op)3)

#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_BYTE ((MPI_Datatype)2)
#define MPI_INT ((MPI_Datatype)3)
#define MPI_FLOAT ((MPI_Datatype)4)
#define MPI_DOUBLE ((MPI_Datatype)5)
#define MPI_LONG_LONG ((MPI_Datatype)6)

int MPI_Init(int *argc, char ***argv);
int MPI_Init_thread(int *argc, char ***argv, int required, int *provided);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Barrier(MPI_Comm comm);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
double MPI_Wtime(void);
int MPI_Error_string(int code, char *string, int *len);

int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *newtype);
int MPI_Type_indexed(int count, const int blocklens[], const int displs[], MPI_Datatype old, MPI_Datatype *newtype);
int MPI_Type_create_resized(MPI_Datatype old, MPI_Aint lb, MPI_Aint extent, MPI_Datatype *newtype);
int MPI_Type_dup(MPI_Datatype old, MPI_Datatype *newtype);
int MPI_Type_commit(MPI_Datatype *t);
int MPI_Type_free(MPI_Datatype *t);
int MPI_Type_size(MPI_Datatype t, int *size);
int MPI_Type_get_extent(MPI_Datatype t, MPI_Aint *lb, MPI_Aint *extent);
int MPI_Type_get_true_extent(MPI_Datatype t, MPI_Aint *lb, MPI_Aint *extent);

int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Waitall(int count, MPI_Request reqs[], MPI_Status statuses[]);

/* ---- driver-side control (not MPI) ---- */
/* Run fn(rank, arg) on nranks threads as MPI ranks; returns 0 when every
 * rank finished without MPI_Abort or a shim error. */
int shim_run(int nranks, void (*fn)(int rank, void *arg), void *arg);
/* Message of the first error (abort, truncation, timeout) of the last run. */
const char *shim_error(void);
/* Set the rank/size seen by the calling thread outside shim_run. */
void shim_set_self(int rank, int size);

#ifdef __cplusplus
}
#endif
#endif
