#ifndef DMG_VMPI_H
#define DMG_VMPI_H
/**
 * @file dmg_vmpi.h
 * Virtual communicator and datatype handles for the single-GPU virtual
 * processor grid.
 *
 * The reference library runs one MPI process per rank and passes an
 * `MPI_Comm` and `MPI_Datatype` through its whole API (reshape.h:11-301,
 * split_fft.h:51-63).  Here one process drives every rank of a virtual
 * processor grid on one GPU, so:
 *
 *  - `MPI_Comm` is a virtual communicator: the number of virtual ranks and a
 *    "view rank".  Every descriptor holds the data of all virtual ranks; the
 *    per-rank fields that the reference structs expose (for example
 *    `axis_decomp.my_rank_in_dimension`) describe the view rank, so code that
 *    inspects them reads what rank `view` would have seen under MPI.
 *  - `MPI_Datatype` is an element size in bytes.  `MPI_Type_contiguous`
 *    multiplies it, which is all the reference uses to build its base types
 *    (split_fft.c:339, split_plan_test.c:247).
 *
 * No symbol named MPI_* is exported by the library: these are static inline,
 * so a process that also links a real MPI sees no clash.
 */
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/** A virtual communicator over `size` virtual ranks. */
struct dmg_vcomm {
  int magic;   /**< DMG_VCOMM_MAGIC while alive */
  int size;    /**< number of virtual ranks */
  int rank;    /**< view rank for the reference-compatible per-rank fields */
};
#define DMG_VCOMM_MAGIC 0x564d5049

typedef struct dmg_vcomm *MPI_Comm;
typedef int MPI_Datatype; /**< element size in bytes */
typedef long long MPI_Aint;

#define MPI_SUCCESS 0
#define MPI_ERR_COMM 5
#define MPI_ERR_ARG 12
#define MPI_ERR_TYPE 3

#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_SHORT ((MPI_Datatype)2)
#define MPI_INT ((MPI_Datatype)4)
#define MPI_FLOAT ((MPI_Datatype)4)
#define MPI_LONG_LONG ((MPI_Datatype)8)
#define MPI_INT64_T ((MPI_Datatype)8)
#define MPI_DOUBLE ((MPI_Datatype)8)
#define MPI_C_FLOAT_COMPLEX ((MPI_Datatype)8)
#define MPI_C_DOUBLE_COMPLEX ((MPI_Datatype)16)

/** Create a virtual communicator of `nranks` ranks (view rank 0).
 * Returns NULL when nranks < 1. */
MPI_Comm dmg_comm_create(int nranks);
/** Free a virtual communicator.  Descriptors made on it must be freed first. */
void dmg_comm_free(MPI_Comm comm);
/** Select which virtual rank the per-rank fields of descriptors created
 * afterwards describe.  Returns MPI_SUCCESS or MPI_ERR_ARG. */
int dmg_comm_set_rank(MPI_Comm comm, int rank);

static inline int MPI_Comm_size(MPI_Comm comm, int *size) {
  if (comm == NULL || comm->magic != DMG_VCOMM_MAGIC) return MPI_ERR_COMM;
  *size = comm->size;
  return MPI_SUCCESS;
}
static inline int MPI_Comm_rank(MPI_Comm comm, int *rank) {
  if (comm == NULL || comm->magic != DMG_VCOMM_MAGIC) return MPI_ERR_COMM;
  *rank = comm->rank;
  return MPI_SUCCESS;
}
static inline int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *newtype) {
  if (count < 1 || old < 1) return MPI_ERR_TYPE;
  *newtype = count * old;
  return MPI_SUCCESS;
}
static inline int MPI_Type_commit(MPI_Datatype *t) { (void)t; return MPI_SUCCESS; }
static inline int MPI_Type_free(MPI_Datatype *t) { *t = 0; return MPI_SUCCESS; }
static inline int MPI_Type_size(MPI_Datatype t, int *size) { *size = t; return MPI_SUCCESS; }
static inline int MPI_Type_get_extent(MPI_Datatype t, MPI_Aint *lb, MPI_Aint *extent) {
  *lb = 0;
  *extent = t;
  return MPI_SUCCESS;
}

#ifdef __cplusplus
}
#endif
#endif
