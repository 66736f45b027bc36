#ifndef RESHAPE
#define RESHAPE
/**
 * @file reshape.h
 * Decomposition descriptors and reshape plans on a single-GPU virtual
 * processor grid.
 *
 * Same types, fields and entry points as the reference's reshape.h
 * (reshape.h:11-301).  What changes is where the ranks live: a Decomp over a
 * virtual communicator of P ranks describes one device array holding every
 * rank's local buffer, rank r's buffer starting at element r * pitch
 * (pitch = extent(D) unless set otherwise).  Inside a rank's buffer the
 * layout is exactly the reference's (offset = sum of memory_stride *
 * type_offset over the axes).  A reshape moves the whole virtual grid in one
 * permutation kernel launch on the GPU.
 *
 * Errors: where the reference called MPI_Abort (reshape.c:12-21) these
 * functions record an error (dmg_last_error()) and return NULL / nonzero.
 */
#include <stdio.h>
#include "dmg_vmpi.h"
#include "index.h"

#ifdef __cplusplus
extern "C" {
#endif

/** Record an error for dmg_last_error() and print it to stderr (when
 * printing is on); replaces the reference's aborting raise_error
 * (reshape.c:12-21).  @private */
void raise_error(MPI_Comm comm, char *msg, ...);

typedef struct dim_decomp *DimDecomp;

/** Maps a global coordinate to a position along the processor-grid axis
 * (reference reshape.h:21). */
typedef int (*rank_mapper)(DimDecomp, int);
/** Maps a global coordinate to a local offset along the axis
 * (reference reshape.h:26). */
typedef int (*offset_mapper)(DimDecomp, int);
/** Optional printer (reference reshape.h:31). */
typedef void (*print_decomp)(FILE *, DimDecomp);
/** Clone (reference reshape.h:36). */
typedef DimDecomp (*clone_decomp)(DimDecomp);

/** Per-axis decomposition plugin (reference reshape.h:45-54).
 *
 * This is the plugin API: application code may supply its own DimDecomp
 * (allocate it with calloc, fill the methods).  The planner calls
 * rank_offset/type_offset on the host once per global coordinate and turns
 * the results into device address tables, so any plugin runs on the GPU. */
struct dim_decomp {
  rank_mapper rank_offset;     /**< global coord -> position along the axis */
  offset_mapper type_offset;   /**< global coord -> local offset */
  void (*destroy)(DimDecomp);  /**< release what the decomp owns, may be NULL */
  print_decomp printer;        /**< extra debug info, may be NULL */
  clone_decomp cloner;         /**< deep copy */
  char *type;                  /**< runtime type name */
  int coord_size;              /**< number of global coordinates */
  int proc_size;               /**< number of positions along the axis */
};
/** Free a DimDecomp (reference reshape.h:58). */
void freeDimDecomp(DimDecomp);
/** Clone a DimDecomp; NULL when it has no cloner (reference reshape.h:62). */
DimDecomp cloneDimDecomp(DimDecomp);
/** Number of global coordinates (reference reshape.h:68). */
int sizeDimDecomp(DimDecomp d);
/** Print a DimDecomp through its print hook (reference reshape.h:67). */
void describeDimDecomp(FILE *out, DimDecomp d);

typedef struct axis_decomp *AxisDecomp;
/** A DimDecomp with memory and rank strides (reference reshape.h:75-85).
 *
 * The first eight fields are the reference's and describe the view rank of
 * the communicator.  The fields after them hold the same facts for every
 * position along the axis and every virtual rank. */
struct axis_decomp {
  DimDecomp decomp;          /**< decomposition along this axis (owned) */
  MPI_Comm comm;             /**< virtual communicator */
  int memory_stride;         /**< memory stride seen by the view rank */
  int rank_stride;           /**< rank stride */
  int my_rank_in_dimension;  /**< position of the view rank along the axis */
  int n_local;               /**< local points of the view rank */
  int max_local;             /**< largest local offset of the view rank */
  Index index;               /**< local offsets of the view rank */
  /* virtual-grid additions */
  long long *rank_memory_stride; /**< [comm size] memory stride of every virtual rank */
  int *pos_n_local;              /**< [proc_size] local points at each position */
  int *pos_max_local;            /**< [proc_size] largest local offset at each position (0 when empty) */
  Index *pos_index;              /**< [proc_size] local offsets at each position */
};

/** NULL-terminated per-position index lists of the coordinates local to the
 * view rank, split by their position in `remote` (reference reshape.h:92). */
Index *makeIndexList(AxisDecomp local, DimDecomp remote);
/** Global coordinates local to the view rank (reference reshape.h:101). */
Index makeGlobalIndex(AxisDecomp local);

/** Create an AxisDecomp; takes ownership of `d` (reference reshape.h:119).
 * Returns NULL (and records an error) for an illegal rank_stride. */
AxisDecomp makeAxisDecomp(MPI_Comm comm, DimDecomp d, int stride, int rank_stride);
/** Free an AxisDecomp and its DimDecomp (reference reshape.h:122). */
void freeAxisDecomp(AxisDecomp);
/** Print an AxisDecomp (reference reshape.h:122). */
void describeAxisDecomp(FILE *out, AxisDecomp d);
/** Is `global` local to the view rank along this axis (reference reshape.h:129). */
int isLocal(AxisDecomp d, int global);

typedef struct decomp *Decomp;
/** N-D decomposition (reference reshape.h:137-142). */
struct decomp {
  int ndim;          /**< number of dimensions */
  MPI_Comm comm;     /**< virtual communicator */
  int proc_used;     /**< virtual ranks used: 1 + sum rank_stride*(proc_size-1) */
  AxisDecomp *dims;  /**< per-dimension axis decompositions (owned) */
};

/** Make a Decomp from AxisDecomps; takes ownership of them
 * (reference reshape.h:148).  NULL on error. */
Decomp makeDecomp(int ndim, AxisDecomp dims[]);
/** Make a Decomp with C-order packed memory strides; per virtual rank the
 * stride of dim i is the product of (max_local+1) of the later dims on that
 * rank (reference reshape.h:155, reshape.c:218-241). */
Decomp makePackedDecomp(MPI_Comm comm, int ndim, DimDecomp dims[]);
/** Free a Decomp with its axes (reference reshape.h:158). */
void freeDecomp(Decomp d);
/** Print a Decomp (reference spelling, reshape.h:160). */
void describeDeomp(FILE *out, Decomp d);
/** The same, spelled correctly. */
void describeDecomp(FILE *out, Decomp d);
/** Largest memory extent over the virtual ranks, in elements
 * (reference reshape.h:164).  This is the default per-rank pitch of a
 * virtual-grid array.  Returns -1 when it does not fit in an int; use
 * extent64(). */
int extent(Decomp d);
/** 64-bit extent (largest over the virtual ranks). */
long long extent64(Decomp d);
/** Extent of one virtual rank's buffer. */
long long rankExtent64(Decomp d, int rank);

/** Same ndim, communicator and sizes (reference reshape.h:170). */
int compatible(Decomp a, Decomp b);
#define COMPATIBLE 1
#define NOT_COMPATIBLE 0

/** Rank of the view rank in the Decomp (reference reshape.h:185). */
int myRank(Decomp);
/** Is coordinate `pos` of dimension `dim` local to the view rank (reference reshape.h:191). */
int isCoordLocal(Decomp d, int dim, int pos);
/** Are all coordinates local to the view rank (reference reshape.h:196). */
int areCoordsLocal(Decomp d, int *pos);
/** Local offset of a coordinate on the view rank (reference reshape.h:201). */
int getOffset(Decomp d, int *pos);
/** Virtual rank holding a global coordinate, -1 when none holds it. */
int ownerRank(Decomp d, int *pos);
/** Element offset of a global coordinate in the virtual-grid array with
 * the given per-rank pitch: owner * pitch + local offset; -1 when unowned. */
long long globalOffset64(Decomp d, int *pos, long long pitch);

/** A plan for reshaping data (reference reshape.h:257-263).
 * The plan keeps pointers to src and dest for information only; the caller
 * keeps ownership of them. */
struct dmg_reshape_impl;
struct reshape_plan {
  MPI_Comm comm;   /**< virtual communicator */
  Decomp src;      /**< source decomposition (borrowed) */
  Decomp dest;     /**< destination decomposition (borrowed) */
  int *order;      /**< dimension order, fastest first (reshape.c:330-350) */
  struct dmg_reshape_impl *impl; /**< device address tables and launch setup */
};
typedef struct reshape_plan *ReshapePlan;

/** Plan a reshape of elements of type `base` from `src` to `dest`
 * (reference reshape.h:272).  NULL on error (incompatible decomps, rank
 * maps that are not a proper grid, ...). */
ReshapePlan makeReshapePlan(MPI_Comm comm, MPI_Datatype base, Decomp src, Decomp dest);
/** Free a plan (reference reshape.h:277). */
void freeReshapePlan(ReshapePlan plan);
/** Run a plan (reference reshape.h:285).  `src` and `dest` are device
 * pointers to virtual-grid arrays; the move is enqueued on the current
 * stream (dmg_set_stream) and is asynchronous to the host.  On failure the
 * error is recorded for dmg_last_error(). */
void runReshapePlan(MPI_Comm comm, ReshapePlan plan, void *src, void *dest);
/** Check a plan against per-rank array lengths in elements; 0 when every
 * access is in bounds (reference reshape.h:293). */
int checkReshapePlanBounds(ReshapePlan plan, int type_size, int src_len, int dest_len);

#ifdef __cplusplus
}
#endif
#endif
